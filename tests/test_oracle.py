"""The CPU oracle is pinned to the reference: bit-identical to the outputs
the reference's own C path produced for every golden fixture, and (where the
reference tree was compiled into oracle/_ref) to the reference kernels on
fresh cases."""
import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from _cases import CASE_FIXTURES, FIXTURES, fixture_kwargs, random_problem


@pytest.mark.parametrize("name", FIXTURES)
def test_port_reproduces_reference_outputs(name):
    kw, expected_u, expected_rec, meta = fixture_kwargs(name)
    u, rec, _ = oracle.forward("port", **kw)
    if isinstance(expected_u, tuple):
        slot, expected_u = expected_u
        u = u[slot:slot + 1]
    assert np.array_equal(u, expected_u)
    assert np.array_equal(rec, expected_rec)


def test_port_x_stride_variants_agree_on_cubes_only():
    cube = random_problem(sw, 3, 6, True, "none", 0, n=16, tf=0.02, seed=5)
    a = oracle.forward("port", x_stride="reference", **cube)[0].copy()
    cube = random_problem(sw, 3, 6, True, "none", 0, n=16, tf=0.02, seed=5)
    b = oracle.forward("port", x_stride="layout", **cube)[0]
    assert np.array_equal(a, b)
    box = random_problem(sw, 3, 6, True, "none", 0, shape=(16, 19, 14),
                         tf=0.02, seed=5)
    a = oracle.forward("port", x_stride="reference", **box)[0].copy()
    box = random_problem(sw, 3, 6, True, "none", 0, shape=(16, 19, 14),
                         tf=0.02, seed=5)
    b = oracle.forward("port", x_stride="layout", **box)[0]
    assert not np.array_equal(a, b)


needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference kernels not compiled here")


@needs_ref
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("vd", [False, True])
@pytest.mark.parametrize("stride", [0, 1, 2, 5])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_port_bitwise_vs_reference_build(dim, vd, stride, dtype):
    bc = ("null_neumann", "null_dirichlet", "none", "null_dirichlet",
          "null_neumann", "null_dirichlet")[:2 * dim]
    n = 36 if dim == 2 else 18
    a = random_problem(sw, dim, 6, vd, bc, stride, dtype=dtype, n=n,
                       tf=0.04, seed=11, nsrc=2, nrec=5)
    b = random_problem(sw, dim, 6, vd, bc, stride, dtype=dtype, n=n,
                       tf=0.04, seed=11, nsrc=2, nrec=5)
    oracle.forward("port", **a)
    oracle.forward("ref", language="c", **b)
    assert np.array_equal(a["u_full"], b["u_full"])
    assert np.array_equal(a["shot_record"], b["shot_record"])


@needs_ref
@pytest.mark.parametrize("order", range(2, 22, 2))
def test_port_bitwise_all_orders(order):
    a = random_problem(sw, 2, order, True, "null_neumann", 0, n=48,
                       tf=0.03, seed=order)
    b = random_problem(sw, 2, order, True, "null_neumann", 0, n=48,
                       tf=0.03, seed=order)
    oracle.forward("port", **a)
    oracle.forward("ref", language="omp", **b)
    assert np.array_equal(a["u_full"], b["u_full"])
    assert np.array_equal(a["shot_record"], b["shot_record"])
