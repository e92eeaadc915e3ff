"""The front end's fast setup paths give the same bits as the plain
formulas they replace: the damping mask (raised over the layer slabs only)
and the edge-padded models (layer and halo in one copy)."""
import numpy as np
import pytest

import simwave_gb300 as sw


def _model(rng, dim, dtype):
    shape = tuple(int(v) for v in rng.integers(12, 40, size=dim))
    h = 10.0
    box = []
    for a in range(dim):
        box += [0.0, (shape[a] - 1) * h]
    vel = (1500 + 1000 * rng.random(shape)).astype(dtype)
    den = (1000 + 500 * rng.random(shape)).astype(dtype)
    sm = sw.SpaceModel(tuple(box), (h,) * dim, vel, den,
                       space_order=int(rng.choice([2, 4, 8, 16])), dtype=dtype)
    lengths = tuple(float(rng.integers(0, 8)) * h for _ in range(2 * dim))
    sm.config_boundary(damping_length=lengths, boundary_condition="null_neumann",
                       damping_polynomial_degree=int(rng.integers(0, 4)),
                       damping_alpha=0.001)
    return sm


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fast_setup_paths_are_bit_identical(dim, dtype):
    rng = np.random.default_rng(10 * dim + (dtype == np.float64))
    for _ in range(8):
        sm = _model(rng, dim, dtype)
        ramp = np.pad(np.zeros(sm.shape, dtype=sm.dtype), pad_width=sm.nbl_pad_width,
                      mode="linear_ramp", end_values=sm.nbl_pad_width)
        mask = np.pad((ramp ** sm.damping_polynomial_degree) * sm.damping_alpha,
                      pad_width=sm.halo_pad_width)
        assert sm.damping_mask.dtype == mask.dtype
        assert np.array_equal(sm.damping_mask, mask)
        for data, ext in ((sm.velocity_model, sm.extended_velocity_model),
                          (sm.density_model, sm.extended_density_model)):
            ref = np.pad(np.pad(data, sm.nbl_pad_width, mode="edge"), sm.halo_pad_width,
                         mode="edge")
            assert np.array_equal(ext, ref)
