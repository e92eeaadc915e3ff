"""Float64 adjoint-state velocity gradient of the 2D forward loop, constant
or variable density (TEST INFRASTRUCTURE ONLY).

Only tests/ and bench.py's checks use this module; the product package never
imports it. The reference has no adjoint (its compiler offers only the
forward operator, simwave/kernel/backend/compiler.py:128-130), so this is the
exact transpose of the reference's discrete forward loop, written out step by
step in numpy from the forward's sections
(simwave/kernel/backend/c_code/forward/constant_density/2d/wave.c):

  step n (begin <= n <= end), all on the extended grid:
    w       = (2 u^n - N u^(n-1)) / D + c (L u^n + s_n)    interior points
              D = 1 + damp dt v^2 / 2, N = 1 - damp dt v^2 / 2,
              c = dt^2 v^2 / D                            (wave.c:155-178)
              s_n = sum over sources of kws * wavelet[n-1]  (wave.c:182-271)
    u^(n+1) = B w    boundary conditions, x edges then z edges
                                                         (wave.c:274-393)
    rec[n-1] = R u^n  KWS gather of the current level     (wave.c:395-464)

With variable density (simwave/kernel/backend/c_code/forward/
variable_density/2d/wave.c:143-201) L becomes
    A u = L u - sum_a G_a fd_a(u),  G_a = fd_a(rho) / (4 h_a^2 rho),
    fd_a(f)(p) = sum_k c1_k (f(p + k e_a) - f(p - k e_a))
at the interior points (rho read on the whole grid, G_a formed at the
interior points only), and L^T in the recursion below becomes
    A^T z = L^T z + sum_a fd_a(G_a z)   (z supported on the interior),
the first differences being antisymmetric.

The gradient of J(v) = sum(g * rec(v)) for a given g (the shot-record
cotangent) follows the adjoint-state recursion, with mu^m the adjoint of the
interior values w of level m before the boundary conditions:

  mu^m = B^T [ R^T g[m-1] + (2/D) mu^(m+1) - (N/D) mu^(m+2) + L^T (c mu^(m+1)) ]
  dJ/dv = sum_n mu^(n+1) * (2 v / D^2) * (dt^2 (L u^n + s_n) - damp dt (u^n - u^(n-1)))

with mu^(end+1) = mu^(end+2) = 0. B^T applies the transposed boundary
operations in reverse order (z edges, then x edges): a Dirichlet zero stays a
zero, a Neumann copy u[halo] = u[mirror] becomes lam[mirror] += lam[halo].
dt, the damping mask and the KWS windows are held fixed (they do not depend
on v in the derivative). The initial levels u^(begin-1), u^begin are zero.

The gradient uses the Laplacian form above, not the second time difference
the GPU kernels use, so the two are independent derivations.
"""
import numpy as np

import oracle as _oracle

_BC = {'none': 0, 'null_dirichlet': 1, 'null_neumann': 2}


class Problem2D:
    """The forward problem of middleware keyword arguments (2D, constant or
    variable density), in float64."""

    def __init__(self, kwargs):
        kw = _oracle._normalise(kwargs)
        if kw['velocity_model'].ndim != 2:
            raise ValueError("2D problems only")
        self.vel = np.asarray(kw['velocity_model'], dtype=np.float64)
        den = kw.get('density_model')
        self.den = None if den is None else np.asarray(den, dtype=np.float64)
        self.damp = np.asarray(kw['damping_mask'], dtype=np.float64)
        self.nz, self.nx = self.vel.shape
        self.order = int(kw['space_order'])
        self.r = self.order // 2
        self.c2 = np.asarray(kw['second_order_fd_coefficients'], dtype=np.float64)
        self.c1 = None
        if self.den is not None:
            self.c1 = np.asarray(kw['first_order_fd_coefficients'], dtype=np.float64)
        self.dz, self.dx = float(kw['dz']), float(kw['dx'])
        self.dt = float(kw['dt'])
        self.bc = [int(b) for b in kw['boundary_condition']]
        self.begin = int(kw['begin_timestep'])
        self.end = int(kw['end_timestep'])
        w = np.asarray(kw['wavelet'], dtype=np.float64)
        self.wcount = int(kw['wavelet_count'])
        self.nsrc = int(kw['num_sources'])
        self.nrec = int(kw['num_receivers'])
        self.wavelet = w.reshape(-1, self.nsrc) if self.wcount > 1 else w.reshape(-1, 1)
        self.src = self._windows(kw['src_points_interval'], kw['src_points_values'],
                                 kw['src_points_values_offset'], self.nsrc)
        self.rec = self._windows(kw['rec_points_interval'], kw['rec_points_values'],
                                 kw['rec_points_values_offset'], self.nrec)

    def _windows(self, iv, vals, off, count):
        iv = np.asarray(iv, dtype=np.int64).reshape(count, 4) if count else []
        vals = np.asarray(vals, dtype=np.float64)
        off = np.asarray(off, dtype=np.int64)
        out = []
        r = self.r
        for s in range(count):
            z0, z1, x0, x1 = (int(v) for v in iv[s])
            if z0 < r or x0 < r or z1 > self.nz - r - 1 or x1 > self.nx - r - 1:
                raise ValueError("KWS window reaches the halo")
            lz = z1 - z0 + 1
            kz = vals[off[s]:off[s] + lz]
            kx = vals[off[s] + lz:off[s] + lz + (x1 - x0 + 1)]
            out.append((slice(z0, z1 + 1), slice(x0, x1 + 1), np.outer(kz, kx)))
        return out

    def with_velocity(self, vel):
        p = object.__new__(Problem2D)
        p.__dict__.update(self.__dict__)
        p.vel = np.asarray(vel, dtype=np.float64)
        p._G = None
        return p

    # -- operators -----------------------------------------------------------
    def _fd(self, f, axis, interior):
        """fd_axis(f): at the interior points (`interior`, zero elsewhere;
        reads the halo) or, for f supported on the interior, at every point."""
        r, nz, nx = self.r, self.nz, self.nx
        if interior:
            I, J = slice(r, nz - r), slice(r, nx - r)
            s = np.zeros((nz - 2 * r, nx - 2 * r))
            for k in range(1, r + 1):
                if axis == 1:
                    s = s + self.c1[k] * (f[I, r + k:nx - r + k] - f[I, r - k:nx - r - k])
                else:
                    s = s + self.c1[k] * (f[r + k:nz - r + k, J] - f[r - k:nz - r - k, J])
            out = np.zeros((nz, nx))
            out[I, J] = s
            return out
        fp = np.pad(f, r)
        s = np.zeros((nz, nx))
        for k in range(1, r + 1):
            if axis == 1:
                s = s + self.c1[k] * (fp[r:r + nz, r + k:r + k + nx] - fp[r:r + nz, r - k:r - k + nx])
            else:
                s = s + self.c1[k] * (fp[r + k:r + k + nz, r:r + nx] - fp[r - k:r - k + nz, r:r + nx])
        return s

    def density_terms(self):
        """G_z, G_x at the interior points (zero elsewhere)."""
        if getattr(self, '_G', None) is None:
            h2 = (self.dz * self.dz, self.dx * self.dx)
            self._G = tuple(self._fd(self.den, a, True) / (4.0 * h2[a] * self.den)
                            for a in (0, 1))
        return self._G

    def op(self, u):
        """A u: L u, less the density term with variable density."""
        out = self.lap(u)
        if self.den is not None:
            for a, G in enumerate(self.density_terms()):
                out = out - G * self._fd(u, a, True)
        return out

    def op_t(self, z):
        """A^T z for z supported on the interior, at every grid point."""
        out = self.lap_t(z)
        if self.den is not None:
            for a, G in enumerate(self.density_terms()):
                out = out + self._fd(G * z, a, False)
        return out

    def lap(self, u):
        """L u at the interior points (zero elsewhere); reads the halo."""
        r, nz, nx = self.r, self.nz, self.nx
        I, J = slice(r, nz - r), slice(r, nx - r)
        sx = self.c2[0] * u[I, J]
        sz = self.c2[0] * u[I, J]
        for k in range(1, r + 1):
            sx = sx + self.c2[k] * (u[I, r + k:nx - r + k] + u[I, r - k:nx - r - k])
            sz = sz + self.c2[k] * (u[r + k:nz - r + k, J] + u[r - k:nz - r - k, J])
        out = np.zeros_like(u)
        out[I, J] = sx / (self.dx * self.dx) + sz / (self.dz * self.dz)
        return out

    def lap_t(self, z):
        """L^T z for z supported on the interior: the same symmetric stencil
        evaluated at every grid point (halo included)."""
        r = self.r
        zp = np.pad(z, r)
        nz, nx = self.nz, self.nx
        sx = self.c2[0] * z
        sz = self.c2[0] * z
        for k in range(1, r + 1):
            sx = sx + self.c2[k] * (zp[r:r + nz, r + k:r + k + nx] + zp[r:r + nz, r - k:r - k + nx])
            sz = sz + self.c2[k] * (zp[r + k:r + k + nz, r:r + nx] + zp[r - k:r - k + nz, r:r + nx])
        return sx / (self.dx * self.dx) + sz / (self.dz * self.dz)

    def source_field(self, n):
        s = np.zeros((self.nz, self.nx))
        for i, (zs, xs, k) in enumerate(self.src):
            w = self.wavelet[n - 1, i if self.wcount > 1 else 0]
            s[zs, xs] += k * w
        return s

    def boundary(self, u):
        """B: the boundary conditions on a new level, in place."""
        r, nz, nx = self.r, self.nz, self.nx
        I, J = slice(r, nz - r), slice(r, nx - r)
        bz0, bz1, bx0, bx1 = self.bc
        if bx0 == 1:
            u[I, r] = 0.0
        elif bx0 == 2:
            for q in range(1, r + 1):
                u[I, r - q] = u[I, r + q]
        if bx1 == 1:
            u[I, nx - r - 1] = 0.0
        elif bx1 == 2:
            for q in range(1, r + 1):
                u[I, nx - r - 1 + q] = u[I, nx - r - 1 - q]
        if bz0 == 1:
            u[r, J] = 0.0
        elif bz0 == 2:
            for q in range(1, r + 1):
                u[r - q, J] = u[r + q, J]
        if bz1 == 1:
            u[nz - r - 1, J] = 0.0
        elif bz1 == 2:
            for q in range(1, r + 1):
                u[nz - r - 1 + q, J] = u[nz - r - 1 - q, J]
        return u

    def boundary_t(self, lam):
        """B^T: the transposed operations in reverse order; returns the
        interior-supported adjoint."""
        lam = lam.copy()
        r, nz, nx = self.r, self.nz, self.nx
        I, J = slice(r, nz - r), slice(r, nx - r)
        bz0, bz1, bx0, bx1 = self.bc
        if bz1 == 1:
            lam[nz - r - 1, J] = 0.0
        elif bz1 == 2:
            for q in range(1, r + 1):
                lam[nz - r - 1 - q, J] += lam[nz - r - 1 + q, J]
                lam[nz - r - 1 + q, J] = 0.0
        if bz0 == 1:
            lam[r, J] = 0.0
        elif bz0 == 2:
            for q in range(1, r + 1):
                lam[r + q, J] += lam[r - q, J]
                lam[r - q, J] = 0.0
        if bx1 == 1:
            lam[I, nx - r - 1] = 0.0
        elif bx1 == 2:
            for q in range(1, r + 1):
                lam[I, nx - r - 1 - q] += lam[I, nx - r - 1 + q]
                lam[I, nx - r - 1 + q] = 0.0
        if bx0 == 1:
            lam[I, r] = 0.0
        elif bx0 == 2:
            for q in range(1, r + 1):
                lam[I, r + q] += lam[I, r - q]
                lam[I, r - q] = 0.0
        mu = np.zeros_like(lam)
        mu[I, J] = lam[I, J]
        return mu

    def coefficients(self):
        v2 = self.vel * self.vel
        half = self.damp * self.dt * v2 / 2.0
        D = 1.0 + half
        N = 1.0 - half
        c = self.dt * self.dt * v2 / D
        return D, N, c

    # -- forward and adjoint -------------------------------------------------
    def forward(self):
        """All levels u^(begin-1) .. u^(end+1) (index k - begin + 1) and the
        shot record (end rows, row n-1 from level n)."""
        D, N, c = self.coefficients()
        r, nz, nx = self.r, self.nz, self.nx
        I, J = slice(r, nz - r), slice(r, nx - r)
        levels = [np.zeros((nz, nx)), np.zeros((nz, nx))]
        rec = np.zeros((self.end, self.nrec))
        for n in range(self.begin, self.end + 1):
            un, up = levels[-1], levels[-2]
            w = (2.0 * un - N * up) / D + c * (self.op(un) + self.source_field(n))
            nxt = np.zeros((nz, nx))
            nxt[I, J] = w[I, J]
            levels.append(self.boundary(nxt))
            for s, (zs, xs, k) in enumerate(self.rec):
                rec[n - 1, s] = np.sum(k * un[zs, xs])
        return levels, rec

    def gradient(self, g, levels=None):
        """dJ/dv of J = sum(g * rec) on the extended grid."""
        if levels is None:
            levels, _ = self.forward()
        D, N, c = self.coefficients()
        r, nz, nx = self.r, self.nz, self.nx
        I, J = slice(r, nz - r), slice(r, nx - r)
        b, e = self.begin, self.end
        at = lambda k: levels[k - b + 1]  # noqa: E731
        mu1 = np.zeros((nz, nx))
        mu2 = np.zeros((nz, nx))
        grad = np.zeros((nz, nx))
        dvdD = 2.0 * self.vel / (D * D)
        for m in range(e, b, -1):
            lam = np.zeros((nz, nx))
            for s, (zs, xs, k) in enumerate(self.rec):
                lam[zs, xs] += k * g[m - 1, s]
            lam[I, J] += (2.0 / D[I, J]) * mu1[I, J] - (N[I, J] / D[I, J]) * mu2[I, J]
            lam += self.op_t(c * mu1)
            mu = self.boundary_t(lam)
            n = m - 1
            term = self.dt * self.dt * (self.op(at(n)) + self.source_field(n)) \
                - self.damp * self.dt * (at(n) - at(n - 1))
            grad[I, J] += (mu * dvdD * term)[I, J]
            mu2, mu1 = mu1, mu
        return grad


def shot_record(kwargs, vel=None):
    p = Problem2D(kwargs)
    if vel is not None:
        p = p.with_velocity(vel)
    return p.forward()[1]


def gradient(kwargs, g, vel=None):
    p = Problem2D(kwargs)
    if vel is not None:
        p = p.with_velocity(vel)
    return p.gradient(np.asarray(g, dtype=np.float64))
