// sw_gradient.cu -- velocity gradient of the 2D float32 forward loop,
// constant or variable density: a forward pass that keeps checkpoints and a
// reverse pass that recomputes one segment of levels at a time and runs the
// discrete adjoint.
//
// The reference has no adjoint (its compiler offers only the forward
// operator, simwave/kernel/backend/compiler.py:128-130). The forward step n
// (constant_density/2d/wave.c) is
//   w       = (2 u^n - N u^(n-1)) / D + C (L u^n + s_n)   interior points
//   u^(n+1) = B w              boundary conditions (x edges, then z edges)
//   rec[n-1] = R u^n           KWS gather of the current level
// with D = 1 + q, N = 1 - q, q = damp dt v^2 / 2, C = dt^2 v^2 / D. For a
// cotangent g of the shot record, the adjoint of w at level m, scaled by C,
//   nu^m = C * B^T [ R^T g[m-1] + (2/D) mu^(m+1) - (N/D) mu^(m+2) + L^T (C mu^(m+1)) ],
//   mu = nu / C,
// is, written out, the forward update itself applied to nu with a zero halo
//   nu^m = (2 nu^(m+1) - N nu^(m+2)) / D + C L nu^(m+1)  (+ C R^T g[m-1]),
// followed by the transposed boundary operations (z edges, then x edges):
// a Dirichlet zero stays a zero; a Neumann copy u[halo] = u[mirror] becomes
// nu[mirror] += C[mirror] * (L nu^(m+1))[halo]. So the reverse pass runs the
// forward's own stencil on the adjoint levels. The velocity derivative of w,
// (2 v / D^2) (dt^2 (L u^n + s_n) - damp dt (u^n - u^(n-1))), becomes
// 2 (w^(n+1) - 2 u^n + u^(n-1)) / (D v) once the update is substituted for
// dt^2 (L u^n + s_n); with mu = nu / C the gradient is
//   dJ/dv = sum_m nu^m * 2 / (v^3 dt^2) * (w^m - 2 u^(m-1) + u^(m-2)),
// where w^m equals u^m except on the Dirichlet lines, whose values before
// the boundary conditions are saved during the recomputation.
//
// With variable density (variable_density/2d/wave.c:143-201) L is the
// forward's A u = L u - sum_a G_a fd_a(u), G_a = fd_a(rho) / (4 h_a^2 rho)
// at interior points (fd_a the first difference with the c1 weights), and
// the adjoint update applies A^T nu = L nu + sum_a fd_a(G_a nu) (the first
// differences are antisymmetric, nu has a zero halo); the Neumann fold adds
// the halo point's first-difference term, +- sum_k c1_k (G_a nu)(mirror side)
// (+ at the edge before the interior, - after it). The velocity derivative
// is the same expression with A for L, so the gradient term is unchanged.
//
// Checkpoints: the pair (u^(n-1), u^n) before every `interval`-th step,
// stored by the forward pass in a caller buffer; the reverse pass rebuilds
// `interval` levels from each pair, last segment first.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>
#include <vector>

#include "simwave_gb300.h"
#include "sw_kernels.cuh"
#include "sw_tile2d.cuh"
#include "sw_tiled.h"

namespace sw {

void record_error(const std::string& message);

namespace grad {

struct Refusal {
    int code;
    std::string message;
};

[[noreturn]] static void refuse(int code, const std::string& m) { throw Refusal{code, m}; }

#define GR_CUDA(expr)                                                               \
    do {                                                                            \
        cudaError_t e_ = (expr);                                                    \
        if (e_ != cudaSuccess)                                                      \
            ::sw::grad::refuse(e_ == cudaErrorMemoryAllocation ? SIMWAVE_E_MEMORY   \
                                                               : SIMWAVE_E_CUDA,    \
                               std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define GR_LAUNCHED(name)                                                          \
    do {                                                                           \
        cudaError_t e_ = cudaGetLastError();                                       \
        if (e_ != cudaSuccess)                                                     \
            ::sw::grad::refuse(SIMWAVE_E_CUDA, std::string("launch ") + name + ": " + \
                                                   cudaGetErrorString(e_));        \
    } while (0)

// ---------------------------------------------------------------------------
// kernels

// K = 2 / (v^3 dt^2): the velocity factor of the gradient.
__global__ void gradient_factor(const float* __restrict__ vel, float* __restrict__ K,
                                long long n, float dt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = vel[i];
        K[i] = 2.0f / (v * v * v * (dt * dt));
    }
}

// G_a = s1_a fd_a(rho) / rho at interior points (zero elsewhere; the
// arrays are cleared first): the density terms of the adjoint operator.
__global__ void density_terms(const float* __restrict__ den, float* __restrict__ Gz,
                              float* __restrict__ Gx, Layout L, Weights<float> W) {
    const int r = L.r;
    const long long j = r + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long i = r + blockIdx.y * (long long)blockDim.y + threadIdx.y;
    if (j >= L.nx - r || i >= L.nz - r) return;
    const long long p = L.at2(i, j);
    float fz = 0.0f, fx = 0.0f;
    for (int k = 1; k <= r; k++) {
        fz += W.c1[k] * (den[p + k * L.pitch] - den[p - k * L.pitch]);
        fx += W.c1[k] * (den[p + k] - den[p - k]);
    }
    Gz[p] = __fdiv_rn(W.s1[0] * fz, den[p]);
    Gx[p] = __fdiv_rn(W.s1[1] * fx, den[p]);
}

// The ring of interior points next to the halo (the Dirichlet lines): the
// rows z = r and z = nz-r-1 over the interior columns, then the columns
// x = r and x = nx-r-1 over the rows strictly between those two.
__host__ __device__ __forceinline__ long long ring_length(const Layout& L) {
    const long long w = L.nx - 2 * L.r, h = L.nz - 2 * L.r - 2;
    return 2 * w + 2 * h;
}

__device__ __forceinline__ long long ring_index(const Layout& L, long long i, long long j) {
    const int r = L.r;
    const long long w = L.nx - 2 * r, h = L.nz - 2 * r - 2;
    if (i == r) return j - r;
    if (i == L.nz - r - 1) return w + (j - r);
    if (j == r) return 2 * w + (i - r - 1);
    if (j == L.nx - r - 1) return 2 * w + h + (i - r - 1);
    return -1;
}

__global__ void save_ring(const float* __restrict__ u, Layout L, float* __restrict__ ring) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int r = L.r;
    const long long w = L.nx - 2 * r, h = L.nz - 2 * r - 2;
    long long i, j;
    if (t < w) { i = r; j = r + t; }
    else if (t < 2 * w) { i = L.nz - r - 1; j = r + (t - w); }
    else if (t < 2 * w + h) { i = r + 1 + (t - 2 * w); j = r; }
    else if (t < 2 * w + 2 * h) { i = r + 1 + (t - 2 * w - h); j = L.nx - r - 1; }
    else return;
    ring[t] = u[L.at2(i, j)];
}

// Transposed boundary operation of one edge (after: edge 1, before: edge 0)
// on the line at index `line` of the other axis. `nu1` is the previous
// adjoint level (zero halo), read for A^T nu^(m+1) at the halo points; `Ga`
// the density term of `axis` (variable density) or null.
__device__ __forceinline__ void fold_edge(float* __restrict__ nu, const float* __restrict__ nu1,
                                          const float* __restrict__ C, const Layout& L,
                                          const Weights<float>& W, int axis, long long line,
                                          int edge, int type, const float* __restrict__ Ga) {
    if (type == 0) return;
    const int r = L.r;
    const int other = axis == 0 ? 1 : 0;
    long long idx[2];
    idx[other] = line;
    idx[axis] = edge ? L.extent(axis) - r - 1 : r;
    const long long first = L.at2(idx[0], idx[1]);
    if (type == 1) {
        nu[first] = 0.0f;
        return;
    }
    // Neumann: halo a = first + dir q step mirrors b = first - dir q step
    const long long step = L.stride(axis);
    const float ih2 = W.ih2[axis];
    const long long inward = edge ? -step : step;
    for (int q = 1; q <= r; q++) {
        float lam = 0.0f;
        for (int k = q; k <= r; k++) lam += W.c2[k] * nu1[first + (k - q) * inward];
        const long long b = first + q * inward;
        if (Ga) {
            // the halo point's first difference reaches the interior on the
            // inward side only: + before the interior, - after it
            float d = 0.0f;
            for (int k = q; k <= r; k++) {
                const long long pk_ = first + (k - q) * inward;
                d += W.c1[k] * (Ga[pk_] * nu1[pk_]);
            }
            nu[b] += C[b] * (lam * ih2 + (edge ? -d : d));
        } else {
            nu[b] += C[b] * (lam * ih2);
        }
    }
}

// Transposed boundary operations of the edges normal to `axis`, one thread
// per line: the after edge, then the before edge (the forward applies them
// in the opposite order; they touch disjoint points).
__global__ void fold_phase(float* __restrict__ nu, const float* __restrict__ nu1,
                           const float* __restrict__ C, Layout L, Weights<float> W, int axis,
                           int before, int after, const float* __restrict__ Ga) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= boundary_lines(L, axis)) return;
    fold_edge(nu, nu1, C, L, W, axis, L.r + t, 1, after, Ga);
    fold_edge(nu, nu1, C, L, W, axis, L.r + t, 0, before, Ga);
}

// Receiver transposes of table point t (receiver order within the point,
// no atomics, so the sum order is fixed): nu[p] += C[p] * sum_e wt[e] g[rec[e]].
__device__ __forceinline__ void inject_point(float* __restrict__ nu, const float* __restrict__ C,
                                             const long long* __restrict__ pts,
                                             const int* __restrict__ rowptr,
                                             const int* __restrict__ rec,
                                             const float* __restrict__ wt,
                                             const float* __restrict__ g_row, int t) {
    float s = 0.0f;
    for (int e = rowptr[t]; e < rowptr[t + 1]; e++) s += wt[e] * g_row[rec[e]];
    const long long p = pts[t];
    nu[p] += C[p] * s;
}

__global__ void adjoint_receivers(float* __restrict__ nu, const float* __restrict__ C,
                                  const long long* __restrict__ pts,
                                  const int* __restrict__ rowptr, const int* __restrict__ rec,
                                  const float* __restrict__ wt,
                                  const float* __restrict__ g_row, int npts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < npts) inject_point(nu, C, pts, rowptr, rec, wt, g_row, t);
}

// grad += nu^m K (w^m - 2 u^(m-1) + u^(m-2)) at interior point (i, j); w^m
// comes from the saved ring where `ring` is set.
__device__ __forceinline__ void accumulate_point(float* __restrict__ grad,
                                                 const float* __restrict__ nu,
                                                 const float* __restrict__ u_m,
                                                 const float* __restrict__ u_m1,
                                                 const float* __restrict__ u_m2,
                                                 const float* __restrict__ K,
                                                 const float* __restrict__ ring, const Layout& L,
                                                 long long i, long long j) {
    const long long p = L.at2(i, j);
    float w = u_m[p];
    if (ring) {
        const long long ri = ring_index(L, i, j);
        if (ri >= 0) w = ring[ri];
    }
    const float d2 = (w - 2.0f * u_m1[p]) + u_m2[p];
    grad[p] += nu[p] * K[p] * d2;
}

__global__ void accumulate_gradient(float* __restrict__ grad, const float* __restrict__ nu,
                                    const float* __restrict__ u_m,
                                    const float* __restrict__ u_m1,
                                    const float* __restrict__ u_m2,
                                    const float* __restrict__ K,
                                    const float* __restrict__ ring, Layout L) {
    const int r = L.r;
    const long long j = r + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long i = r + blockIdx.y * (long long)blockDim.y + threadIdx.y;
    if (j >= L.nx - r || i >= L.nz - r) return;
    accumulate_point(grad, nu, u_m, u_m1, u_m2, K, ring, L, i, j);
}

// ---- one adjoint step in one launch -----------------------------------------
// Tiles of 16 x 128 interior points, as in the forward's tiled kernel. A CTA
// computes the stencil on nu for its tile, then, for the points it owns, the
// receiver transposes (the table is tile-major), the transposed z edges, the
// transposed x edges and the gradient terms -- the separate kernels' order,
// exact when the first and last tiles hold r + 1 rows and columns (an
// edge's fold reaches r points in from the edge line).
struct AdjointTiles {
    Layout L;
    const float *C, *Q, *K;
    const float *Gz, *Gx;  // variable density: the density terms, else null
    Weights<float> W;
    int zb[4];
    int bc[4];
    int tiles_x, tiles_z;
    int zoff;  // the 16-row tiles start zoff rows above the interior
    const long long* pts;
    const int *rowptr, *rec, *tile_ptr;
    const float* wt;
    float* grad;
};

extern __shared__ __align__(16) float4 sw_grad_smem[];

template <int R, bool VD>
__device__ __forceinline__ void adjoint_tile_step(const AdjointTiles& A, int t, float* num,
                                                  const float* nu1, const float* nu2,
                                                  const float* g_row, const float* u_m,
                                                  const float* u_m1, const float* u_m2,
                                                  const float* ring) {
    const int tz = t / A.tiles_x, tx = t - (t / A.tiles_x) * A.tiles_x;
    const Layout& L = A.L;
    if (VD)
        batch::adjoint2d_density_tile<R, 16>(reinterpret_cast<float*>(sw_grad_smem), L, num,
                                             nu1, nu2, A.C, A.Q, A.Gz, A.Gx, A.W, A.zb, tz, tx,
                                             A.zoff);
    else
        batch::stencil2d_tile<R, false, 16>(reinterpret_cast<float*>(sw_grad_smem), L, num, nu1,
                                            nu2, A.C, A.Q, nullptr, A.W, A.zb, tz, tx, A.zoff);
    __syncthreads();
    if (A.pts)
        for (int e = A.tile_ptr[t] + threadIdx.x; e < A.tile_ptr[t + 1]; e += blockDim.x)
            inject_point(num, A.C, A.pts, A.rowptr, A.rec, A.wt, g_row, e);
    __syncthreads();
    const int nz = (int)L.nz, nx = (int)L.nx;
    const int z0 = max(R + 16 * tz - A.zoff, R), z1 = min(R + 16 * (tz + 1) - A.zoff, nz - R);
    const int x0 = R + 128 * tx, x1 = min(x0 + 128, nx - R);
    // transposed order: z edges (the columns of this tile), then x edges
    if ((tz == A.tiles_z - 1 && A.bc[1]) || (tz == 0 && A.bc[0])) {
        for (int c = x0 + threadIdx.x; c < x1; c += blockDim.x) {
            if (tz == A.tiles_z - 1) fold_edge(num, nu1, A.C, L, A.W, 0, c, 1, A.bc[1], A.Gz);
            if (tz == 0) fold_edge(num, nu1, A.C, L, A.W, 0, c, 0, A.bc[0], A.Gz);
        }
    }
    __syncthreads();
    if ((tx == A.tiles_x - 1 && A.bc[3]) || (tx == 0 && A.bc[2])) {
        for (int i = z0 + threadIdx.x; i < z1; i += blockDim.x) {
            if (tx == A.tiles_x - 1) fold_edge(num, nu1, A.C, L, A.W, 1, i, 1, A.bc[3], A.Gx);
            if (tx == 0) fold_edge(num, nu1, A.C, L, A.W, 1, i, 0, A.bc[2], A.Gx);
        }
    }
    __syncthreads();
    const int w = x1 - x0;
    for (int q = threadIdx.x; q < (z1 - z0) * w; q += blockDim.x) {
        const int i = z0 + q / w, j = x0 + q % w;
        accumulate_point(A.grad, num, u_m, u_m1, u_m2, A.K, ring, L, i, j);
    }
}

template <int R, bool VD>
__global__ void __launch_bounds__(batch::kThreads)
adjoint2d_step(const AdjointTiles A, float* num, const float* nu1, const float* nu2,
               const float* g_row, const float* u_m, const float* u_m1, const float* u_m2,
               const float* ring) {
    adjoint_tile_step<R, VD>(A, blockIdx.x, num, nu1, nu2, g_row, u_m, u_m1, u_m2, ring);
}

// One adjoint step of several shots of one layout in one launch (the
// lockstep reverse pass): `tiles` blocks a shot. Adjoint levels i_num,
// i_nu1, i_nu2 of the shot's array nu, forward levels u^m, u^(m-1), u^(m-2)
// at k + 1, k, k - 1 of its segment array, cotangent row m - 1, ring row at
// element `ring_off`; the gradient terms go to the shot's own grid (A.grad).
struct AdjShot {
    AdjointTiles A;
    float* nu;
    const float* seg;
    const float* g;
    const float* ring;
    int nrec;
};

template <int R, bool VD>
__global__ void __launch_bounds__(batch::kThreads)
adjoint2d_step_shots(const AdjShot* __restrict__ shots, int tiles, long long G, int i_num,
                     int i_nu1, int i_nu2, int k, long long m, long long ring_off) {
    const int s = blockIdx.x / tiles, t = blockIdx.x - s * tiles;
    const AdjShot& Q = shots[s];
    adjoint_tile_step<R, VD>(Q.A, t, Q.nu + i_num * G, Q.nu + i_nu1 * G, Q.nu + i_nu2 * G,
                             Q.g + (m - 1) * Q.nrec, Q.seg + (k + 1) * G, Q.seg + k * G,
                             Q.seg + (k - 1) * G, Q.ring ? Q.ring + ring_off : nullptr);
}

// Tile stencil of the adjoint alone (the separate-kernel path): nu_next
// from nu, nu_prev over 16 x 128 tiles.
template <int R, bool VD>
__global__ void __launch_bounds__(batch::kThreads)
adjoint2d_tiles(const AdjointTiles A, float* num, const float* nu1, const float* nu2) {
    const int t = blockIdx.x;
    const int tz = t / A.tiles_x, tx = t - (t / A.tiles_x) * A.tiles_x;
    if (VD)
        batch::adjoint2d_density_tile<R, 16>(reinterpret_cast<float*>(sw_grad_smem), A.L, num,
                                             nu1, nu2, A.C, A.Q, A.Gz, A.Gx, A.W, A.zb, tz, tx,
                                             A.zoff);
    else
        batch::stencil2d_tile<R, false, 16>(reinterpret_cast<float*>(sw_grad_smem), A.L, num,
                                            nu1, nu2, A.C, A.Q, nullptr, A.W, A.zb, tz, tx,
                                            A.zoff);
}

template <int R, bool VD>
static void adjoint_r(const AdjointTiles& A, bool fused, float* num, const float* nu1,
                      const float* nu2, const float* g_row, const float* u_m,
                      const float* u_m1, const float* u_m2, const float* ring,
                      cudaStream_t st) {
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 3 : 1) * (16 + 2 * R) * (128 + 2 * HX) * 4;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    GR_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        GR_CUDA(cudaFuncSetAttribute(adjoint2d_step<R, VD>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        GR_CUDA(cudaFuncSetAttribute(adjoint2d_tiles<R, VD>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        configured[dev & 63] = true;
    }
    if (fused)
        adjoint2d_step<R, VD><<<A.tiles_x * A.tiles_z, batch::kThreads, bytes, st>>>(
            A, num, nu1, nu2, g_row, u_m, u_m1, u_m2, ring);
    else
        adjoint2d_tiles<R, VD><<<A.tiles_x * A.tiles_z, batch::kThreads, bytes, st>>>(
            A, num, nu1, nu2);
}

// The adjoint step in one launch (`fused`), or its tile stencil alone.
static void adjoint_launch(const AdjointTiles& A, bool fused, float* num, const float* nu1,
                           const float* nu2, const float* g_row, const float* u_m,
                           const float* u_m1, const float* u_m2, const float* ring,
                           cudaStream_t st) {
    const bool vd = A.Gz != nullptr;
#define GR_A(RR)                                                                            \
    case RR:                                                                                \
        if (vd) adjoint_r<RR, true>(A, fused, num, nu1, nu2, g_row, u_m, u_m1, u_m2, ring, st); \
        else adjoint_r<RR, false>(A, fused, num, nu1, nu2, g_row, u_m, u_m1, u_m2, ring, st);   \
        break;
    switch (A.L.r) {
        GR_A(1) GR_A(2) GR_A(3) GR_A(4) GR_A(5) GR_A(6) GR_A(7) GR_A(8) GR_A(9) GR_A(10)
    }
#undef GR_A
}

template <int R, bool VD>
static void adjoint_shots_r(const AdjShot* shots, int nshots, int tiles, long long G, int i_num,
                            int i_nu1, int i_nu2, int k, long long m, long long ring_off,
                            cudaStream_t st) {
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 3 : 1) * (16 + 2 * R) * (128 + 2 * HX) * 4;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    GR_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        GR_CUDA(cudaFuncSetAttribute(adjoint2d_step_shots<R, VD>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        configured[dev & 63] = true;
    }
    adjoint2d_step_shots<R, VD><<<nshots * tiles, batch::kThreads, bytes, st>>>(
        shots, tiles, G, i_num, i_nu1, i_nu2, k, m, ring_off);
}

static void adjoint_launch_shots(const AdjShot* shots, int nshots, int tiles, int r, bool vd,
                                 long long G, int i_num, int i_nu1, int i_nu2, int k,
                                 long long m, long long ring_off, cudaStream_t st) {
#define GR_AS(RR)                                                                        \
    case RR:                                                                             \
        if (vd) adjoint_shots_r<RR, true>(shots, nshots, tiles, G, i_num, i_nu1, i_nu2, k, m, \
                                          ring_off, st);                                 \
        else adjoint_shots_r<RR, false>(shots, nshots, tiles, G, i_num, i_nu1, i_nu2, k, m, \
                                        ring_off, st);                                   \
        break;
    switch (r) {
        GR_AS(1) GR_AS(2) GR_AS(3) GR_AS(4) GR_AS(5) GR_AS(6) GR_AS(7) GR_AS(8) GR_AS(9) GR_AS(10)
    }
#undef GR_AS
}

// out += sum of the shots' gradient grids
__global__ void sum_grids(float* __restrict__ out, const float* __restrict__ grids, int nshots,
                          long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float acc = out[i];
        for (int s = 0; s < nshots; s++) acc += grids[(long long)s * n + i];
        out[i] = acc;
    }
}

// ---------------------------------------------------------------------------
// host side

struct Scratch {
    cudaStream_t st;
    std::vector<void*> blocks;
    explicit Scratch(cudaStream_t s) : st(s) {}
    template <typename T>
    T* get(size_t count) {
        void* p = nullptr;
        GR_CUDA(cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), st));
        blocks.push_back(p);
        return static_cast<T*>(p);
    }
    ~Scratch() {
        for (void* p : blocks) cudaFreeAsync(p, st);
    }
};

struct Ctx {
    Layout L;
    Weights<float> W;
    float dt;
    const float* vel;
    const float* damp;
    const float* den = nullptr;  // variable density, else null
    bool vd = false;
    const float* wavelet;
    size_t wavelet_count;
    Windows<float> src, rec;
    int bc[4];
    size_t begin, end;
    float* C = nullptr;
    float* Q = nullptr;
    int zero_box[6] = {0, 0, 0, 0, 0, 0};
    bool tiled = false;
    long long grid = 0;  // elements of one grid (nz * pitch)
    bool dirichlet = false;
    float* receivers = nullptr;
    // one launch per step (tiled, owner-computes sources and edges): with
    // the receiver record, and without it (recomputed segments)
    bool fused = false;
    Shot2D shot{}, shot_quiet{};
};

// Checks the problem and copies the windows to the host (`src_iv`, ...).
struct HostWindows {
    std::vector<size_t> iv, off;
    std::vector<float> val;
};

static void fetch_windows(const size_t* div, const float* dval, const size_t* doff,
                          size_t val_size, size_t count, HostWindows& H, cudaStream_t st) {
    H.iv.assign(count * 4, 0);
    H.off.assign(count + 1, 0);
    H.val.assign(val_size, 0.0f);
    if (!count) return;
    GR_CUDA(cudaMemcpyAsync(H.iv.data(), div, H.iv.size() * sizeof(size_t),
                            cudaMemcpyDeviceToHost, st));
    GR_CUDA(cudaMemcpyAsync(H.off.data(), doff, count * sizeof(size_t),
                            cudaMemcpyDeviceToHost, st));
    if (val_size)
        GR_CUDA(cudaMemcpyAsync(H.val.data(), dval, val_size * sizeof(float),
                                cudaMemcpyDeviceToHost, st));
    GR_CUDA(cudaStreamSynchronize(st));
}

static void check_interior_windows(const char* what, const HostWindows& H, size_t count,
                                   const Layout& L) {
    for (size_t s = 0; s < count; s++) {
        const size_t* b = &H.iv[s * 4];
        const long long ext[2] = {L.nz, L.nx};
        for (int a = 0; a < 2; a++) {
            if (b[2 * a] > b[2 * a + 1] || (long long)b[2 * a] < L.r ||
                (long long)b[2 * a + 1] > ext[a] - L.r - 1)
                refuse(SIMWAVE_E_ARGUMENT,
                       std::string(what) + " window " + std::to_string(s) +
                           " reaches the halo or is empty (the gradient needs "
                           "windows inside the interior)");
        }
        const size_t len = (b[1] - b[0] + 1) + (b[3] - b[2] + 1);
        if (H.off[s] + len > H.val.size())
            refuse(SIMWAVE_E_ARGUMENT, std::string(what) + " values offsets out of range");
    }
}

static Ctx make_ctx(const simwave_problem* P, cudaStream_t st, HostWindows* rec_out) {
    if (!P) refuse(SIMWAVE_E_ARGUMENT, "null problem");
    if (P->dim != 2 || P->precision != 4)
        refuse(SIMWAVE_E_ARGUMENT, "the gradient supports 2D float32 problems");
    if (P->variable_density && (!P->density || !P->coeff_order1))
        refuse(SIMWAVE_E_ARGUMENT, "variable density needs the density and the first-order weights");
    if (P->space_order < 2 || P->space_order > 2 * kMaxRadius || P->space_order % 2)
        refuse(SIMWAVE_E_ARGUMENT, "space_order must be even, 2..20");
    if (!P->velocity || !P->damp || !P->coeff_order2 || !P->boundary_conditions ||
        (P->num_sources && (!P->wavelet || !P->src_points_interval ||
                            !P->src_points_values || !P->src_points_values_offset)) ||
        (P->num_receivers && (!P->receivers || !P->rec_points_interval ||
                              !P->rec_points_values || !P->rec_points_values_offset)))
        refuse(SIMWAVE_E_ARGUMENT, "null array argument");
    if (P->begin_timestep < 1 || P->end_timestep < P->begin_timestep)
        refuse(SIMWAVE_E_ARGUMENT, "need 1 <= begin_timestep <= end_timestep");
    if (P->num_sources && P->wavelet_size < P->end_timestep)
        refuse(SIMWAVE_E_ARGUMENT, "wavelet shorter than end_timestep");
    if (P->num_sources && P->wavelet_count != 1 && P->wavelet_count != P->num_sources)
        refuse(SIMWAVE_E_ARGUMENT, "wavelet_count must be 1 or num_sources");
    Ctx X;
    const int r = P->space_order / 2;
    X.L.dim = 2;
    X.L.r = r;
    X.L.nz = (long long)P->nz;
    X.L.nx = (long long)P->nx;
    X.L.ny = 1;
    X.L.pitch = (long long)P->pitch;
    X.L.lead = (long long)P->lead;
    X.L.plane = X.L.pitch;
    X.L.slot = X.L.nz * X.L.pitch;
    X.grid = X.L.slot;
    if (P->pitch < P->lead + P->nx) refuse(SIMWAVE_E_ARGUMENT, "pitch < lead + nx");
    // interior lines of opposite edges must not overlap (Neumann mirrors)
    if (X.L.nz - 2 * r < 2 * r + 2 || X.L.nx - 2 * r < 2 * r + 2)
        refuse(SIMWAVE_E_ARGUMENT, "grid too small for the space order");
    for (int e = 0; e < 4; e++) {
        if (P->boundary_conditions[e] > 2)
            refuse(SIMWAVE_E_ARGUMENT, "boundary code must be 0, 1 or 2");
        X.bc[e] = (int)P->boundary_conditions[e];
        X.dirichlet |= X.bc[e] == 1;
    }
    HostWindows S;
    fetch_windows(P->src_points_interval, (const float*)P->src_points_values,
                  P->src_points_values_offset, P->src_points_values_size, P->num_sources, S,
                  st);
    check_interior_windows("source", S, P->num_sources, X.L);
    HostWindows R;
    fetch_windows(P->rec_points_interval, (const float*)P->rec_points_values,
                  P->rec_points_values_offset, P->rec_points_values_size, P->num_receivers,
                  R, st);
    check_interior_windows("receiver", R, P->num_receivers, X.L);
    if (rec_out) *rec_out = std::move(R);
    X.vd = P->variable_density != 0;
    X.den = X.vd ? (const float*)P->density : nullptr;
    X.W = make_weights<float>((const float*)P->coeff_order2,
                              X.vd ? (const float*)P->coeff_order1 : nullptr, r, P->dz, P->dx,
                              1.0);
    X.dt = (float)P->dt;
    X.vel = (const float*)P->velocity;
    X.damp = (const float*)P->damp;
    X.wavelet = (const float*)P->wavelet;
    X.wavelet_count = P->wavelet_count;
    X.src = Windows<float>{P->src_points_interval, (const float*)P->src_points_values,
                           P->src_points_values_offset, P->num_sources};
    X.rec = Windows<float>{P->rec_points_interval, (const float*)P->rec_points_values,
                           P->rec_points_values_offset, P->num_receivers};
    X.begin = P->begin_timestep;
    X.end = P->end_timestep;
    X.receivers = (float*)P->receivers;
    return X;
}

// Per-point coefficients C, Q of the forward stencil and the damping-free box.
static void prepare_coefficients(Ctx& X, Scratch& mem, bool aligned) {
    X.C = mem.get<float>((size_t)X.grid);
    X.Q = mem.get<float>((size_t)X.grid);
    form_coefficients(X.vel, X.damp, X.C, X.Q, X.grid, X.dt, mem.st);
    GR_LAUNCHED("form_coefficients");
    X.tiled = aligned && tiled2d_supported(X.L) &&
              (!X.vd || (reinterpret_cast<uintptr_t>(X.den) & 15) == 0);
    if (!X.tiled) {
        if (X.vd)
            refuse(SIMWAVE_E_ARGUMENT,
                   "the variable-density gradient needs the tiled layout (simwave_layout())");
        return;
    }
    int* words = mem.get<int>(16);
    find_zero_box(X.Q, X.L, words, mem.st);
    GR_LAUNCHED("find_zero_box");
    int box[7];
    GR_CUDA(cudaMemcpyAsync(box, words, sizeof(box), cudaMemcpyDeviceToHost, mem.st));
    GR_CUDA(cudaStreamSynchronize(mem.st));
    const bool good = box[6] == 0 && box[1] > box[0] && box[3] > box[2];
    for (int i = 0; i < 6; i++) X.zero_box[i] = good ? box[i] : 0;
    X.fused = shot2d_prepare(X.shot, X.L, X.C, X.Q, X.den, X.vel, X.damp, X.W, X.zero_box,
                             X.src, X.wavelet, X.wavelet_count, X.dt, X.rec, X.receivers,
                             X.bc) &&
              X.shot.fused;
    X.shot_quiet = X.shot;
    X.shot_quiet.rec.count = 0;
    if (!X.receivers) X.shot.rec.count = 0;
}

// The forward stencil on (un, uc, up): the tiled kernel on C and Q, else the
// one-thread-per-point kernel.
static void stencil(const Ctx& X, float* un, const float* uc, const float* up,
                    cudaStream_t st) {
    if (X.tiled) {
        tiled2d_launch(X.L, X.vd, un, uc, up, X.C, X.Q, X.den, X.W, X.zero_box, st);
        GR_LAUNCHED("stencil2d_single");
        return;
    }
    const int r = X.L.r;
    dim3 block(32, 8, 1);
    dim3 grid((unsigned)((X.L.nx - 2 * r + 31) / 32), (unsigned)((X.L.nz - 2 * r + 7) / 8), 1);
    stencil_generic<float, 2, false><<<grid, block, 0, st>>>(
        un, uc, up, X.vel, nullptr, X.damp, X.L, X.W, X.dt, X.dt * X.dt);
    GR_LAUNCHED("stencil_generic");
}

// One forward step n: u^(n+1) into un from uc = u^n, up = u^(n-1); the
// values of the Dirichlet lines before the boundary conditions into
// `ring_row`, the record of u^n into `rec_row` (either may be null).
static void forward_step(const Ctx& X, float* un, const float* uc, const float* up,
                         size_t n, float* ring_row, float* rec_row, cudaStream_t st) {
    if (X.fused) {
        // the record goes to X.receivers + (n - 1) * count, where rec_row points
        step2d_launch(rec_row ? X.shot : X.shot_quiet, X.vd, un, uc, up, (long long)n, st,
                      ring_row);
        GR_LAUNCHED("stencil2d_step");
        return;
    }
    stencil(X, un, uc, up, st);
    if (X.src.count) {
        inject_sources<float, 2><<<(unsigned)X.src.count, 128, 0, st>>>(
            un, X.vel, X.damp, X.L, X.src, X.wavelet, X.wavelet_count, n, X.dt,
            X.dt * X.dt);
        GR_LAUNCHED("inject_sources");
    }
    if (ring_row) {
        const long long len = ring_length(X.L);
        save_ring<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(un, X.L, ring_row);
        GR_LAUNCHED("save_ring");
    }
    const int phases[2] = {1, 0};  // x edges, then z edges
    for (int a : phases) {
        const int b0 = X.bc[2 * a], b1 = X.bc[2 * a + 1];
        if (!b0 && !b1) continue;
        const long long lines = boundary_lines(X.L, a);
        boundary_phase<float><<<(unsigned)((lines + 255) / 256), 256, 0, st>>>(un, X.L, a,
                                                                               b0, b1);
        GR_LAUNCHED("boundary_phase");
    }
    if (rec_row && X.rec.count) {
        const size_t threads = X.rec.count * 32;
        record_receivers<float, 2><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
            rec_row, uc, X.L, X.rec);
        GR_LAUNCHED("record_receivers");
    }
}

static size_t checkpoint_count(size_t steps, size_t interval) {
    return (steps + interval - 1) / interval;
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

static void forward_pass(const simwave_problem* P, size_t interval, float* ck,
                         cudaStream_t st) {
    if (interval < 1) refuse(SIMWAVE_E_ARGUMENT, "interval must be >= 1");
    if (!ck) refuse(SIMWAVE_E_ARGUMENT, "null checkpoint buffer");
    Ctx X = make_ctx(P, st, nullptr);
    Scratch mem(st);
    float* lev = mem.get<float>(3 * (size_t)X.grid);
    GR_CUDA(cudaMemsetAsync(lev, 0, 3 * (size_t)X.grid * sizeof(float), st));
    prepare_coefficients(X, mem, aligned16(lev));
    const size_t bytes = (size_t)X.grid * sizeof(float);
    float* rec = (float*)P->receivers;
    for (size_t n = X.begin; n <= X.end; n++) {
        float* un = lev + ((n + 1) % 3) * X.grid;
        const float* uc = lev + (n % 3) * X.grid;
        const float* up = lev + ((n + 2) % 3) * X.grid;  // (n - 1) mod 3
        const size_t i = n - X.begin;
        if (i % interval == 0) {
            float* dst = ck + 2 * (i / interval) * X.grid;
            GR_CUDA(cudaMemcpyAsync(dst, up, bytes, cudaMemcpyDeviceToDevice, st));
            GR_CUDA(cudaMemcpyAsync(dst + X.grid, uc, bytes, cudaMemcpyDeviceToDevice, st));
        }
        forward_step(X, un, uc, up, n, nullptr, rec ? rec + (n - 1) * X.rec.count : nullptr,
                     st);
    }
}

// Receiver transposes as a point-major table (receiver order within a
// point), points grouped by the 16 x 128 interior tile that holds them
// (`tile_ptr`: each tile's range) and in grid order within a tile.
struct AdjointTable {
    long long* pts = nullptr;
    int* rowptr = nullptr;
    int* rec = nullptr;
    float* wt = nullptr;
    int* tile_ptr = nullptr;
    int npts = 0;
};

static AdjointTable build_table(const HostWindows& H, size_t count, const Layout& L, int zoff,
                                Scratch& mem) {
    struct Entry {
        long long p;
        int s;
        float w;
        int tile;
    };
    const int r = L.r;
    const int tiles_x = (int)((L.nx - 2 * r + 127) / 128);
    const int tiles_z = (int)((L.nz - 2 * r + zoff + 15) / 16);
    auto tile_of = [&](long long z, long long x) {
        const long long tz =
            std::min<long long>(std::max<long long>(z - r + zoff, 0) / 16, tiles_z - 1);
        const long long tx = std::min<long long>(std::max<long long>(x - r, 0) / 128, tiles_x - 1);
        return (int)(tz * tiles_x + tx);
    };
    std::vector<Entry> e;
    for (size_t s = 0; s < count; s++) {
        const size_t* b = &H.iv[s * 4];
        const size_t lz = b[1] - b[0] + 1, lx = b[3] - b[2] + 1;
        const float* kz = H.val.data() + H.off[s];
        const float* kx = kz + lz;
        for (size_t iz = 0; iz < lz; iz++)
            for (size_t ix = 0; ix < lx; ix++)
                e.push_back({L.at2((long long)(b[0] + iz), (long long)(b[2] + ix)), (int)s,
                             kz[iz] * kx[ix],
                             tile_of((long long)(b[0] + iz), (long long)(b[2] + ix))});
    }
    std::stable_sort(e.begin(), e.end(), [](const Entry& a, const Entry& b) {
        return a.tile != b.tile ? a.tile < b.tile : a.p < b.p;
    });
    std::vector<long long> pts;
    std::vector<int> rowptr{0}, rec, tile_ptr(tiles_x * tiles_z + 1, 0);
    std::vector<float> wt;
    for (size_t k = 0; k < e.size(); k++) {
        if (k == 0 || e[k].p != e[k - 1].p) {
            if (k) rowptr.push_back((int)rec.size());
            pts.push_back(e[k].p);
            tile_ptr[e[k].tile + 1]++;
        }
        rec.push_back(e[k].s);
        wt.push_back(e[k].w);
    }
    if (!e.empty()) rowptr.push_back((int)rec.size());
    for (size_t t = 1; t < tile_ptr.size(); t++) tile_ptr[t] += tile_ptr[t - 1];
    AdjointTable T;
    T.npts = (int)pts.size();
    if (!T.npts) return T;
    T.tile_ptr = mem.get<int>(tile_ptr.size());
    GR_CUDA(cudaMemcpyAsync(T.tile_ptr, tile_ptr.data(), tile_ptr.size() * sizeof(int),
                            cudaMemcpyHostToDevice, mem.st));
    T.pts = mem.get<long long>(pts.size());
    T.rowptr = mem.get<int>(rowptr.size());
    T.rec = mem.get<int>(rec.size());
    T.wt = mem.get<float>(wt.size());
    GR_CUDA(cudaMemcpyAsync(T.pts, pts.data(), pts.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, mem.st));
    GR_CUDA(cudaMemcpyAsync(T.rowptr, rowptr.data(), rowptr.size() * sizeof(int),
                            cudaMemcpyHostToDevice, mem.st));
    GR_CUDA(cudaMemcpyAsync(T.rec, rec.data(), rec.size() * sizeof(int),
                            cudaMemcpyHostToDevice, mem.st));
    GR_CUDA(cudaMemcpyAsync(T.wt, wt.data(), wt.size() * sizeof(float),
                            cudaMemcpyHostToDevice, mem.st));
    // the host vectors die at return: wait for the copies
    GR_CUDA(cudaStreamSynchronize(mem.st));
    return T;
}

static void reverse_pass(const simwave_problem* P, size_t interval, const float* ck,
                         const float* g, float* grad, cudaStream_t st) {
    if (interval < 1) refuse(SIMWAVE_E_ARGUMENT, "interval must be >= 1");
    if (!ck || !grad || (P && P->num_receivers && !g))
        refuse(SIMWAVE_E_ARGUMENT, "null checkpoint, cotangent or gradient buffer");
    HostWindows R;
    Ctx X = make_ctx(P, st, &R);
    Scratch mem(st);
    const size_t G = (size_t)X.grid, bytes = G * sizeof(float);
    const size_t steps = X.end - X.begin + 1;
    const size_t K = std::min(interval, steps);
    float* seg = mem.get<float>((K + 2) * G);
    float* nu = mem.get<float>(3 * G);
    float* Kf = mem.get<float>(G);
    const long long ring_len = ring_length(X.L);
    float* ring = X.dirichlet ? mem.get<float>(K * (size_t)ring_len) : nullptr;
    GR_CUDA(cudaMemsetAsync(seg, 0, (K + 2) * bytes, st));
    GR_CUDA(cudaMemsetAsync(nu, 0, 3 * bytes, st));
    GR_CUDA(cudaMemsetAsync(grad, 0, bytes, st));
    prepare_coefficients(X, mem, aligned16(seg) && aligned16(nu));
    gradient_factor<<<1024, 256, 0, st>>>(X.vel, Kf, (long long)G, X.dt);
    GR_LAUNCHED("gradient_factor");
    const AdjointTable T = build_table(R, P->num_receivers, X.L, X.tiled ? X.shot.zoff : 0, mem);
    float *Gz = nullptr, *Gx = nullptr;
    if (X.vd) {
        Gz = mem.get<float>(2 * G);
        Gx = Gz + G;
        GR_CUDA(cudaMemsetAsync(Gz, 0, 2 * bytes, st));
        const int rr = X.L.r;
        const dim3 blk(32, 8, 1);
        const dim3 grd((unsigned)((X.L.nx - 2 * rr + 31) / 32),
                       (unsigned)((X.L.nz - 2 * rr + 7) / 8), 1);
        density_terms<<<grd, blk, 0, st>>>(X.den, Gz, Gx, X.L, X.W);
        GR_LAUNCHED("density_terms");
    }
    AdjointTiles A{};
    if (X.tiled) {
        A.Gz = Gz;
        A.Gx = Gx;
        A.L = X.L;
        A.C = X.C;
        A.Q = X.Q;
        A.K = Kf;
        A.W = X.W;
        for (int i = 0; i < 4; i++) {
            A.zb[i] = X.zero_box[i];
            A.bc[i] = X.bc[i];
        }
        A.tiles_x = X.shot.tiles_x;
        A.tiles_z = X.shot.tiles_z;
        A.zoff = X.shot.zoff;
        A.pts = T.npts ? T.pts : nullptr;
        A.rowptr = T.rowptr;
        A.rec = T.rec;
        A.wt = T.wt;
        A.tile_ptr = T.tile_ptr;
        A.grad = grad;
    }

    const int r = X.L.r;
    const dim3 gblock(32, 8, 1);
    const dim3 ggrid((unsigned)((X.L.nx - 2 * r + 31) / 32),
                     (unsigned)((X.L.nz - 2 * r + 7) / 8), 1);
    const size_t b = X.begin, e = X.end;
    const size_t nck = checkpoint_count(steps, interval);
    for (size_t j = nck; j-- > 0;) {
        const size_t n0 = b + j * interval;
        const size_t n1 = std::min(n0 + interval - 1, e);
        // levels u^(n0-1) .. u^(n1+1) at seg[k - (n0 - 1)]
        GR_CUDA(cudaMemcpyAsync(seg, ck + 2 * j * G, 2 * bytes, cudaMemcpyDeviceToDevice, st));
        for (size_t n = n0; n <= n1; n++) {
            const size_t k = n - n0;
            forward_step(X, seg + (k + 2) * G, seg + (k + 1) * G, seg + k * G, n,
                         ring ? ring + k * (size_t)ring_len : nullptr, nullptr, st);
        }
        for (size_t m = n1 + 1; m >= n0 + 1; m--) {
            if (m == e + 1) continue;  // nu^(e+1) = 0: no record reads u^(e+1)
            float* num = nu + (m % 3) * G;
            const float* nu1 = nu + ((m + 1) % 3) * G;
            const float* nu2 = nu + ((m + 2) % 3) * G;
            if (X.fused) {  // the whole adjoint step in one launch
                const size_t k = m - n0;
                adjoint_launch(A, true, num, nu1, nu2, g + (m - 1) * P->num_receivers,
                               seg + (k + 1) * G, seg + k * G, seg + (k - 1) * G,
                               ring ? ring + (m - 1 - n0) * (size_t)ring_len : nullptr, st);
                GR_LAUNCHED("adjoint2d_step");
                continue;
            }
            if (X.vd) {
                adjoint_launch(A, false, num, nu1, nu2, nullptr, nullptr, nullptr, nullptr,
                               nullptr, st);
                GR_LAUNCHED("adjoint2d_tiles");
            } else {
                stencil(X, num, nu1, nu2, st);
            }
            if (T.npts) {
                adjoint_receivers<<<(unsigned)((T.npts + 255) / 256), 256, 0, st>>>(
                    num, X.C, T.pts, T.rowptr, T.rec, T.wt, g + (m - 1) * P->num_receivers,
                    T.npts);
                GR_LAUNCHED("adjoint_receivers");
            }
            const int phases[2] = {0, 1};  // transposed order: z edges, then x edges
            for (int a : phases) {
                const int b0 = X.bc[2 * a], b1 = X.bc[2 * a + 1];
                if (!b0 && !b1) continue;
                const long long lines = boundary_lines(X.L, a);
                fold_phase<<<(unsigned)((lines + 127) / 128), 128, 0, st>>>(
                    num, nu1, X.C, X.L, X.W, a, b0, b1, a == 0 ? Gz : Gx);
                GR_LAUNCHED("fold_phase");
            }
            const size_t k = m - n0;  // seg index of u^(m-1); u^m at k + 1
            accumulate_gradient<<<ggrid, gblock, 0, st>>>(
                grad, num, seg + (k + 1) * G, seg + k * G, seg + (k - 1) * G, Kf,
                ring ? ring + (m - 1 - n0) * (size_t)ring_len : nullptr, X.L);
            GR_LAUNCHED("accumulate_gradient");
        }
    }
}

// ---- several shots in lockstep -----------------------------------------------
// Shots of one layout, order, density kind and step range (the shots of one
// inversion) advance together: one launch per forward, recomputed or adjoint
// step for all of them (their tiles one after the other), when every shot
// takes the fused step; otherwise one shot after another.

static void check_same(const std::vector<Ctx>& X) {
    for (size_t s = 1; s < X.size(); s++) {
        const Layout &a = X[0].L, &b = X[s].L;
        if (a.nz != b.nz || a.nx != b.nx || a.pitch != b.pitch || a.lead != b.lead ||
            a.r != b.r || X[s].begin != X[0].begin || X[s].end != X[0].end ||
            X[s].vd != X[0].vd)
            refuse(SIMWAVE_E_ARGUMENT,
                   "shots of one call need one layout, space order, density kind and "
                   "step range");
    }
}

static void forward_pass_shots(const simwave_problem* P, size_t ns, size_t interval,
                               float* const* ck, cudaStream_t st) {
    if (interval < 1) refuse(SIMWAVE_E_ARGUMENT, "interval must be >= 1");
    if (!P || !ck) refuse(SIMWAVE_E_ARGUMENT, "null problems or checkpoint buffers");
    if (!ns) return;
    std::vector<Ctx> X;
    for (size_t s = 0; s < ns; s++) {
        if (!ck[s]) refuse(SIMWAVE_E_ARGUMENT, "null checkpoint buffer");
        X.push_back(make_ctx(&P[s], st, nullptr));
    }
    check_same(X);
    Scratch mem(st);
    const size_t G = (size_t)X[0].grid, bytes = G * sizeof(float);
    float* lev = mem.get<float>(3 * G * ns);
    GR_CUDA(cudaMemsetAsync(lev, 0, 3 * bytes * ns, st));
    bool lockstep = true;
    for (size_t s = 0; s < ns; s++) {
        prepare_coefficients(X[s], mem, aligned16(lev) && G % 4 == 0);
        lockstep = lockstep && X[s].tiled && X[s].fused;
    }
    if (!lockstep) {
        for (size_t s = 0; s < ns; s++) forward_pass(&P[s], interval, ck[s], st);
        return;
    }
    std::vector<StepShot> tab(ns);
    int per_shot = 0;
    for (size_t s = 0; s < ns; s++) {
        tab[s] = StepShot{X[s].shot, lev + 3 * G * s, nullptr};
        per_shot = std::max(per_shot, X[s].shot.ntiles +
                                          (int)((X[s].shot.rec.count + batch::kWarps - 1) /
                                                batch::kWarps));
    }
    StepShot* dtab = mem.get<StepShot>(ns);
    GR_CUDA(cudaMemcpyAsync(dtab, tab.data(), ns * sizeof(StepShot), cudaMemcpyHostToDevice, st));
    const Ctx& X0 = X[0];
    for (size_t n = X0.begin; n <= X0.end; n++) {
        const size_t i = n - X0.begin;
        if (i % interval == 0)
            for (size_t s = 0; s < ns; s++) {
                const float* base = lev + 3 * G * s;
                float* dst = ck[s] + 2 * (i / interval) * G;
                GR_CUDA(cudaMemcpyAsync(dst, base + ((n + 2) % 3) * G, bytes,
                                        cudaMemcpyDeviceToDevice, st));
                GR_CUDA(cudaMemcpyAsync(dst + G, base + (n % 3) * G, bytes,
                                        cudaMemcpyDeviceToDevice, st));
            }
        step2d_launch_shots(dtab, (int)ns, per_shot, X0.L.r, X0.vd, (long long)G,
                            (int)((n + 1) % 3), (int)(n % 3), (int)((n + 2) % 3), (long long)n,
                            0, true, st);
        GR_LAUNCHED("stencil2d_step_shots");
    }
    // the table must outlive its copy: wait for the stream before returning
    GR_CUDA(cudaStreamSynchronize(st));
}

static void reverse_pass_shots(const simwave_problem* P, size_t ns, size_t interval,
                               const float* const* ck, const float* const* g, float* grad,
                               cudaStream_t st) {
    if (interval < 1) refuse(SIMWAVE_E_ARGUMENT, "interval must be >= 1");
    if (!P || !ck || !grad || !g) refuse(SIMWAVE_E_ARGUMENT, "null argument");
    if (!ns) return;
    std::vector<Ctx> X;
    std::vector<HostWindows> R(ns);
    for (size_t s = 0; s < ns; s++) {
        if (!ck[s] || (P[s].num_receivers && !g[s]))
            refuse(SIMWAVE_E_ARGUMENT, "null checkpoint or cotangent buffer");
        X.push_back(make_ctx(&P[s], st, &R[s]));
    }
    check_same(X);
    Scratch mem(st);
    const size_t G = (size_t)X[0].grid, bytes = G * sizeof(float);
    const size_t steps = X[0].end - X[0].begin + 1;
    const size_t K = std::min(interval, steps);
    const long long ring_len = ring_length(X[0].L);
    const bool dir = X[0].dirichlet;
    // per shot: segment levels, adjoint levels, the gradient factor, the
    // shot's gradient, the ring rows (Dirichlet edges)
    float* seg = mem.get<float>((K + 2) * G * ns);
    float* nu = mem.get<float>(3 * G * ns);
    float* Kf = mem.get<float>(G * ns);
    float* grads = mem.get<float>(G * ns);
    float* ring = nullptr;
    bool lockstep = true;
    for (size_t s = 0; s < ns; s++) lockstep = lockstep && X[s].dirichlet == dir;
    if (dir) ring = mem.get<float>(K * (size_t)ring_len * ns);
    GR_CUDA(cudaMemsetAsync(seg, 0, (K + 2) * bytes * ns, st));
    GR_CUDA(cudaMemsetAsync(nu, 0, 3 * bytes * ns, st));
    GR_CUDA(cudaMemsetAsync(grads, 0, bytes * ns, st));
    GR_CUDA(cudaMemsetAsync(grad, 0, bytes, st));
    for (size_t s = 0; s < ns; s++) {
        prepare_coefficients(X[s], mem, aligned16(seg) && aligned16(nu) && G % 4 == 0);
        lockstep = lockstep && X[s].tiled && X[s].fused;
    }
    if (!lockstep) {
        for (size_t s = 0; s < ns; s++) {
            reverse_pass(&P[s], interval, ck[s], g[s], grads + s * G, st);
        }
        sum_grids<<<1024, 256, 0, st>>>(grad, grads, (int)ns, (long long)G);
        GR_LAUNCHED("sum_grids");
        GR_CUDA(cudaStreamSynchronize(st));
        return;
    }
    std::vector<AdjShot> adj(ns);
    std::vector<StepShot> rec(ns);
    const int r = X[0].L.r;
    for (size_t s = 0; s < ns; s++) {
        Ctx& Xs = X[s];
        float* Ks = Kf + s * G;
        gradient_factor<<<1024, 256, 0, st>>>(Xs.vel, Ks, (long long)G, Xs.dt);
        GR_LAUNCHED("gradient_factor");
        const AdjointTable T = build_table(R[s], P[s].num_receivers, Xs.L, Xs.shot.zoff, mem);
        float *Gz = nullptr, *Gx = nullptr;
        if (Xs.vd) {
            Gz = mem.get<float>(2 * G);
            Gx = Gz + G;
            GR_CUDA(cudaMemsetAsync(Gz, 0, 2 * bytes, st));
            const dim3 blk(32, 8, 1);
            const dim3 grd((unsigned)((Xs.L.nx - 2 * r + 31) / 32),
                           (unsigned)((Xs.L.nz - 2 * r + 7) / 8), 1);
            density_terms<<<grd, blk, 0, st>>>(Xs.den, Gz, Gx, Xs.L, Xs.W);
            GR_LAUNCHED("density_terms");
        }
        AdjointTiles A{};
        A.L = Xs.L;
        A.C = Xs.C;
        A.Q = Xs.Q;
        A.K = Ks;
        A.Gz = Gz;
        A.Gx = Gx;
        A.W = Xs.W;
        for (int i = 0; i < 4; i++) {
            A.zb[i] = Xs.zero_box[i];
            A.bc[i] = Xs.bc[i];
        }
        A.tiles_x = Xs.shot.tiles_x;
        A.tiles_z = Xs.shot.tiles_z;
        A.zoff = Xs.shot.zoff;
        A.pts = T.npts ? T.pts : nullptr;
        A.rowptr = T.rowptr;
        A.rec = T.rec;
        A.wt = T.wt;
        A.tile_ptr = T.tile_ptr;
        A.grad = grads + s * G;
        float* ring_s = dir ? ring + s * K * (size_t)ring_len : nullptr;
        adj[s] = AdjShot{A, nu + 3 * G * s, seg + (K + 2) * G * s, g[s], ring_s,
                         (int)P[s].num_receivers};
        rec[s] = StepShot{Xs.shot_quiet, seg + (K + 2) * G * s, ring_s};
    }
    AdjShot* dadj = mem.get<AdjShot>(ns);
    StepShot* drec = mem.get<StepShot>(ns);
    GR_CUDA(cudaMemcpyAsync(dadj, adj.data(), ns * sizeof(AdjShot), cudaMemcpyHostToDevice, st));
    GR_CUDA(cudaMemcpyAsync(drec, rec.data(), ns * sizeof(StepShot), cudaMemcpyHostToDevice, st));
    const int tiles = X[0].shot.ntiles;
    const size_t b = X[0].begin, e = X[0].end;
    const size_t nck = checkpoint_count(steps, interval);
    for (size_t j = nck; j-- > 0;) {
        const size_t n0 = b + j * interval;
        const size_t n1 = std::min(n0 + interval - 1, e);
        for (size_t s = 0; s < ns; s++)
            GR_CUDA(cudaMemcpyAsync(seg + (K + 2) * G * s, ck[s] + 2 * j * G, 2 * bytes,
                                    cudaMemcpyDeviceToDevice, st));
        for (size_t n = n0; n <= n1; n++) {
            const size_t k = n - n0;
            step2d_launch_shots(drec, (int)ns, tiles, r, X[0].vd, (long long)G, (int)(k + 2),
                                (int)(k + 1), (int)k, (long long)n,
                                (long long)(k * (size_t)ring_len), false, st);
            GR_LAUNCHED("stencil2d_step_shots");
        }
        for (size_t m = n1 + 1; m >= n0 + 1; m--) {
            if (m == e + 1) continue;  // nu^(e+1) = 0: no record reads u^(e+1)
            const size_t k = m - n0;
            adjoint_launch_shots(dadj, (int)ns, tiles, r, X[0].vd, (long long)G, (int)(m % 3),
                                 (int)((m + 1) % 3), (int)((m + 2) % 3), (int)k, (long long)m,
                                 (long long)((m - 1 - n0) * (size_t)ring_len), st);
            GR_LAUNCHED("adjoint2d_step_shots");
        }
    }
    sum_grids<<<1024, 256, 0, st>>>(grad, grads, (int)ns, (long long)G);
    GR_LAUNCHED("sum_grids");
    // the tables must outlive their copies
    GR_CUDA(cudaStreamSynchronize(st));
}

template <typename F>
static int guarded(F&& f) {
    try {
        f();
        return SIMWAVE_OK;
    } catch (const Refusal& r) {
        ::sw::record_error(r.message);
        return r.code;
    } catch (const std::exception& ex) {
        ::sw::record_error(ex.what());
        return SIMWAVE_E_CUDA;
    }
}

}  // namespace grad
}  // namespace sw

extern "C" int simwave_gradient_checkpoints(const simwave_problem* problem, size_t interval,
                                            size_t* grids) {
    return sw::grad::guarded([&] {
        if (!problem || !grids || interval < 1 ||
            problem->end_timestep < problem->begin_timestep)
            sw::grad::refuse(SIMWAVE_E_ARGUMENT, "invalid checkpoint request");
        const size_t steps = problem->end_timestep - problem->begin_timestep + 1;
        *grids = 2 * sw::grad::checkpoint_count(steps, interval);
    });
}

extern "C" int simwave_gradient_forward(const simwave_problem* problem, size_t interval,
                                        void* checkpoints, void* stream) {
    return sw::grad::guarded([&] {
        sw::grad::forward_pass(problem, interval, static_cast<float*>(checkpoints),
                               static_cast<cudaStream_t>(stream));
    });
}

extern "C" int simwave_gradient_backward(const simwave_problem* problem, size_t interval,
                                         const void* checkpoints, const void* grad_receivers,
                                         void* grad_velocity, void* stream) {
    return sw::grad::guarded([&] {
        sw::grad::reverse_pass(problem, interval, static_cast<const float*>(checkpoints),
                               static_cast<const float*>(grad_receivers),
                               static_cast<float*>(grad_velocity),
                               static_cast<cudaStream_t>(stream));
    });
}

extern "C" int simwave_gradient_forward_shots(const simwave_problem* problems, size_t nshots,
                                              size_t interval, void* const* checkpoints,
                                              void* stream) {
    return sw::grad::guarded([&] {
        sw::grad::forward_pass_shots(problems, nshots, interval,
                                     reinterpret_cast<float* const*>(checkpoints),
                                     static_cast<cudaStream_t>(stream));
    });
}

extern "C" int simwave_gradient_backward_shots(const simwave_problem* problems, size_t nshots,
                                               size_t interval, const void* const* checkpoints,
                                               const void* const* grad_receivers,
                                               void* grad_velocity, void* stream) {
    return sw::grad::guarded([&] {
        sw::grad::reverse_pass_shots(problems, nshots, interval,
                                     reinterpret_cast<const float* const*>(checkpoints),
                                     reinterpret_cast<const float* const*>(grad_receivers),
                                     static_cast<float*>(grad_velocity),
                                     static_cast<cudaStream_t>(stream));
    });
}
