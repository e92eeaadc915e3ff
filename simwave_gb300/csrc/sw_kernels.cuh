// sw_kernels.cuh -- per-step kernels of the forward operator.
//
// One time step n of simwave's forward loop (reference C path,
// constant_density/2d/wave.c:108-516, variable_density/3d/wave.c:108-640):
//   1. stencil     u_next = (2 u_cur - N u_prev + dt^2 v^2 L(u_cur)) / D
//                  D = 1 + damp dt v^2 / 2, N = 1 - damp dt v^2 / 2
//   2. sources     u_next += dt^2 v^2 kws w[n-1] / D over each KWS window
//   3. boundaries  Dirichlet zero on the first/last interior index, Neumann
//                  mirror into the halo; y, x, z edges in 3D, x, z in 2D
//   4. receivers   rec[n-1] = sum kws u_cur over each KWS window
// L is the order-2r Laplacian; with variable density the cross term
// sum_axes (D1 u)(D1 rho) / (4 h^2 rho) is subtracted (D1 = first-derivative
// half weights), exactly as the reference writes it
// (variable_density/2d/wave.c:186-189).
#pragma once

#include "sw_common.cuh"

namespace sw {

// Damped leapfrog update of one point given the spatial operator `lap`
// (already divided by h^2). Same algebra as the reference
// (constant_density/2d/wave.c:170-178): value = lap * dt^2 v^2 / D,
// u_next = 2/D u_cur - N/D u_prev + value.
template <typename T>
__device__ __forceinline__ T leapfrog(T lap, T vel, T damp, T ucur, T uprev,
                                      T dt, T dt2) {
    T v2 = vel * vel;
    T q = damp * dt * v2 * T(0.5);
    T rden = T(1) / (T(1) + q);
    return (T(2) * ucur - (T(1) - q) * uprev + dt2 * v2 * lap) * rden;
}

// ---- generic stencil: one thread per interior point, runtime radius ------
// Grid: x -> fastest axis, y -> middle axis, z -> slowest axis (3D).
// `un` and `up` may be the same slot: with a saving stride > 1 the reference
// writes level n+1 over level n-1 (constant_density/2d/wave.c:509-513); each
// point reads its own previous value before writing it.
template <typename T, int DIM, bool VD>
__global__ void __launch_bounds__(256)
stencil_generic(T* un, const T* __restrict__ uc,
                const T* up, const T* __restrict__ vel,
                const T* __restrict__ den, const T* __restrict__ damp,
                Layout L, Weights<T> W, T dt, T dt2) {
    const int r = L.r;
    const long long f = r + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long m = r + (long long)blockIdx.y * blockDim.y + threadIdx.y;
    const long long s = DIM == 3 ? r + (long long)blockIdx.z : 0;
    if (f >= L.nfast() - r || m >= L.nmid() - r) return;
    const long long p = L.at(s, m, f);
    // axes: fastest (stride 1), middle (pitch), slowest (plane, 3D only)
    const int af = DIM == 3 ? 2 : 1;
    const int am = DIM == 3 ? 1 : 0;
    const long long sm = L.pitch, ss = L.plane;
    const T u0 = uc[p];
    T lap_f = W.c2[0] * u0, lap_m = W.c2[0] * u0, lap_s = W.c2[0] * u0;
    T gu_f = 0, gu_m = 0, gu_s = 0, gr_f = 0, gr_m = 0, gr_s = 0;
    for (int k = 1; k <= r; k++) {
        const T fp = uc[p + k], fm = uc[p - k];
        const T mp = uc[p + k * sm], mm = uc[p - k * sm];
        lap_f += W.c2[k] * (fp + fm);
        lap_m += W.c2[k] * (mp + mm);
        if (VD) {
            gu_f += W.c1[k] * (fp - fm);
            gu_m += W.c1[k] * (mp - mm);
            gr_f += W.c1[k] * (den[p + k] - den[p - k]);
            gr_m += W.c1[k] * (den[p + k * sm] - den[p - k * sm]);
        }
        if (DIM == 3) {
            const T sp = uc[p + k * ss], sq = uc[p - k * ss];
            lap_s += W.c2[k] * (sp + sq);
            if (VD) {
                gu_s += W.c1[k] * (sp - sq);
                gr_s += W.c1[k] * (den[p + k * ss] - den[p - k * ss]);
            }
        }
    }
    // axis order of the reference's sum: y, x, z (3D); x, z (2D)
    T lap = lap_f * W.ih2[af] + lap_m * W.ih2[am];
    if (DIM == 3) lap += lap_s * W.ih2[0];
    if (VD) {
        T cross = gu_f * gr_f * W.s1[af] + gu_m * gr_m * W.s1[am];
        if (DIM == 3) cross += gu_s * gr_s * W.s1[0];
        lap -= cross / den[p];
    }
    un[p] = leapfrog(lap, vel[p], damp[p], u0, up[p], dt, dt2);
}

// ---- window helpers --------------------------------------------------------
// Decompose flat index t of a window into its (z, x[, y]) offsets.
template <int DIM>
__device__ __forceinline__ void window_point(const size_t* b, long long t,
                                             long long& iz, long long& ix,
                                             long long& iy) {
    const long long lx = (long long)(b[3] - b[2] + 1);
    const long long ly = DIM == 3 ? (long long)(b[5] - b[4] + 1) : 1;
    iz = t / (lx * ly);
    const long long rem = t - iz * lx * ly;
    ix = rem / ly;
    iy = rem - ix * ly;
}

template <int DIM>
__device__ __forceinline__ long long window_size(const size_t* b) {
    long long n = (long long)(b[1] - b[0] + 1) * (long long)(b[3] - b[2] + 1);
    if (DIM == 3) n *= (long long)(b[5] - b[4] + 1);
    return n;
}

template <typename T, int DIM>
__device__ __forceinline__ T window_weight(const size_t* b, const T* v,
                                           long long iz, long long ix,
                                           long long iy) {
    const long long lz = (long long)(b[1] - b[0] + 1);
    const long long lx = (long long)(b[3] - b[2] + 1);
    T w = v[iz] * v[lz + ix];
    if (DIM == 3) w = w * v[lz + lx + iy];
    return w;
}

template <int DIM>
__device__ __forceinline__ long long window_offset(const Layout& L,
                                                   const size_t* b,
                                                   long long iz, long long ix,
                                                   long long iy) {
    if (DIM == 3) return L.at3(b[0] + iz, b[2] + ix, b[4] + iy);
    return L.at2(b[0] + iz, b[2] + ix);
}

// ---- sources: KWS injection of one source window ---------------------------
// (constant_density/2d/wave.c:182-271): u_next += dt^2 v^2 kws w / D over the
// window; threads t0, t0 + tstride, ... of the window. Overlapping windows of
// different sources add through atomics, like the reference's `omp atomic`.
template <typename T, int DIM>
__device__ __forceinline__ void inject_window(T* un, const T* vel, const T* damp,
                                              const Layout& L, const size_t* b,
                                              const T* v, T w, T dt, T dt2, int t0,
                                              int tstride) {
    const long long total = window_size<DIM>(b);
    for (long long t = t0; t < total; t += tstride) {
        long long iz, ix, iy;
        window_point<DIM>(b, t, iz, ix, iy);
        const T kws = window_weight<T, DIM>(b, v, iz, ix, iy);
        const long long p = window_offset<DIM>(L, b, iz, ix, iy);
        const T vv = vel[p] * vel[p];
        const T d = T(1) + damp[p] * dt * vv * T(0.5);
        atomicAdd(un + p, dt2 * vv * kws * w / d);
    }
}

// Wavelet sample of source s at step n (wave.c:199-205).
template <typename T>
__device__ __forceinline__ T wavelet_at(const T* wavelet, size_t count, size_t n,
                                        size_t nsrc, size_t s) {
    return count > 1 ? wavelet[(n - 1) * nsrc + s] : wavelet[n - 1];
}

// One block per source, threads over its window.
template <typename T, int DIM>
__global__ void inject_sources(T* __restrict__ un, const T* __restrict__ vel,
                               const T* __restrict__ damp, Layout L,
                               Windows<T> src, const T* __restrict__ wavelet,
                               size_t wavelet_count, size_t n, T dt, T dt2) {
    const size_t s = blockIdx.x;
    if (s >= src.count) return;
    const T w = wavelet_at(wavelet, wavelet_count, n, src.count, s);
    if (w == T(0)) return;
    inject_window<T, DIM>(un, vel, damp, L, src.interval + s * 2 * DIM,
                          src.values + src.offsets[s], w, dt, dt2, threadIdx.x,
                          blockDim.x);
}

// ---- receivers: KWS gather of one receiver window by one warp --------------
// (constant_density/2d/wave.c:395-464); reads the current level. Eight lanes
// run along the window's contiguous axis (y in 3D, x in 2D) and the four
// lane groups take alternate rows, so one load instruction touches four
// 32-byte window rows; the lane sums are reduced with shuffles. Returns the
// sum in every lane.
template <typename T, int DIM>
__device__ __forceinline__ T gather_window(const T* uc, const Layout& L, const size_t* b,
                                           const T* v, int lane) {
    const int lz = (int)(b[1] - b[0] + 1), lx = (int)(b[3] - b[2] + 1);
    const int nf = DIM == 3 ? (int)(b[5] - b[4] + 1) : lx;  // contiguous extent
    const int rows = DIM == 3 ? lz * lx : lz;
    const T* vf = DIM == 3 ? v + lz + lx : v + lz;          // contiguous-axis weights
    const int sub = lane & 7, grp = lane >> 3;
    T sum = 0;
    for (int f = sub; f - sub < nf; f += 8) {
        if (f >= nf) continue;
        const T wf = vf[f];
        for (int row = grp; row < rows; row += 4) {
            if (DIM == 3) {
                const int iz = row / lx, ix = row - iz * lx;
                const T wzx = v[iz] * v[lz + ix];
                sum += uc[L.at3(b[0] + iz, b[2] + ix, b[4] + f)] * (wzx * wf);
            } else {
                sum += uc[L.at2(b[0] + row, b[2] + f)] * (v[row] * wf);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    return sum;
}

// One warp per receiver.
template <typename T, int DIM>
__global__ void record_receivers(T* __restrict__ rec_row,
                                 const T* __restrict__ uc, Layout L,
                                 Windows<T> rec) {
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= (long long)rec.count) return;
    const T sum = gather_window<T, DIM>(uc, L, rec.interval + warp * 2 * DIM,
                                        rec.values + rec.offsets[warp], lane);
    if (lane == 0) rec_row[warp] = sum;
}

// ---- boundary conditions: one line normal to `axis` --------------------------
// Applies the before edge then the after edge of one axis, like one
// iteration of the reference's BC loops (constant_density/2d/wave.c:274-393,
// constant_density/3d/wave.c:299-481). Phases (axes) are separate launches
// so that their order (y, x, z in 3D; x, z in 2D) is kept.
template <typename T>
__device__ __forceinline__ void apply_edge(T* u, long long first,
                                           long long step, int r, int type,
                                           int dir) {
    if (type == 1) u[first] = T(0);
    if (type == 2) {
        for (int q = 1; q <= r; q++) {
            if (dir < 0) u[first - q * step] = u[first + q * step];
            else u[first + q * step] = u[first - q * step];
        }
    }
}

// Number of lines of the phase normal to `axis`.
__host__ __device__ __forceinline__ long long boundary_lines(const Layout& L, int axis) {
    const int a1 = axis == 0 ? 1 : 0;
    const int a2 = L.dim == 3 ? (axis == 2 ? 1 : 2) : -1;
    return (L.extent(a1) - 2 * L.r) * (a2 >= 0 ? L.extent(a2) - 2 * L.r : 1);
}

// Line t of the phase normal to `axis`.
template <typename T>
__device__ __forceinline__ void boundary_line(T* u, const Layout& L, int axis, int before,
                                              int after, long long t) {
    const int r = L.r;
    const int a1 = axis == 0 ? 1 : 0;  // the two other axes, increasing
    const int a2 = L.dim == 3 ? (axis == 2 ? 1 : 2) : -1;
    const long long n2 = a2 >= 0 ? L.extent(a2) - 2 * r : 1;
    long long idx[3] = {0, 0, 0};
    idx[a1] = r + t / n2;
    if (a2 >= 0) idx[a2] = r + t % n2;
    const long long step = L.stride(axis);
    idx[axis] = r;
    long long first = L.dim == 3 ? L.at3(idx[0], idx[1], idx[2]) : L.at2(idx[0], idx[1]);
    apply_edge(u, first, step, r, before, -1);
    idx[axis] = L.extent(axis) - r - 1;
    first = L.dim == 3 ? L.at3(idx[0], idx[1], idx[2]) : L.at2(idx[0], idx[1]);
    apply_edge(u, first, step, r, after, +1);
}

template <typename T>
__global__ void boundary_phase(T* __restrict__ u, Layout L, int axis,
                               int before, int after) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= boundary_lines(L, axis)) return;
    boundary_line(u, L, axis, before, after, t);
}

// ---- layout conversion: dense rows <-> pitched rows -----------------------
// `rows` rows of `width` elements; dense row r at src + r * width, pitched
// row r at dst + r * pitch + lead (to_pitched), or the reverse.
template <typename T>
__global__ void __launch_bounds__(128, 16)
repack_rows(T* __restrict__ dst, const T* __restrict__ src, long long rows, long long width,
            long long pitch, long long lead, bool to_pitched) {
    const long long ss = to_pitched ? width : pitch, so = to_pitched ? 0 : lead;
    const long long ds = to_pitched ? pitch : width, dof = to_pitched ? lead : 0;
    // 16-byte moves where every row start is 16-byte aligned
    constexpr int V = 16 / sizeof(T);
    const bool vec = width % V == 0 && pitch % V == 0 && lead % V == 0 &&
                     ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    const int w = vec ? (int)(width / V) : (int)width;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const T* s = src + r * ss + so;
        T* d = dst + r * ds + dof;
        if (vec) {
            for (int c = threadIdx.x; c < w; c += blockDim.x)
                reinterpret_cast<float4*>(d)[c] = reinterpret_cast<const float4*>(s)[c];
        } else {
            for (int c = threadIdx.x; c < w; c += blockDim.x) d[c] = s[c];
        }
    }
}

}  // namespace sw
