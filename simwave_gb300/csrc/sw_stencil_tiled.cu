// sw_stencil_tiled.cu -- tiled 3D stencil for float32 on sm_103a.
//
// One CTA owns a 32 (y) x TX (x) column of the interior and streams along z
// over a chunk of planes. Per output plane z:
//   * the plane's u_cur tile and, with variable density, rho tile, each with
//     an R-wide x/y halo, are staged in shared memory by TMA
//     (cp.async.bulk.tensor, mbarrier completion), three planes deep, so the
//     copy of plane z+2 overlaps the arithmetic of plane z;
//   * the z-derivatives come from per-thread register queues holding planes
//     z-R .. z+R of the thread's own points; the queue head (plane z+R+1) is
//     fetched with one coalesced load per point a step ahead;
//   * each thread computes NX consecutive x points of one y column, so the
//     x-neighbour loads from shared memory are shared by its NX points;
//   * u_prev, velocity and damping are read once per point (damping only
//     outside the box where the mask is known to be zero), u_next written once.
// DRAM traffic per point update is therefore u_cur, u_prev, velocity,
// (rho), u_next and, in the damping layer, damp: 16/20 B (+4 B in the layer).
//
// Every mbarrier wait is bounded; on expiry the CTA records an error code,
// drains its outstanding copies (also bounded) and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "simwave_gb300.h"
#include "sw_pairs.cuh"
#include "sw_tiled.h"
#include "sw_tma.cuh"

namespace sw {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;
constexpr int kStages = 3;              // planes in flight per field

template <int R>
struct Tile {
    static constexpr int NX = R <= 4 ? 4 : (R <= 7 ? 2 : 1);  // x points per thread
    static constexpr int TX = kWarps * NX;                    // x extent of a tile
    static constexpr int HY = round4(R);                      // y halo (16 B aligned)
    static constexpr int W = 32 + 2 * HY;                     // tile row length
    static constexpr int H = TX + 2 * R;                      // tile rows
    static constexpr int ELEMS = W * H;
    static constexpr int BYTES = ELEMS * 4;                   // one TMA box
    static constexpr int STRIDE = (ELEMS + 31) & ~31;         // 128 B aligned slots
};

// ---- per-point coefficients --------------------------------------------------
//
// The tiled kernels read two time-invariant per-point coefficients instead of
// velocity and damping, formed once per run exactly as the reference forms
// them every step (constant_density/2d/wave.c:170-178):
//   Q = damp * dt / (2 * slowness),  slowness = 1 / v^2
//   C = (dt^2 / slowness) / (1 + Q)
// so that u_next = 2/D u_cur - N/D u_prev + C L(u_cur), D = 1 + Q, N = 1 - Q.
// Q is zero wherever the damping mask is, so its loads are skipped there.

__global__ void form_coefficients(const float* __restrict__ vel,
                                  const float* __restrict__ damp, float* __restrict__ C,
                                  float* __restrict__ Q, long long n, float dt) {
    const float dt2 = dt * dt;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = vel[i];
        const float slowness = __frcp_rn(v * v);
        const float q = __fdiv_rn(damp[i] * dt, 2.f * slowness);
        const float den = 1.f + q;
        C[i] = __fdiv_rn(__fdiv_rn(dt2, slowness), den);
        Q[i] = q;
    }
}

// gz = s1_z * sum_k c1_k (rho(z+k) - rho(z-k)) over the interior (3D): the
// density's z term of the variable-density cross term, time-invariant.
__global__ void form_density_z(const float* __restrict__ den, float* __restrict__ gz, Layout L,
                               Weights<float> W) {
    const int r = L.r;
    const long long ny = L.ny - 2 * r, nx = L.nx - 2 * r, nz = L.nz - 2 * r;
    const long long total = nz * nx * ny;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long k = r + t % ny, j = r + (t / ny) % nx, i = r + t / (ny * nx);
        const long long p = L.at3(i, j, k);
        float f = W.c1[1] * (den[p + L.plane] - den[p - L.plane]);
        for (int q = 2; q <= r; q++)
            f = fmaf(W.c1[q], den[p + q * L.plane] - den[p - q * L.plane], f);
        gz[p] = f * W.s1[0];
    }
}

// u_next from the spatial operator, C, Q, u_cur and u_prev.
__device__ __forceinline__ float leapfrog_cq(float lap, float c, float q, float ucur,
                                             float uprev) {
    const float a = fmaf(-(1.f - q), uprev, 2.f * ucur);
    const float b = q == 0.f ? a : a * __fdividef(1.f, 1.f + q);
    return fmaf(lap, c, b);
}

// ---- the kernel ------------------------------------------------------------

struct ZeroBox {  // interior box where the damping mask is zero
    int z0, z1, x0, x1, y0, y1;
};

template <int R, bool VD>
__global__ void __launch_bounds__(kThreads, 2)
stencil3d_tiled(const __grid_constant__ CUtensorMap map_u,
                const __grid_constant__ CUtensorMap map_rho,
                float* un, const float* __restrict__ uc,
                const float* up, const float* __restrict__ vel,
                const float* __restrict__ den, const float* __restrict__ damp,
                Layout L, Weights<float> Wt, float dt, float dt2, int slot_cur,
                int zchunk, ZeroBox zb, int* __restrict__ err) {
    using TL = Tile<R>;
    constexpr int NX = TL::NX, TX = TL::TX, HY = TL::HY, TW = TL::W;
    constexpr int NF = VD ? 2 : 1;
    // dynamic shared memory only (no static shared data), so the region
    // starts at the base of the CTA's shared window: 128-byte aligned TMA
    // destinations, then the mbarriers and the abort flag
    float* tiles = reinterpret_cast<float*>(sw_dyn_smem);  // [NF][kStages][STRIDE]
    unsigned long long* bars =
        reinterpret_cast<unsigned long long*>(tiles + NF * kStages * TL::STRIDE);
    int& s_abort = *reinterpret_cast<int*>(bars + kStages);
    if (*(volatile int*)err) return;  // an earlier launch already failed
    if (smem_addr(tiles) & 127) {    // layout assumption broken: refuse
        if (threadIdx.x == 0) atomicExch(err, SIMWAVE_E_ARGUMENT);
        return;
    }

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int y = R + blockIdx.x * 32 + lane;             // interior y of this lane
    const int xb = R + blockIdx.y * TX;                    // first x of the tile
    const int x0 = xb + warp * NX;                         // first x of this thread
    const int zbeg = R + blockIdx.z * zchunk;
    const int zend = min(zbeg + zchunk, (int)L.nz - R);
    if (zbeg >= zend) return;
    const bool yok = y < (int)L.ny - R;

    // TMA box origin: columns of the pitched row, rows of x, plane, slot
    const int col0 = (int)L.lead + R + blockIdx.x * 32 - HY;
    const int row0 = xb - R;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();

    auto issue = [&](int plane, int stage) {
        mbar_expect_tx(&bars[stage], NF * TL::BYTES);
        tma_load_4d(tiles + stage * TL::STRIDE, &map_u, &bars[stage], col0, row0, plane,
                    slot_cur);
        if (VD)
            tma_load_4d(tiles + (kStages + stage) * TL::STRIDE, &map_rho, &bars[stage], col0,
                        row0, plane, 0);
    };
    int issued = 0;  // planes zbeg .. zbeg + issued - 1 requested (thread 0)
    if (threadIdx.x == 0)
        for (; issued < kStages && zbeg + issued < zend; issued++) issue(zbeg + issued, issued);

    // register queues: q[i][j] = field at plane z - R + j of point (x0 + i, y)
    float qu[NX][2 * R + 1];
    float qr[VD ? NX : 1][VD ? 2 * R + 1 : 1];
    bool xok[NX];
    int off[NX];  // element offset of (x0 + i, y) within a plane
#pragma unroll
    for (int i = 0; i < NX; i++) {
        xok[i] = yok && (x0 + i < (int)L.nx - R);
        off[i] = (x0 + i) * (int)L.pitch + (int)L.lead + y;
    }
#pragma unroll
    for (int j = 0; j < 2 * R; j++) {
        const long long pz = (long long)(zbeg - R + j) * L.plane;
#pragma unroll
        for (int i = 0; i < NX; i++) {
            qu[i][j] = xok[i] ? __ldg(uc + pz + off[i]) : 0.f;
            if (VD) qr[i][j] = xok[i] ? __ldg(den + pz + off[i]) : 0.f;
        }
    }
    float hu[NX], hr[NX];  // queue heads (plane z + R)
    {
        const long long pz = (long long)(zbeg + R) * L.plane;
#pragma unroll
        for (int i = 0; i < NX; i++) {
            hu[i] = xok[i] ? __ldg(uc + pz + off[i]) : 0.f;
            hr[i] = (VD && xok[i]) ? __ldg(den + pz + off[i]) : 0.f;
        }
    }

    // per-point operands fetched one plane ahead; u_prev with a plain load:
    // it may be the slot this kernel writes
    float nprev[NX], nvel[NX], ndamp[NX];
    auto fetch = [&](int zz) {
        const long long p = (long long)zz * L.plane;
        const bool zin = zz >= zb.z0 && zz < zb.z1 && y >= zb.y0 && y < zb.y1;
#pragma unroll
        for (int i = 0; i < NX; i++) {
            nprev[i] = xok[i] ? up[p + off[i]] : 0.f;
            nvel[i] = xok[i] ? __ldg(vel + p + off[i]) : 0.f;
            const bool inbox = zin && x0 + i >= zb.x0 && x0 + i < zb.x1;
            ndamp[i] = (xok[i] && !inbox) ? __ldg(damp + p + off[i]) : 0.f;
        }
    };
    fetch(zbeg);
    int aborted_at = -1;
    for (int z = zbeg; z < zend; z++) {
        const int it = z - zbeg;
        const int stage = it % kStages;
#pragma unroll
        for (int i = 0; i < NX; i++) {
            qu[i][2 * R] = hu[i];
            if (VD) qr[i][2 * R] = hr[i];
        }
        if (z + 1 < zend) {  // next queue heads
            const long long pz = (long long)(z + 1 + R) * L.plane;
#pragma unroll
            for (int i = 0; i < NX; i++) {
                hu[i] = xok[i] ? __ldg(uc + pz + off[i]) : 0.f;
                if (VD) hr[i] = xok[i] ? __ldg(den + pz + off[i]) : 0.f;
            }
        }
        // per-point operands of this plane (fetched one plane ahead)
        const long long pz = (long long)z * L.plane;
        float vprev[NX], vvel[NX], vdamp[NX];
#pragma unroll
        for (int i = 0; i < NX; i++) {
            vprev[i] = nprev[i];
            vvel[i] = nvel[i];
            vdamp[i] = ndamp[i];
        }
        if (z + 1 < zend) fetch(z + 1);

        const bool ok = mbar_wait(&bars[stage], (unsigned)((it / kStages) & 1));
        if (!ok) s_abort = 1;
        if (ok) {
        const float* tu = tiles + stage * TL::STRIDE;
        const float* tr = tiles + (kStages + stage) * TL::STRIDE;
        const int cy = lane + HY;  // tile column of this lane

        // x-direction neighbours: rows x0 - R .. x0 + NX - 1 + R of this column
        float colu[NX + 2 * R], colr[VD ? NX + 2 * R : 1];
#pragma unroll
        for (int j = 0; j < NX + 2 * R; j++) {
            colu[j] = tu[(warp * NX + j) * TW + cy];
            if (VD) colr[j] = tr[(warp * NX + j) * TW + cy];
        }

#pragma unroll
        for (int i = 0; i < NX; i++) {
            const float* rowu = tu + (warp * NX + i + R) * TW + cy;
            const float* rowr = tr + (warp * NX + i + R) * TW + cy;
            const float u0 = qu[i][R];
            float ly = Wt.c2[0] * u0, lx = Wt.c2[0] * u0, lz = Wt.c2[0] * u0;
            float gy = 0.f, gx = 0.f, gz = 0.f, ry = 0.f, rx = 0.f, rz = 0.f;
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const float yp = rowu[k], ym = rowu[-k];
                const float xp = colu[i + R + k], xm = colu[i + R - k];
                const float zp = qu[i][R + k], zm = qu[i][R - k];
                ly = fmaf(Wt.c2[k], yp + ym, ly);
                lx = fmaf(Wt.c2[k], xp + xm, lx);
                lz = fmaf(Wt.c2[k], zp + zm, lz);
                if (VD) {
                    gy = fmaf(Wt.c1[k], yp - ym, gy);
                    gx = fmaf(Wt.c1[k], xp - xm, gx);
                    gz = fmaf(Wt.c1[k], zp - zm, gz);
                    ry = fmaf(Wt.c1[k], rowr[k] - rowr[-k], ry);
                    rx = fmaf(Wt.c1[k], colr[i + R + k] - colr[i + R - k], rx);
                    rz = fmaf(Wt.c1[k], qr[i][R + k] - qr[i][R - k], rz);
                }
            }
            float lap = ly * Wt.ih2[2] + lx * Wt.ih2[1];
            lap = fmaf(lz, Wt.ih2[0], lap);
            if (VD) {
                float cross = gy * ry * Wt.s1[2] + gx * rx * Wt.s1[1];
                cross = fmaf(gz * rz, Wt.s1[0], cross);
                lap -= __fdividef(cross, qr[i][R]);
            }
            const float unew = leapfrog_cq(lap, vvel[i], vdamp[i], u0, vprev[i]);
            if (xok[i]) un[pz + off[i]] = unew;
        }
        }  // ok

        __syncthreads();  // the stage is free again; abort is uniform here
        if (s_abort) {
            aborted_at = it;
            break;
        }
        if (threadIdx.x == 0 && z + kStages < zend) {
            issue(z + kStages, stage);
            issued++;
        }
#pragma unroll
        for (int i = 0; i < NX; i++) {
#pragma unroll
            for (int j = 0; j < 2 * R; j++) {
                qu[i][j] = qu[i][j + 1];
                if (VD) qr[i][j] = qr[i][j + 1];
            }
        }
    }
    if (aborted_at >= 0 && threadIdx.x == 0) {
        atomicExch(err, SIMWAVE_E_TIMEOUT);
        // drain the copies still in flight into this CTA's shared memory
        for (int p = aborted_at; p < issued; p++)
            mbar_wait(&bars[p % kStages], (unsigned)((p / kStages) & 1));
    }
}


// ---- vectorised kernel: 4 consecutive y points per thread (orders <= 8) ----
//
// Warp w of the CTA owns x row R + 8*blockIdx.y + w; lane l owns y points
// y0 .. y0+3, y0 = R + 128*blockIdx.x + 4l. Global traffic is float4 per
// thread; the y window (4 + 2*HY values) and the x neighbours come from the
// TMA tile as 16-byte shared loads; z neighbours from float4 register queues.

__device__ __forceinline__ float4 f4(float a) { return make_float4(a, a, a, a); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 sub4(float4 a, float4 b) {
    return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 fma4(float c, float4 a, float4 acc) {
    return make_float4(fmaf(c, a.x, acc.x), fmaf(c, a.y, acc.y), fmaf(c, a.z, acc.z),
                       fmaf(c, a.w, acc.w));
}
__device__ __forceinline__ float4 mul4(float c, float4 a) {
    return make_float4(c * a.x, c * a.y, c * a.z, c * a.w);
}
__device__ __forceinline__ float comp(const float4& a, int v) {
    return v == 0 ? a.x : (v == 1 ? a.y : (v == 2 ? a.z : a.w));
}
__device__ __forceinline__ void set_comp(float4& a, int v, float x) {
    if (v == 0) a.x = x; else if (v == 1) a.y = x; else if (v == 2) a.z = x; else a.w = x;
}

// float4 load of points y0..y0+3 of a row; partial chunks load what exists
// in memory (the row is never the last of its allocation) and are masked at
// the store.
__device__ __forceinline__ float4 ld4(const float* p, bool any) {
    return any ? __ldg(reinterpret_cast<const float4*>(p)) : f4(0.f);
}

template <int R>
struct VecTile {
    static constexpr int HY = round4(R);
    static constexpr int TW = 128 + 2 * HY;  // floats per tile row
    static constexpr int TH = kWarps + 2 * R;
    static constexpr int ELEMS = TW * TH;
    static constexpr int BYTES = ELEMS * 4;
    static constexpr int STRIDE = (ELEMS + 31) & ~31;
    static constexpr int NC = (2 * HY) / 4 + 1;  // float4 chunks of a y window
};

// QS: keep the density z-queue in shared memory (a per-thread circular
// buffer of 2R+1 float4, read only by its owner) instead of registers.
// ROT: unroll the plane loop by the queue length 2R+1 so that queue slots are
// compile-time constants (no register moves, no index arithmetic).
// Queue slot of plane p: (p - zbeg + R) mod (2R+1).
template <int R, bool VD, int MINB, bool QS, bool ROT>
__global__ void __launch_bounds__(kThreads, MINB)
stencil3d_vec4(const __grid_constant__ CUtensorMap map_u,
               const __grid_constant__ CUtensorMap map_rho, float* un,
               const float* __restrict__ uc, const float* up,
               const float* __restrict__ coefC, const float* __restrict__ den,
               const float* __restrict__ coefQ, Layout L, Weights<float> Wt,
               int slot_cur, int zchunk, ZeroBox zb, int* __restrict__ err) {
    using VT = VecTile<R>;
    constexpr int HY = VT::HY, TW = VT::TW, NC = VT::NC;
    constexpr int NF = VD ? 2 : 1;
    constexpr int QN = 2 * R + 1;
    constexpr bool RQ = VD && !QS;  // density queue in registers
    // dynamic shared memory only: TMA tiles (128-byte aligned), the shared
    // density queue, then the mbarriers and the abort flag
    float* tiles = reinterpret_cast<float*>(sw_dyn_smem);
    float4* sq_base = reinterpret_cast<float4*>(tiles + NF * kStages * VT::STRIDE);
    unsigned long long* bars =
        reinterpret_cast<unsigned long long*>(sq_base + (VD && QS ? QN * kThreads : 0));
    int& s_abort = *reinterpret_cast<int*>(bars + kStages);
    if (*(volatile int*)err) return;
    if (smem_addr(tiles) & 127) {
        if (threadIdx.x == 0) atomicExch(err, SIMWAVE_E_ARGUMENT);
        return;
    }

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int yb = R + blockIdx.x * 128;
    const int y0 = yb + 4 * lane;
    const int x = R + blockIdx.y * kWarps + warp;
    const int zbeg = R + blockIdx.z * zchunk;
    const int zend = min(zbeg + zchunk, (int)L.nz - R);
    if (zbeg >= zend) return;
    const int ylim = (int)L.ny - R;
    const bool any = x < (int)L.nx - R && y0 < ylim;
    const bool full = any && y0 + 3 < ylim;
    const int off = x * (int)L.pitch + (int)L.lead + y0;
    const int col0 = (int)L.lead + yb - HY;
    const int row0 = blockIdx.y * kWarps;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();
    auto issue = [&](int plane, int stage) {
        mbar_expect_tx(&bars[stage], NF * VT::BYTES);
        tma_load_4d(tiles + stage * VT::STRIDE, &map_u, &bars[stage], col0, row0, plane,
                    slot_cur);
        if (VD)
            tma_load_4d(tiles + (kStages + stage) * VT::STRIDE, &map_rho, &bars[stage], col0,
                        row0, plane, 0);
    };
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < kStages && zbeg + issued < zend; issued++) issue(zbeg + issued, issued);

    // queues hold planes z-R .. z+R; slot of plane p = (p - zbeg + R) mod QN
    float4 qu[QN];
    float4 qr[RQ ? QN : 1];
    float4* sq = sq_base + threadIdx.x;
#pragma unroll
    for (int j = 0; j < QN; j++) {
        const long long pz = (long long)(zbeg - R + j) * L.plane + off;
        qu[j] = ld4(uc + pz, any);
        if (RQ) qr[j] = ld4(den + pz, any);
        if (VD && QS) sq[j * kThreads] = ld4(den + pz, any);
    }
    // per-point operands of the next plane; u_prev with a plain load: it may
    // be the slot this kernel writes (each point reads its own previous value
    // before writing it)
    const bool xybox = x >= zb.x0 && x < zb.x1 && y0 >= zb.y0 && y0 + 3 < zb.y1;
    float4 nprev, ncoef, nq;
    auto fetch = [&](int zz) {
        const long long p = (long long)zz * L.plane + off;
        nprev = any ? *reinterpret_cast<const float4*>(up + p) : f4(0.f);
        ncoef = ld4(coefC + p, any);
        nq = ld4(coefQ + p, any && !(xybox && zz >= zb.z0 && zz < zb.z1));
    };
    fetch(zbeg);
    const float c20 = Wt.c2[0];
    int aborted_at = -1;
    static_assert(ROT || !QS, "the shared density queue needs the unrolled plane loop");

    // one plane; J = (z - zbeg) mod QN when known at compile time (ROT)
    auto plane_step = [&](const int z, const int J) -> bool {
        const int it = z - zbeg;
        const int stage = it % kStages;
        auto slot = [&](int d) { return (J + R + d) % QN; };  // plane z + d
        const float4 vprev = nprev, vcoef = ncoef, vq = nq;
        float4 hu = f4(0.f), hr = f4(0.f);
        const bool more = z + 1 < zend;
        if (more) {
            const long long ph = (long long)(z + 1 + R) * L.plane + off;
            hu = ld4(uc + ph, any);
            if (VD) hr = ld4(den + ph, any);
            fetch(z + 1);
        }
        const long long pz = (long long)z * L.plane + off;

        // z axis: queues
        const float4 u0 = qu[slot(0)];
        float4 sdz = mul4(c20, u0), fuz = f4(0.f), frz = f4(0.f);
#pragma unroll
        for (int k = 1; k <= R; k++) {
            const float4 a = qu[slot(k)], b = qu[slot(-k)];
            sdz = fma4(Wt.c2[k], add4(a, b), sdz);
            if (VD) {
                fuz = fma4(Wt.c1[k], sub4(a, b), fuz);
                const float4 pa = RQ ? qr[slot(k)] : sq[slot(k) * kThreads];
                const float4 pb = RQ ? qr[slot(-k)] : sq[slot(-k) * kThreads];
                frz = fma4(Wt.c1[k], sub4(pa, pb), frz);
            }
        }
        float4 rho0 = f4(1.f);
        if (VD) rho0 = RQ ? qr[slot(0)] : sq[slot(0) * kThreads];

        const bool ok = mbar_wait(&bars[stage], (unsigned)((it / kStages) & 1));
        if (!ok) s_abort = 1;
        if (ok) {
            const float* tu = tiles + stage * VT::STRIDE + (warp + R) * TW + 4 * lane;
            const float* tr = tiles + (kStages + stage) * VT::STRIDE + (warp + R) * TW + 4 * lane;
            // x axis: rows x +- k of the tile, this thread's 4 columns
            float4 sdx = mul4(c20, u0), fux = f4(0.f), frx = f4(0.f);
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const float4 a = *reinterpret_cast<const float4*>(tu + k * TW + HY);
                const float4 b = *reinterpret_cast<const float4*>(tu - k * TW + HY);
                sdx = fma4(Wt.c2[k], add4(a, b), sdx);
                if (VD) {
                    fux = fma4(Wt.c1[k], sub4(a, b), fux);
                    const float4 ra = *reinterpret_cast<const float4*>(tr + k * TW + HY);
                    const float4 rb = *reinterpret_cast<const float4*>(tr - k * TW + HY);
                    frx = fma4(Wt.c1[k], sub4(ra, rb), frx);
                }
            }
            // y axis: window of 4 + 2*HY values of this thread's row
            float wu[4 * NC];
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const float4 t = *reinterpret_cast<const float4*>(tu + 4 * c);
                wu[4 * c] = t.x; wu[4 * c + 1] = t.y; wu[4 * c + 2] = t.z; wu[4 * c + 3] = t.w;
            }
            float4 sdy = mul4(c20, u0), fuy = f4(0.f), fry = f4(0.f);
#pragma unroll
            for (int v = 0; v < 4; v++) {
                float sy = comp(sdy, v), g = 0.f;
#pragma unroll
                for (int k = 1; k <= R; k++) {
                    sy = fmaf(Wt.c2[k], wu[HY + v + k] + wu[HY + v - k], sy);
                    if (VD) g = fmaf(Wt.c1[k], wu[HY + v + k] - wu[HY + v - k], g);
                }
                set_comp(sdy, v, sy);
                set_comp(fuy, v, g);
            }
            if (VD) {
                float wr[4 * NC];
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    const float4 t = *reinterpret_cast<const float4*>(tr + 4 * c);
                    wr[4 * c] = t.x; wr[4 * c + 1] = t.y; wr[4 * c + 2] = t.z; wr[4 * c + 3] = t.w;
                }
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    float g = 0.f;
#pragma unroll
                    for (int k = 1; k <= R; k++)
                        g = fmaf(Wt.c1[k], wr[HY + v + k] - wr[HY + v - k], g);
                    set_comp(fry, v, g);
                }
            }
            // combine (reference order y, x, z) and update
            float4 out;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                float lap = comp(sdy, v) * Wt.ih2[2] + comp(sdx, v) * Wt.ih2[1];
                lap = fmaf(comp(sdz, v), Wt.ih2[0], lap);
                if (VD) {
                    float cross = comp(fuy, v) * comp(fry, v) * Wt.s1[2] +
                                  comp(fux, v) * comp(frx, v) * Wt.s1[1];
                    cross = fmaf(comp(fuz, v) * comp(frz, v), Wt.s1[0], cross);
                    lap -= __fdividef(cross, comp(rho0, v));
                }
                set_comp(out, v, leapfrog_cq(lap, comp(vcoef, v), comp(vq, v), comp(u0, v),
                                             comp(vprev, v)));
            }
            if (full) {
                *reinterpret_cast<float4*>(un + pz) = out;
            } else if (any) {
#pragma unroll
                for (int v = 0; v < 4; v++)
                    if (y0 + v < ylim) un[pz + v] = comp(out, v);
            }
        }
        __syncthreads();  // the stage is free again; abort is uniform here
        if (s_abort) {
            aborted_at = it;
            return false;
        }
        if (threadIdx.x == 0 && z + kStages < zend) {
            issue(z + kStages, stage);
            issued++;
        }
        // plane z - R leaves the queues; plane z + R + 1 takes its slot
        if (more) {
            if (ROT) {
                qu[slot(-R)] = hu;
                if (RQ) qr[slot(-R)] = hr;
            } else {
#pragma unroll
                for (int j = 0; j < QN - 1; j++) {
                    qu[j] = qu[j + 1];
                    if (RQ) qr[j] = qr[j + 1];
                }
                qu[QN - 1] = hu;
                if (RQ) qr[QN - 1] = hr;
            }
            if (VD && QS) sq[slot(-R) * kThreads] = hr;
        }
        return true;
    };

    if (ROT) {
        for (int zb0 = zbeg; zb0 < zend; zb0 += QN) {
#pragma unroll
            for (int J = 0; J < QN; J++) {
                if (zb0 + J >= zend || !plane_step(zb0 + J, J)) break;
            }
            if (aborted_at >= 0) break;
        }
    } else {
        // register queues shifted every plane: plane z + d sits in slot R + d
        for (int z = zbeg; z < zend; z++)
            if (!plane_step(z, 0)) break;
    }
    if (aborted_at >= 0 && threadIdx.x == 0) {
        atomicExch(err, SIMWAVE_E_TIMEOUT);
        for (int p = aborted_at; p < issued; p++)
            mbar_wait(&bars[p % kStages], (unsigned)((p / kStages) & 1));
    }
}

// The float4 kernel's plane loop on pairs: z, x and y derivatives, the
// combine and the update on .f32x2. The plane loop is unrolled by the queue
// length (static queue slots). Variable density takes the density's z term
// either from a z-queue in shared memory (GZ false) or, with GZ, from the
// per-point array gz = s1_z * sum_k c1_k (rho(z+k) - rho(z-k)) formed once
// per run (form_density_z): 4 more bytes per point from memory, in exchange
// for the queue's shared-memory traffic (9 loads and a store per plane).
template <int R, bool VD, int MINB, bool GZ>
__global__ void __launch_bounds__(kThreads, MINB)
stencil3d_vec4p(const __grid_constant__ CUtensorMap map_u,
                const __grid_constant__ CUtensorMap map_rho, float* un,
                const float* __restrict__ uc, const float* up,
                const float* __restrict__ coefC, const float* __restrict__ den,
                const float* __restrict__ coefQ, const float* __restrict__ gz,
                Layout L, Weights<float> Wt, PairWeights PW, int slot_cur, int zchunk,
                ZeroBox zb, int* __restrict__ err) {
    using VT = VecTile<R>;
    constexpr int HY = VT::HY, TW = VT::TW, NC = VT::NC;
    constexpr int NF = VD ? 2 : 1;
    constexpr int QN = 2 * R + 1;
    constexpr bool SQ = VD && !GZ;  // density z-queue in shared memory
    static_assert(!GZ || VD, "gz is a variable-density term");
    float* tiles = reinterpret_cast<float*>(sw_dyn_smem);
    float4* sq_base = reinterpret_cast<float4*>(tiles + NF * kStages * VT::STRIDE);
    unsigned long long* bars =
        reinterpret_cast<unsigned long long*>(sq_base + (SQ ? QN * kThreads : 0));
    int& s_abort = *reinterpret_cast<int*>(bars + kStages);
    if (*(volatile int*)err) return;
    if (smem_addr(tiles) & 127) {
        if (threadIdx.x == 0) atomicExch(err, SIMWAVE_E_ARGUMENT);
        return;
    }

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int yb = R + blockIdx.x * 128;
    const int y0 = yb + 4 * lane;
    const int x = R + blockIdx.y * kWarps + warp;
    const int zbeg = R + blockIdx.z * zchunk;
    const int zend = min(zbeg + zchunk, (int)L.nz - R);
    if (zbeg >= zend) return;
    const int ylim = (int)L.ny - R;
    const bool any = x < (int)L.nx - R && y0 < ylim;
    const bool full = any && y0 + 3 < ylim;
    const int off = x * (int)L.pitch + (int)L.lead + y0;
    // threads past the interior load from the last interior row / chunk
    // (always inside the grid) instead of selecting zeros; only their
    // stores are masked
    const int xl = min(x, (int)L.nx - R - 1);
    const int yl = min(y0, R + 4 * ((ylim - 1 - R) / 4));
    const int offl = xl * (int)L.pitch + (int)L.lead + yl;
    const int col0 = (int)L.lead + yb - HY;
    const int row0 = blockIdx.y * kWarps;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();
    auto issue = [&](int plane, int stage) {
        mbar_expect_tx(&bars[stage], NF * VT::BYTES);
        tma_load_4d(tiles + stage * VT::STRIDE, &map_u, &bars[stage], col0, row0, plane,
                    slot_cur);
        if (VD)
            tma_load_4d(tiles + (kStages + stage) * VT::STRIDE, &map_rho, &bars[stage], col0,
                        row0, plane, 0);
    };
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < kStages && zbeg + issued < zend; issued++) issue(zbeg + issued, issued);

    // weight pairs held in registers for the whole chunk
    P2 w2[R + 1], w1[R + 1];
#pragma unroll
    for (int k = 0; k <= R; k++) {
        w2[k].v = PW.c2[k];
        w1[k].v = PW.c1[k];
    }
    auto vs = [&](int k, V4 x, V4 acc) -> V4 { return vfma(w2[k], x, acc); };
    auto vw = [&](bool first, int k, V4 x, V4 acc) -> V4 {
        return first ? vmul(w1[k], x) : vfma(w1[k], x, acc);
    };
    auto vs0 = [&](V4 x) -> V4 { return vmul(w2[0], x); };

    // queues hold planes z-R .. z+R; slot of plane p = (p - zbeg + R) mod QN
    V4 qu[QN];
    float4* sq = sq_base + threadIdx.x;
#pragma unroll
    for (int j = 0; j < QN; j++) {
        const long long pz = (long long)(zbeg - R + j) * L.plane + offl;
        qu[j] = ldg_v4(uc + pz, true);
        if (SQ) sts_v4(sq + j * kThreads, ldg_v4(den + pz, true));
    }
    const bool xybox = x >= zb.x0 && x < zb.x1 && y0 >= zb.y0 && y0 + 3 < zb.y1;
    // per-point operands of the next plane, fetched a plane ahead
    V4 nprev, ncoef, nq, ngz = vzero();
    bool nbox;
    auto fetch = [&](int zz) {
        const long long p = (long long)zz * L.plane + offl;
        nprev = ld_v4(up + p, true);
        ncoef = ldg_v4(coefC + p, true);
        if (GZ) ngz = ldg_v4(gz + p, true);
        nbox = xybox && zz >= zb.z0 && zz < zb.z1;
        nq = ldg_v4(coefQ + p, !nbox);
    };
    fetch(zbeg);
    int aborted_at = -1;
    long long zoff = (long long)zbeg * L.plane;  // z * plane of the current plane

    // plane z = zbeg + QN m + J: with QN a multiple of the stage count the
    // stage and the barrier parity are compile-time functions of J
    auto plane_step = [&](const int z, const int J, const int m) -> bool {
        constexpr bool kStatic = QN % kStages == 0;
        const int it = QN * m + J;
        const int stage = kStatic ? J % kStages : it % kStages;
        const unsigned parity =
            kStatic ? (unsigned)(((QN / kStages) * m + J / kStages) & 1) : (unsigned)((it / kStages) & 1);
        auto slot = [&](int d) { return (J + R + d) % QN; };  // plane z + d
        const V4 vprev = nprev, vcoef = ncoef, vq = nq, vgz = ngz;
        const bool inbox = nbox;
        V4 hu = vzero(), hr = vzero();
        const bool more = z + 1 < zend;
        if (more) {  // queue head (plane z+R+1) and the next plane's operands
            const long long ph = zoff + (long long)(R + 1) * L.plane + offl;
            hu = ldg_v4(uc + ph, true);
            if (SQ) hr = ldg_v4(den + ph, true);
            fetch(z + 1);
        }
        const long long pz = zoff + off;
        zoff += L.plane;

        // z axis: queues (first-derivative sums start at their k = 1 term)
        const V4 u0 = qu[slot(0)];
        V4 sdz = vs0(u0), fuz, frz;
#pragma unroll
        for (int k = 1; k <= R; k++) {
            const V4 a = qu[slot(k)], b = qu[slot(-k)];
            sdz = vs(k, vadd(a, b), sdz);
            if (VD) {
                fuz = vw(k == 1, k, vsub(a, b), fuz);
                if (SQ) {
                    const V4 pa = lds_v4(sq + slot(k) * kThreads);
                    const V4 pb = lds_v4(sq + slot(-k) * kThreads);
                    frz = vw(k == 1, k, vsub(pa, pb), frz);
                }
            }
        }
        V4 rho0 = vzero();
        if (SQ) rho0 = lds_v4(sq + slot(0) * kThreads);

        const bool ok = mbar_wait(&bars[stage], parity);
        if (!ok) s_abort = 1;
        if (ok) {
            const float* tu = tiles + stage * VT::STRIDE + (warp + R) * TW + 4 * lane;
            const float* tr = tiles + (kStages + stage) * VT::STRIDE + (warp + R) * TW + 4 * lane;
            // x axis: rows x +- k of the tile, this thread's 4 columns
            V4 sdx = vs0(u0), fux, frx;
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const V4 a = lds_v4(tu + k * TW + HY);
                const V4 b = lds_v4(tu - k * TW + HY);
                sdx = vs(k, vadd(a, b), sdx);
                if (VD) {
                    fux = vw(k == 1, k, vsub(a, b), fux);
                    const V4 ra = lds_v4(tr + k * TW + HY);
                    const V4 rb = lds_v4(tr - k * TW + HY);
                    frx = vw(k == 1, k, vsub(ra, rb), frx);
                }
            }
            // y axis on pairs: the window's pairs starting at even offsets
            // are the loaded 64-bit halves; odd offsets are repacked once
            V4 sdy, fuy, fry;
            {
                P2 ev[2 * NC], od[2 * NC - 1];
                YWindow<NC>::load(tu, ev, od);
                P2 s[2], g[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    s[h] = mul2(w2[0], h ? u0.hi : u0.lo);
#pragma unroll
                    for (int k = 1; k <= R; k++) {
                        const P2 a = YWindow<NC>::at(ev, od, HY + 2 * h + k);
                        const P2 b = YWindow<NC>::at(ev, od, HY + 2 * h - k);
                        s[h] = fma2(w2[k], add2(a, b), s[h]);
                        if (VD)
                            g[h] = k == 1 ? mul2(w1[k], sub2(a, b)) : fma2(w1[k], sub2(a, b), g[h]);
                    }
                }
                sdy = {s[0], s[1]};
                fuy = {g[0], g[1]};
                if (VD) {
                    YWindow<NC>::load(tr, ev, od);
                    if (GZ) rho0 = {ev[HY / 2], ev[HY / 2 + 1]};
#pragma unroll
                    for (int h = 0; h < 2; h++) {
#pragma unroll
                        for (int k = 1; k <= R; k++) {
                            const P2 a = YWindow<NC>::at(ev, od, HY + 2 * h + k);
                            const P2 b = YWindow<NC>::at(ev, od, HY + 2 * h - k);
                            g[h] = k == 1 ? mul2(w1[k], sub2(a, b)) : fma2(w1[k], sub2(a, b), g[h]);
                        }
                    }
                    fry = {g[0], g[1]};
                }
            }
            // combine (reference order y, x, z) and update, on pairs
            V4 lap = vmul({PW.ih2[2]}, sdy);
            lap = vfma({PW.ih2[1]}, sdx, lap);
            lap = vfma({PW.ih2[0]}, sdz, lap);
            if (VD) {
                const V4 my = {mul2(fuy.lo, fry.lo), mul2(fuy.hi, fry.hi)};
                V4 cross = vmul({PW.s1[2]}, my);
                cross = vfma({PW.s1[1]}, {mul2(fux.lo, frx.lo), mul2(fux.hi, frx.hi)}, cross);
                if (GZ)
                    cross = {fma2(fuz.lo, vgz.lo, cross.lo), fma2(fuz.hi, vgz.hi, cross.hi)};
                else
                    cross = vfma({PW.s1[0]}, {mul2(fuz.lo, frz.lo), mul2(fuz.hi, frz.hi)}, cross);
                const float4 rr = to_f4(rho0);
                const V4 inv = from_f4(make_float4(rcp_approx(rr.x), rcp_approx(rr.y),
                                                   rcp_approx(rr.z), rcp_approx(rr.w)));
                // lap -= cross / rho
                lap = {fma2(sub2({0ull}, cross.lo), inv.lo, lap.lo),
                       fma2(sub2({0ull}, cross.hi), inv.hi, lap.hi)};
            }
            // a = 2 u - (1 - q) u_prev;  b = a / (1 + q);  u_next = b + C lap
            const P2 one{PW.one};
            V4 a = {fma2(sub2(vq.lo, one), vprev.lo, add2(u0.lo, u0.lo)),
                    fma2(sub2(vq.hi, one), vprev.hi, add2(u0.hi, u0.hi))};
            if (!inbox) {
                const float4 qq = to_f4(vq);
                const V4 rq = from_f4(make_float4(
                    rcp_approx(1.f + qq.x), rcp_approx(1.f + qq.y),
                    rcp_approx(1.f + qq.z), rcp_approx(1.f + qq.w)));
                a = {mul2(a.lo, rq.lo), mul2(a.hi, rq.hi)};
            }
            const V4 out = {fma2(lap.lo, vcoef.lo, a.lo), fma2(lap.hi, vcoef.hi, a.hi)};
            if (full) {
                *reinterpret_cast<ulonglong2*>(un + pz) = make_ulonglong2(out.lo.v, out.hi.v);
            } else if (any) {
                const float4 o = to_f4(out);
#pragma unroll
                for (int v = 0; v < 4; v++)
                    if (y0 + v < ylim) un[pz + v] = comp(o, v);
            }
        }
        __syncthreads();  // the stage is free again; abort is uniform here
        if (s_abort) {
            aborted_at = it;
            return false;
        }
        if (threadIdx.x == 0 && z + kStages < zend) {
            issue(z + kStages, stage);
            issued++;
        }
        // plane z - R leaves the queues; plane z + R + 1 takes its slot
        if (more) {
            qu[slot(-R)] = hu;
            if (SQ) sts_v4(sq + slot(-R) * kThreads, hr);
        }
        return true;
    };

    for (int m = 0; zbeg + QN * m < zend; m++) {
#pragma unroll
        for (int J = 0; J < QN; J++) {
            const int z = zbeg + QN * m + J;
            if (z >= zend || !plane_step(z, J, m)) break;
        }
        if (aborted_at >= 0) break;
    }
    if (aborted_at >= 0 && threadIdx.x == 0) {
        atomicExch(err, SIMWAVE_E_TIMEOUT);
        for (int p = aborted_at; p < issued; p++)
            mbar_wait(&bars[p % kStages], (unsigned)((p / kStages) & 1));
    }
}

// ---- host side ---------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 4D map over (pitched row, x, z, slot) with a (W, H, 1, 1) box.
bool encode_map(CUtensorMap* map, const float* base, const Layout& L, long long slots,
                long long slot_stride, int box_w, int box_h) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[4] = {(cuuint64_t)L.pitch, (cuuint64_t)L.nx, (cuuint64_t)L.nz,
                          (cuuint64_t)slots};
    cuuint64_t strides[3] = {(cuuint64_t)L.pitch * 4, (cuuint64_t)L.plane * 4,
                             (cuuint64_t)slot_stride * 4};
    cuuint32_t box[4] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims,
                    strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

struct DeviceInfo {
    int sms = 0;
};

DeviceInfo& device_info() {
    static DeviceInfo info[64];
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceInfo& d = info[dev & 63];
    if (!d.sms) cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    return d;
}


// z chunk length: fill the machine in whole waves, counting the 2R-plane
// warm-up of every chunk as the cost of splitting.
int choose_chunk(int ty, int tx, int nzi, int R, int per_sm) {
    const long long slots = (long long)std::max(per_sm, 1) * device_info().sms;
    int best = 1;
    double best_cost = 1e300;
    for (int zs = 1; zs <= 32 && zs <= nzi; zs++) {
        const long long ctas = (long long)ty * tx * zs;
        const long long waves = (ctas + slots - 1) / slots;
        const int chunk = (nzi + zs - 1) / zs;
        const double cost = (double)waves * (chunk + 2.0 * R * 0.5);
        if (cost < best_cost * 0.999) {
            best_cost = cost;
            best = zs;
        }
    }
    return (nzi + best - 1) / best;
}

template <int R, bool VD>
size_t smem_bytes() {
    return (size_t)(VD ? 2 : 1) * kStages * Tile<R>::STRIDE * 4 + 64;
}

template <int R, bool VD>
void launch_r(float* un, const float* uc, const float* up, const float* vel, const float* den,
              const float* damp, const Layout& L, const Weights<float>& W, float dt, float dt2,
              const TiledContext& ctx, cudaStream_t st) {
    using TL = Tile<R>;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t smem = smem_bytes<R, VD>();
    if (!configured[dev & 63]) {
        cudaFuncSetAttribute(stencil3d_tiled<R, VD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        configured[dev & 63] = true;
    }
    const int ty = (int)((L.ny - 2 * R + 31) / 32);
    const int tx = (int)((L.nx - 2 * R + TL::TX - 1) / TL::TX);
    const int nzi = (int)(L.nz - 2 * R);
    static std::atomic<int> per_sm_of[64];  // resident CTAs per SM, queried once per device
    if (!per_sm_of[dev & 63]) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, stencil3d_tiled<R, VD>, kThreads, smem);
        per_sm_of[dev & 63] = std::max(v, 1);
    }
    const int per_sm = per_sm_of[dev & 63];
    const int chunk = choose_chunk(ty, tx, nzi, R, per_sm);
    const int zsplit = (nzi + chunk - 1) / chunk;
    const long long cur_slot = (uc - ctx.u_base) / ctx.slot_stride;
    ZeroBox zb{ctx.zero_box[0], ctx.zero_box[1], ctx.zero_box[2],
               ctx.zero_box[3], ctx.zero_box[4], ctx.zero_box[5]};
    dim3 grid(ty, tx, zsplit);
    stencil3d_tiled<R, VD><<<grid, kThreads, smem, st>>>(
        *reinterpret_cast<const CUtensorMap*>(ctx.map_u),
        *reinterpret_cast<const CUtensorMap*>(ctx.map_rho), un, uc, up, vel, den, damp, L, W,
        dt, dt2, (int)cur_slot, chunk, zb, ctx.err);
}

// Along each axis line through the grid centre, the run of zeros of the mask
// around the centre: block a scans axis a (strided over its threads) for the
// nearest nonzero on either side (shared-memory max / min); in 2D the y range
// is [0, 1).
__global__ void zero_box_lines(const float* __restrict__ damp, Layout L, int* box) {
    const int a = blockIdx.x;
    if (a >= 3) return;
    __shared__ int below, above;  // nearest nonzero index below / above the centre
    const long long c[3] = {L.nz / 2, L.nx / 2, L.ny / 2};
    const long long n = L.extent(a);
    auto at = [&](long long i) {
        long long idx[3] = {c[0], c[1], c[2]};
        idx[a] = i;
        return damp[L.dim == 3 ? L.at3(idx[0], idx[1], idx[2]) : L.at2(idx[0], idx[1])];
    };
    if (threadIdx.x == 0) {
        below = -1;
        above = (int)n;
    }
    __syncthreads();
    int lo = -1, hi = (int)n;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        if (i == c[a] || at(i) == 0.f) continue;
        if (i < c[a]) lo = max(lo, (int)i);
        else hi = min(hi, (int)i);
    }
    atomicMax(&below, lo);
    atomicMin(&above, hi);
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool centre_zero = at(c[a]) == 0.f;
        box[2 * a] = centre_zero ? below + 1 : 0;
        box[2 * a + 1] = centre_zero ? above : 0;
    }
}

// Verify the candidate box: box[6] becomes nonzero if any point inside has a
// nonzero mask.
__global__ void zero_box_verify(const float* __restrict__ damp, Layout L, int* box) {
    const int z0 = box[0], z1 = box[1], x0 = box[2], x1 = box[3], y0 = box[4], y1 = box[5];
    const long long nyb = y1 - y0, nxb = x1 - x0, nzb = z1 - z0;
    if (nyb <= 0 || nxb <= 0 || nzb <= 0) return;
    const long long total = nzb * nxb * nyb;
    int bad = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long k = t % nyb, j = (t / nyb) % nxb, i = t / (nyb * nxb);
        bad |= damp[L.dim == 3 ? L.at3(z0 + i, x0 + j, y0 + k) : L.at2(z0 + i, x0 + j)] != 0.f;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(box + 6, 1);
}


template <int R, bool VD, bool QS>
size_t vec_smem_bytes() {
    const size_t queue = (VD && QS) ? (size_t)(2 * R + 1) * kThreads * 16 : 0;
    return (size_t)(VD ? 2 : 1) * kStages * VecTile<R>::STRIDE * 4 + queue + 64;
}

template <int R, bool VD, int MINB, bool QS, bool ROT>
void launch_vec(float* un, const float* uc, const float* up, const float* coefC,
                const float* den, const float* coefQ, const Layout& L, const Weights<float>& W,
                const TiledContext& ctx, cudaStream_t st) {
    auto kernel = stencil3d_vec4<R, VD, MINB, QS, ROT>;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t smem = vec_smem_bytes<R, VD, QS>();
    if (!configured[dev & 63]) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured[dev & 63] = true;
    }
    const int ty = (int)((L.ny - 2 * R + 127) / 128);
    const int tx = (int)((L.nx - 2 * R + kWarps - 1) / kWarps);
    const int nzi = (int)(L.nz - 2 * R);
    static std::atomic<int> per_sm_of[64];  // resident CTAs per SM, queried once per device
    if (!per_sm_of[dev & 63]) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, kThreads, smem);
        per_sm_of[dev & 63] = std::max(v, 1);
    }
    const int per_sm = per_sm_of[dev & 63];
    const int chunk = choose_chunk(ty, tx, nzi, R, per_sm);
    const int zsplit = (nzi + chunk - 1) / chunk;
    const long long cur_slot = (uc - ctx.u_base) / ctx.slot_stride;
    ZeroBox zb{ctx.zero_box[0], ctx.zero_box[1], ctx.zero_box[2],
               ctx.zero_box[3], ctx.zero_box[4], ctx.zero_box[5]};
    dim3 grid(ty, tx, zsplit);
    kernel<<<grid, kThreads, smem, st>>>(
        *reinterpret_cast<const CUtensorMap*>(ctx.map_u_vec),
        *reinterpret_cast<const CUtensorMap*>(ctx.map_rho_vec), un, uc, up, coefC, den, coefQ,
        L, W, (int)cur_slot, chunk, zb, ctx.err);
}

template <int R, bool VD, int MINB, bool GZ>
void launch_vecp(float* un, const float* uc, const float* up, const float* coefC,
                 const float* den, const float* coefQ, const Layout& L, const Weights<float>& W,
                 const TiledContext& ctx, cudaStream_t st) {
    auto kernel = stencil3d_vec4p<R, VD, MINB, GZ>;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t smem = vec_smem_bytes<R, VD, VD && !GZ>();
    if (!configured[dev & 63]) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured[dev & 63] = true;
    }
    const int ty = (int)((L.ny - 2 * R + 127) / 128);
    const int tx = (int)((L.nx - 2 * R + kWarps - 1) / kWarps);
    const int nzi = (int)(L.nz - 2 * R);
    static std::atomic<int> per_sm_of[64];  // resident CTAs per SM, queried once per device
    if (!per_sm_of[dev & 63]) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, kThreads, smem);
        per_sm_of[dev & 63] = std::max(v, 1);
    }
    const int per_sm = per_sm_of[dev & 63];
    const int chunk = choose_chunk(ty, tx, nzi, R, per_sm);
    const int zsplit = (nzi + chunk - 1) / chunk;
    const long long cur_slot = (uc - ctx.u_base) / ctx.slot_stride;
    ZeroBox zb{ctx.zero_box[0], ctx.zero_box[1], ctx.zero_box[2],
               ctx.zero_box[3], ctx.zero_box[4], ctx.zero_box[5]};
    dim3 grid(ty, tx, zsplit);
    kernel<<<grid, kThreads, smem, st>>>(
        *reinterpret_cast<const CUtensorMap*>(ctx.map_u_vec),
        *reinterpret_cast<const CUtensorMap*>(ctx.map_rho_vec), un, uc, up, coefC, den, coefQ,
        ctx.coefGz, L, W, pair_weights(W), (int)cur_slot, chunk, zb, ctx.err);
}

// The packed kernel with the density z term from ctx.coefGz where the run
// formed it, else from the shared-memory queue.
template <int R, bool VD, int MINB>
void launch_vecp_any(float* un, const float* uc, const float* up, const float* coefC,
                     const float* den, const float* coefQ, const Layout& L,
                     const Weights<float>& W, const TiledContext& ctx, cudaStream_t st) {
    if (VD && ctx.coefGz)
        launch_vecp<R, VD, MINB, VD>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
    else
        launch_vecp<R, VD, MINB, false>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
}

// The kernel AUTO runs for radius r (measured on a 408^3 grid, ms per
// launch): the packed kernel for r <= 4 (constant density at order 2 keeps
// the float4 kernel: 0.224 vs 0.265); for r = 5..8 the packed kernel where
// it beat the scalar one (constant density: 0.31/0.29/0.41 vs
// 0.37/0.45/0.46 at orders 10/12/14, the one-CTA build at order 16: 0.47 vs
// 0.51; variable density only at order 10: 0.52 vs 0.63, its register
// spills lose above), else the scalar kernel.
int auto_policy(int r, bool vd) {
    // order 8 with variable density (472^3 grid, ms per launch): the
    // stage-release kernel 0.545, the packed kernel 0.555, the TMEM kernel 0.66
    if (r == 4 && vd) return SIMWAVE_POLICY_STAGE_RELEASE;
    if (r <= 4) return (!vd && r == 1) ? SIMWAVE_POLICY_VEC_2CTA : SIMWAVE_POLICY_VEC_PACKED;
    if (r <= 8) {
        if (vd) return r == 5 ? SIMWAVE_POLICY_VEC_PACKED : SIMWAVE_POLICY_SCALAR_TILED;
        return r == 8 ? SIMWAVE_POLICY_VEC_PACKED_1CTA : SIMWAVE_POLICY_VEC_PACKED;
    }
    return SIMWAVE_POLICY_SCALAR_TILED;
}

template <int R, bool VD>
void launch_vec_policy(int policy, float* un, const float* uc, const float* up,
                       const float* coefC, const float* den, const float* coefQ,
                       const Layout& L, const Weights<float>& W, const TiledContext& ctx,
                       cudaStream_t st) {
    if (policy == SIMWAVE_POLICY_AUTO) policy = auto_policy(R, VD);
    switch (policy) {
        case SIMWAVE_POLICY_VEC_2CTA:
            return launch_vec<R, VD, 2, false, false>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        case SIMWAVE_POLICY_VEC_1CTA:
            return launch_vec<R, VD, 1, false, false>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        case SIMWAVE_POLICY_VEC_SMEMQ:
            return launch_vec<R, VD, 2, VD, true>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        case SIMWAVE_POLICY_VEC_2CTA_ROT:
            return launch_vec<R, VD, 2, false, true>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        case SIMWAVE_POLICY_VEC_PACKED:
            return launch_vecp_any<R, VD, 2>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        case SIMWAVE_POLICY_VEC_PACKED_1CTA:
            return launch_vecp_any<R, VD, 1>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
        default:  // SIMWAVE_POLICY_VEC_1CTA_ROT
            return launch_vec<R, VD, 1, false, true>(un, uc, up, coefC, den, coefQ, L, W, ctx, st);
    }
}
}  // namespace

void form_density_z(const float* den, float* gz, const Layout& L, const Weights<float>& W,
                    cudaStream_t st) {
    form_density_z<<<device_info().sms * 8, 256, 0, st>>>(den, gz, L, W);
}

bool wants_density_z(const Layout& L, bool vd) {
    int p = kernel_policy();
    if (p == SIMWAVE_POLICY_AUTO) p = auto_policy(L.r, vd);
    if ((p == SIMWAVE_POLICY_TMEM || p == SIMWAVE_POLICY_STAGE_RELEASE) && L.r <= 4)
        return vd && L.dim == 3 && p == SIMWAVE_POLICY_STAGE_RELEASE;
    return vd && L.dim == 3 && L.r <= 8 &&
           (p == SIMWAVE_POLICY_VEC_PACKED || p == SIMWAVE_POLICY_VEC_PACKED_1CTA);
}

void form_coefficients(const float* vel, const float* damp, float* C, float* Q,
                       long long n, float dt, cudaStream_t st) {
    form_coefficients<<<device_info().sms * 8, 256, 0, st>>>(vel, damp, C, Q, n, dt);
}

static int g_policy = SIMWAVE_POLICY_AUTO;
int kernel_policy() { return g_policy; }
void set_kernel_policy(int p) { g_policy = p; }

void find_zero_box(const float* damp, const Layout& L, int* box, cudaStream_t st) {
    cudaMemsetAsync(box, 0, 7 * sizeof(int), st);
    zero_box_lines<<<3, 256, 0, st>>>(damp, L, box);
    zero_box_verify<<<device_info().sms * 4, 256, 0, st>>>(damp, L, box);
}

static_assert(sizeof(CUtensorMap) <= sizeof(TiledContext::map_u), "map storage");

bool tiled_prepare(TiledContext& ctx, const Layout& L, bool vd, float* u_base,
                   long long nslots, long long slot_stride, const float* den) {
    ctx.ok = false;
    if (L.dim != 3 || L.r < 1 || L.r > kMaxRadius) return false;
    if (L.pitch % 4 || ((L.lead + L.r) % 32) || (reinterpret_cast<uintptr_t>(u_base) % 16) ||
        (slot_stride % 4) || L.nx > (1 << 30) || L.nz > (1 << 30) || nslots > (1 << 30))
        return false;
    if (vd && (!den || reinterpret_cast<uintptr_t>(den) % 16)) return false;
    if (!encode_fn()) return false;
    const int r = L.r;
    const int NX = r <= 4 ? 4 : (r <= 7 ? 2 : 1);
    const int box_w = 32 + 2 * round4(r);
    const int box_h = kWarps * NX + 2 * r;
    if (box_w > 256 || box_h > 256) return false;
    CUtensorMap mu, mr;
    if (!encode_map(&mu, u_base, L, nslots, slot_stride, box_w, box_h)) return false;
    if (vd) {
        if (!encode_map(&mr, den, L, 1, L.nz * L.plane, box_w, box_h)) return false;
    } else {
        mr = mu;
    }
    std::memcpy(ctx.map_u, &mu, sizeof(mu));
    std::memcpy(ctx.map_rho, &mr, sizeof(mr));
    // float4 kernel: orders up to 8, 16-byte aligned rows and arrays
    ctx.vec = false;
    if (r <= 8 && (L.lead + r) % 4 == 0) {
        const int vw = 128 + 2 * round4(r), vh = kWarps + 2 * r;
        CUtensorMap vu, vr;
        if (encode_map(&vu, u_base, L, nslots, slot_stride, vw, vh) &&
            (!vd || encode_map(&vr, den, L, 1, L.nz * L.plane, vw, vh))) {
            if (!vd) vr = vu;
            std::memcpy(ctx.map_u_vec, &vu, sizeof(vu));
            std::memcpy(ctx.map_rho_vec, &vr, sizeof(vr));
            ctx.vec = true;
        }
    }
    // tensor-memory kernel: orders up to 8, boxes of its x rows
    ctx.tm = false;
    const int pol = resolve_policy(kernel_policy(), r, vd);
    if (r <= 4 && (L.lead + r) % 4 == 0 &&
        (pol == SIMWAVE_POLICY_TMEM || pol == SIMWAVE_POLICY_STAGE_RELEASE)) {
        const int rows = tmem_rows(pol);
        const int vw = 128 + 2 * round4(r), vh = rows + 2 * r;
        CUtensorMap tu, trm;
        if (encode_map(&tu, u_base, L, nslots, slot_stride, vw, vh) &&
            (!vd || encode_map(&trm, den, L, 1, L.nz * L.plane, vw, vh))) {
            if (!vd) trm = tu;
            std::memcpy(ctx.map_u_tm, &tu, sizeof(tu));
            std::memcpy(ctx.map_rho_tm, &trm, sizeof(trm));
            ctx.tm = true;
            ctx.tm_rows = rows;
            ctx.tm_tables = pol == SIMWAVE_POLICY_TMEM;
        }
    }
    ctx.u_base = u_base;
    ctx.slot_stride = slot_stride;
    ctx.ok = true;
    return true;
}

int resolve_policy(int policy, int r, bool vd) {
    return policy == SIMWAVE_POLICY_AUTO ? auto_policy(r, vd) : policy;
}

int tiled_launch(const TiledContext& ctx, bool vd, float* un, const float* uc, const float* up,
                  const float* vel, const float* den, const float* damp, const Layout& L,
                  const Weights<float>& W, float dt, float dt2, cudaStream_t st) {
    int policy = kernel_policy();
    const int resolved = resolve_policy(policy, L.r, vd);
    if (resolved == SIMWAVE_POLICY_TMEM || resolved == SIMWAVE_POLICY_STAGE_RELEASE) {
        if (tmem_launch(ctx, resolved, vd, un, uc, up, vel, den, L, W, st)) return resolved;
        policy = SIMWAVE_POLICY_VEC_PACKED;  // the context was prepared for another kernel
    }
    const bool aligned =
        (reinterpret_cast<uintptr_t>(vel) | reinterpret_cast<uintptr_t>(damp) |
         reinterpret_cast<uintptr_t>(un) | reinterpret_cast<uintptr_t>(up) |
         reinterpret_cast<uintptr_t>(uc)) % 16 == 0;
    const int high = (policy == SIMWAVE_POLICY_AUTO && L.r >= 5) ? auto_policy(L.r, vd) : policy;
    if (ctx.vec && L.r >= 5 && L.r <= 8 && aligned &&
        (high == SIMWAVE_POLICY_VEC_PACKED || high == SIMWAVE_POLICY_VEC_PACKED_1CTA)) {
        const bool one = high == SIMWAVE_POLICY_VEC_PACKED_1CTA;
#define SW_VECH(RR)                                                                           \
    case RR:                                                                                  \
        if (vd) {                                                                             \
            if (one) launch_vecp_any<RR, true, 1>(un, uc, up, vel, den, damp, L, W, ctx, st);  \
            else launch_vecp_any<RR, true, 2>(un, uc, up, vel, den, damp, L, W, ctx, st);      \
        } else {                                                                              \
            if (one) launch_vecp_any<RR, false, 1>(un, uc, up, vel, den, damp, L, W, ctx, st); \
            else launch_vecp_any<RR, false, 2>(un, uc, up, vel, den, damp, L, W, ctx, st);     \
        }                                                                                     \
        return high;
        switch (L.r) { SW_VECH(5) SW_VECH(6) SW_VECH(7) SW_VECH(8) }
#undef SW_VECH
    }
    if (ctx.vec && L.r <= 4 && policy != SIMWAVE_POLICY_SCALAR_TILED &&
        (reinterpret_cast<uintptr_t>(vel) | reinterpret_cast<uintptr_t>(damp) |
         reinterpret_cast<uintptr_t>(un) | reinterpret_cast<uintptr_t>(up) |
         reinterpret_cast<uintptr_t>(uc)) % 16 == 0) {
#define SW_VEC(RR)                                                                              \
    case RR:                                                                                    \
        if (vd) launch_vec_policy<RR, true>(policy, un, uc, up, vel, den, damp, L, W, ctx, st); \
        else launch_vec_policy<RR, false>(policy, un, uc, up, vel, den, damp, L, W, ctx, st);   \
        return policy == SIMWAVE_POLICY_AUTO ? auto_policy(RR, vd) : policy;
        switch (L.r) { SW_VEC(1) SW_VEC(2) SW_VEC(3) SW_VEC(4) }
#undef SW_VEC
    }
#define SW_CASE(RR)                                                                    \
    case RR:                                                                           \
        if (vd) launch_r<RR, true>(un, uc, up, vel, den, damp, L, W, dt, dt2, ctx, st); \
        else launch_r<RR, false>(un, uc, up, vel, den, damp, L, W, dt, dt2, ctx, st);   \
        break;
    switch (L.r) {
        SW_CASE(1) SW_CASE(2) SW_CASE(3) SW_CASE(4) SW_CASE(5)
        SW_CASE(6) SW_CASE(7) SW_CASE(8) SW_CASE(9) SW_CASE(10)
        default: break;
    }
#undef SW_CASE
    return SIMWAVE_POLICY_SCALAR_TILED;
}

}  // namespace sw
