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
#include <cstdio>
#include <cstring>
#include <mutex>

#include "simwave_gb300.h"
#include "sw_tiled.h"

namespace sw {

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;
constexpr int kStages = 3;              // planes in flight per field
constexpr unsigned kSpinLimit = 1u << 20;  // mbarrier polls before giving up

__host__ __device__ constexpr int round4(int r) { return (r + 3) & ~3; }

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

// ---- PTX helpers -----------------------------------------------------------

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Bounded wait for phase `parity` of `bar`; returns false on expiry.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const unsigned addr = smem_addr(bar);
    for (unsigned i = 0; i < kSpinLimit; i++) {
        unsigned ok;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map,
                                            unsigned long long* bar, int c0, int c1,
                                            int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
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
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // TMA destinations 128-byte aligned whatever the dynamic base alignment
    float* tiles = reinterpret_cast<float*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));  // [NF][kStages][STRIDE]
    __shared__ __align__(8) unsigned long long bars[kStages];
    if (*(volatile int*)err) return;  // an earlier launch already failed

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
        // per-point operands of this plane
        const long long pz = (long long)z * L.plane;
        float vprev[NX], vvel[NX], vdamp[NX];
        const bool zin = z >= zb.z0 && z < zb.z1 && y >= zb.y0 && y < zb.y1;
#pragma unroll
        for (int i = 0; i < NX; i++) {
            // plain load: u_prev may be the slot this kernel writes
            vprev[i] = xok[i] ? up[pz + off[i]] : 0.f;
            vvel[i] = xok[i] ? __ldg(vel + pz + off[i]) : 0.f;
            const bool inbox = zin && x0 + i >= zb.x0 && x0 + i < zb.x1;
            vdamp[i] = (xok[i] && !inbox) ? __ldg(damp + pz + off[i]) : 0.f;
        }

        const bool ok = mbar_wait(&bars[stage], (unsigned)((it / kStages) & 1));
        if (__syncthreads_or(!ok)) {
            aborted_at = it;
            break;
        }
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
            const float v2 = vvel[i] * vvel[i];
            const float q = vdamp[i] * dt * v2 * 0.5f;
            const float rden = __frcp_rn(1.f + q);
            const float num = fmaf(-(1.f - q), vprev[i], 2.f * u0);
            const float unew = fmaf(dt2 * v2, lap, num) * rden;
            if (xok[i]) un[pz + off[i]] = unew;
        }

        __syncthreads();  // everyone is done with this stage's tiles
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

template <int R, bool VD>
size_t smem_bytes() {
    return (size_t)(VD ? 2 : 1) * kStages * Tile<R>::STRIDE * 4 + 128;
}

template <int R, bool VD>
void launch_r(float* un, const float* uc, const float* up, const float* vel, const float* den,
              const float* damp, const Layout& L, const Weights<float>& W, float dt, float dt2,
              const TiledContext& ctx, cudaStream_t st) {
    using TL = Tile<R>;
    static bool configured[64] = {};
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
    // z chunks: fill the machine in whole waves, with the 2R-plane warm-up
    // of every chunk as the cost of splitting
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stencil3d_tiled<R, VD>, kThreads,
                                                  smem);
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
    const int chunk = (nzi + best - 1) / best;
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

// Walk each axis line through the grid centre outwards while the mask is
// zero; one thread per axis.
__global__ void zero_box_lines(const float* __restrict__ damp, Layout L, int* box) {
    const int a = threadIdx.x;
    if (a >= 3) return;
    const long long c[3] = {L.nz / 2, L.nx / 2, L.ny / 2};
    const long long n = L.extent(a);
    auto at = [&](long long i) {
        long long idx[3] = {c[0], c[1], c[2]};
        idx[a] = i;
        return damp[L.at3(idx[0], idx[1], idx[2])];
    };
    long long lo = c[a], hi = c[a];
    if (at(c[a]) != 0.f) {
        box[2 * a] = 0;
        box[2 * a + 1] = 0;
        return;
    }
    while (lo - 1 >= 0 && at(lo - 1) == 0.f) lo--;
    while (hi + 1 < n && at(hi + 1) == 0.f) hi++;
    box[2 * a] = (int)lo;
    box[2 * a + 1] = (int)hi + 1;
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
        bad |= damp[L.at3(z0 + i, x0 + j, y0 + k)] != 0.f;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(box + 6, 1);
}

}  // namespace

void find_zero_box(const float* damp, const Layout& L, int* box, cudaStream_t st) {
    cudaMemsetAsync(box, 0, 7 * sizeof(int), st);
    zero_box_lines<<<1, 32, 0, st>>>(damp, L, box);
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
    ctx.u_base = u_base;
    ctx.slot_stride = slot_stride;
    ctx.ok = true;
    return true;
}

void tiled_launch(const TiledContext& ctx, bool vd, float* un, const float* uc, const float* up,
                  const float* vel, const float* den, const float* damp, const Layout& L,
                  const Weights<float>& W, float dt, float dt2, cudaStream_t st) {
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
}

}  // namespace sw
