// sw_batch.cu -- many independent 2D shots advanced together.
//
// A shot is one forward problem (2D, float32, any order, density and saving
// stride) whose arrays are resident on the device (the caller owns u, the
// models, the KWS tables, the wavelet and the receivers; the engine owns the
// per-point coefficients C, Q and the shot's slot schedule). Each time step of
// the batch is a fixed sequence of launches over *all* shots:
//   1. stencil   one launch per (radius, density) group; a CTA is one
//                128 x TZ tile of one shot (tile list in device memory)
//   2. sources   one block per (shot, source)
//   3. x edges, then z edges (the reference's order), one block per shot
//   4. receivers one warp per (shot, receiver)
//   5. advance   each shot's step counter
// Every kernel reads the shot's current step from its device descriptor and
// does nothing for a shot that is past its last step, so the launch sequence
// of K steps is captured once into a CUDA graph and replayed until the set of
// shots changes (shots that finish simply go idle).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "simwave_gb300.h"
#include "sw_kernels.cuh"
#include "sw_pairs.cuh"
#include "sw_tiled.h"

namespace sw {

void record_error(const std::string& message);

namespace batch {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxGroups = 2 * kMaxRadius;  // (radius, density) pairs

// Device descriptor of one shot.
struct Shot {
    Layout L;
    float* u;              // slot 0; slots are L.slot apart
    const float* C;        // (dt^2 v^2) / (1 + Q), per point
    const float* Q;        // damp dt v^2 / 2, per point
    const float* vel;      // for the source term
    const float* damp;
    const float* den;      // null for constant density
    Weights<float> W;
    Windows<float> src, rec;
    const float* wavelet;
    unsigned long long wavelet_count;
    float* receivers;      // [end][rec.count]
    const int* slots;      // [end - begin + 1][3]: physical prev, cur, next
    float dt, dt2;
    int n, begin, end;     // next step to run, first and last step
    int bc[4];
    int zb[4];             // z0, z1, x0, x1: box where Q is zero
};

struct ZeroBox2 {
    int b[4];
};

struct TileRef {
    int shot, tz, tx;
};
struct PairRef {
    int shot, item;
};

__device__ __forceinline__ bool active(const Shot& s) { return s.n <= s.end; }

__device__ __forceinline__ void slot_ptrs(const Shot& s, float*& un, const float*& uc,
                                          const float*& up) {
    const int* sl = s.slots + 3 * (s.n - s.begin);
    up = s.u + (long long)sl[0] * s.L.slot;
    uc = s.u + (long long)sl[1] * s.L.slot;
    un = s.u + (long long)sl[2] * s.L.slot;
}

// ---- tiled 2D stencil -------------------------------------------------------------
// Tile: 128 x-points (32 lanes x float4) by TZ rows; u (and rho) with an R
// halo staged in shared memory by plain 16-byte loads; each warp computes
// TZ / 8 rows. Same arithmetic as the 3D tiled kernels: unscaled half
// weights, per-axis 1/h^2, per-point C and Q coefficients.
template <int R, bool VD, int TZ>
__device__ __forceinline__ void stencil2d_tile(float* tile, const Layout& L, float* un,
                                               const float* uc, const float* up,
                                               const float* C, const float* Q,
                                               const float* den, const Weights<float>& W,
                                               const int* zb, int tz, int tx) {
    constexpr int HX = (R + 3) & ~3;
    constexpr int TW = 128 + 2 * HX;   // floats per tile row
    constexpr int TH = TZ + 2 * R;     // tile rows
    constexpr int NF = VD ? 2 : 1;
    constexpr int NC = (4 + 2 * HX) / 4;             // 16-byte chunks of an x window
    constexpr int RPW = (TZ + kWarps - 1) / kWarps;  // rows per warp
    const int z0 = R + tz * TZ;             // first row of the tile
    const int x0 = R + tx * 128;            // first column (interior index)
    const int col0 = (int)L.lead + x0 - HX;  // pitched column of tile column 0
    const int pitch = (int)L.pitch;
    const int nz = (int)L.nz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = x0 + 4 * lane;            // first of this lane's 4 points
    const int xlim = (int)L.nx - R;         // interior x < xlim
    const bool xbox = x >= zb[2] && x + 3 < zb[3];

    // per-point operands of this warp's rows, requested before the tile is
    // staged so that their latency overlaps the staging; partial chunks read
    // into the next row (never the last row) and are masked at the store
    V4 cc[RPW], pv[RPW], qq[RPW];
    bool qzero[RPW];
#pragma unroll
    for (int j = 0; j < RPW; j++) {
        const int z = z0 + warp + j * kWarps;
        const bool ok = warp + j * kWarps < TZ && z < nz - R && x < xlim;
        const long long p = (long long)z * pitch + L.lead + x;
        qzero[j] = xbox && z >= zb[0] && z < zb[1];  // damping-free box
        cc[j] = ldg_v4(C + p, ok);
        pv[j] = ld_v4(up + p, ok);
        qq[j] = ldg_v4(Q + p, ok && !qzero[j]);
    }

    // stage: rows z0-R .. z0+TZ+R-1, columns col0 .. col0+TW-1 (guarded)
    constexpr int CH = TW / 4;  // float4 chunks per row
    for (int f = 0; f < NF; f++) {
        const float* src = f == 0 ? uc : den;
        float* dst = tile + f * TH * TW;
        for (int i = threadIdx.x; i < TH * CH; i += kThreads) {
            const int row = i / CH, ch = i - row * CH;
            const int z = z0 - R + row;
            const int col = col0 + 4 * ch;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            if (z < nz && col + 3 < pitch)
                val = *reinterpret_cast<const float4*>(src + (long long)z * pitch + col);
            *reinterpret_cast<float4*>(dst + row * TW + 4 * ch) = val;
        }
    }
    __syncthreads();

    // weights as pairs {w, w}
    P2 w2[R + 1], w1[R + 1];
#pragma unroll
    for (int k = 0; k <= R; k++) {
        w2[k] = pk(W.c2[k], W.c2[k]);
        w1[k] = pk(W.c1[k], W.c1[k]);
    }
    const P2 ihx = pk(W.ih2[1], W.ih2[1]), ihz = pk(W.ih2[0], W.ih2[0]);
    const P2 one = pk(1.f, 1.f);
#pragma unroll
    for (int j = 0; j < RPW; j++) {
        const int rr = warp + j * kWarps;
        const int z = z0 + rr;
        if (rr >= TZ || z >= nz - R || x >= xlim) continue;
        const float* tu = tile + (rr + R) * TW + 4 * lane;      // row z, chunk start
        const float* tr = tile + TH * TW + (rr + R) * TW + 4 * lane;
        const long long p = (long long)z * pitch + L.lead + x;
        // z axis: rows z +- k of the tile, this lane's 4 columns
        const V4 u0 = lds_v4(tu + HX);
        V4 sz = vmul(w2[0], u0), gz, rz;
#pragma unroll
        for (int k = 1; k <= R; k++) {
            const V4 a = lds_v4(tu + k * TW + HX);
            const V4 b = lds_v4(tu - k * TW + HX);
            sz = vfma(w2[k], vadd(a, b), sz);
            if (VD) {
                gz = k == 1 ? vmul(w1[k], vsub(a, b)) : vfma(w1[k], vsub(a, b), gz);
                const V4 ra = lds_v4(tr + k * TW + HX);
                const V4 rb = lds_v4(tr - k * TW + HX);
                rz = k == 1 ? vmul(w1[k], vsub(ra, rb)) : vfma(w1[k], vsub(ra, rb), rz);
            }
        }
        // x axis on pairs: window pairs at even offsets are the loaded halves,
        // odd offsets are repacked once
        V4 sx, gx, rx, rho;
        {
            P2 ev[2 * NC], od[2 * NC - 1];
            YWindow<NC>::load(tu, ev, od);
            P2 sh[2], gh[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                sh[h] = mul2(w2[0], h ? u0.hi : u0.lo);
#pragma unroll
                for (int k = 1; k <= R; k++) {
                    const P2 a = YWindow<NC>::at(ev, od, HX + 2 * h + k);
                    const P2 b = YWindow<NC>::at(ev, od, HX + 2 * h - k);
                    sh[h] = fma2(w2[k], add2(a, b), sh[h]);
                    if (VD)
                        gh[h] = k == 1 ? mul2(w1[k], sub2(a, b)) : fma2(w1[k], sub2(a, b), gh[h]);
                }
            }
            sx = {sh[0], sh[1]};
            gx = {gh[0], gh[1]};
            if (VD) {
                YWindow<NC>::load(tr, ev, od);
                rho = {ev[HX / 2], ev[HX / 2 + 1]};
#pragma unroll
                for (int h = 0; h < 2; h++) {
#pragma unroll
                    for (int k = 1; k <= R; k++) {
                        const P2 a = YWindow<NC>::at(ev, od, HX + 2 * h + k);
                        const P2 b = YWindow<NC>::at(ev, od, HX + 2 * h - k);
                        gh[h] = k == 1 ? mul2(w1[k], sub2(a, b)) : fma2(w1[k], sub2(a, b), gh[h]);
                    }
                }
                rx = {gh[0], gh[1]};
            }
        }
        // reference order: x then z (constant_density/2d/wave.c:166)
        V4 lap = vfma(ihz, sz, vmul(ihx, sx));
        if (VD) {
            const P2 s1x = pk(W.s1[1], W.s1[1]), s1z = pk(W.s1[0], W.s1[0]);
            V4 cross = {mul2(s1x, mul2(gx.lo, rx.lo)), mul2(s1x, mul2(gx.hi, rx.hi))};
            cross = {fma2(s1z, mul2(gz.lo, rz.lo), cross.lo), fma2(s1z, mul2(gz.hi, rz.hi), cross.hi)};
            const float4 rr4 = to_f4(rho);
            const V4 inv = from_f4(make_float4(rcp_approx(rr4.x), rcp_approx(rr4.y),
                                               rcp_approx(rr4.z), rcp_approx(rr4.w)));
            lap = {fma2(sub2({0ull}, cross.lo), inv.lo, lap.lo),
                   fma2(sub2({0ull}, cross.hi), inv.hi, lap.hi)};
        }
        // a = 2 u - (1 - q) u_prev;  b = a / (1 + q);  u_next = b + C lap
        V4 av = {fma2(sub2(qq[j].lo, one), pv[j].lo, add2(u0.lo, u0.lo)),
                 fma2(sub2(qq[j].hi, one), pv[j].hi, add2(u0.hi, u0.hi))};
        if (!qzero[j]) {
            const float4 q4 = to_f4(qq[j]);
            const V4 rq = from_f4(make_float4(rcp_approx(1.f + q4.x), rcp_approx(1.f + q4.y),
                                              rcp_approx(1.f + q4.z), rcp_approx(1.f + q4.w)));
            av = {mul2(av.lo, rq.lo), mul2(av.hi, rq.hi)};
        }
        const V4 out = {fma2(lap.lo, cc[j].lo, av.lo), fma2(lap.hi, cc[j].hi, av.hi)};
        if (x + 3 < xlim) {
            *reinterpret_cast<ulonglong2*>(un + p) = make_ulonglong2(out.lo.v, out.hi.v);
        } else {
            const float4 o = to_f4(out);
            const float oa[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
            for (int v = 0; v < 4; v++)
                if (x + v < xlim) un[p + v] = oa[v];
        }
    }
}

extern __shared__ __align__(16) float4 sw_batch_smem[];

// A CTA per (shot, tile) of the tile list.
template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_batched(const Shot* __restrict__ shots, const TileRef* __restrict__ tiles) {
    const TileRef t = tiles[blockIdx.x];
    const Shot& S = shots[t.shot];
    if (!active(S)) return;
    float* un;
    const float *uc, *up;
    slot_ptrs(S, un, uc, up);
    const Layout L = S.L;
    stencil2d_tile<R, VD, TZ>(reinterpret_cast<float*>(sw_batch_smem), L, un, uc, up, S.C,
                              S.Q, S.den, S.W, S.zb, t.tz, t.tx);
}

// One shot: grid (x tiles, z tiles).
template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_single(Layout L, float* un, const float* __restrict__ uc, const float* up,
                 const float* __restrict__ C, const float* __restrict__ Q,
                 const float* __restrict__ den, Weights<float> W, ZeroBox2 zb) {
    stencil2d_tile<R, VD, TZ>(reinterpret_cast<float*>(sw_batch_smem), L, un, uc, up, C, Q,
                              den, W, zb.b, blockIdx.y, blockIdx.x);
}

// ---- batched sparse terms --------------------------------------------------------
__global__ void sources_batched(const Shot* __restrict__ shots,
                                const PairRef* __restrict__ pairs) {
    const PairRef pr = pairs[blockIdx.x];
    const Shot& S = shots[pr.shot];
    if (!active(S)) return;
    const size_t s = (size_t)pr.item;
    const float w = wavelet_at(S.wavelet, (size_t)S.wavelet_count, (size_t)S.n,
                               S.src.count, s);
    if (w == 0.f) return;
    float* un;
    const float *uc, *up;
    slot_ptrs(S, un, uc, up);
    inject_window<float, 2>(un, S.vel, S.damp, S.L, S.src.interval + s * 4,
                            S.src.values + S.src.offsets[s], w, S.dt, S.dt2,
                            threadIdx.x, blockDim.x);
}

// axis 1 (x edges) or 0 (z edges) of every shot; one block per shot
__global__ void edges_batched(const Shot* __restrict__ shots, int axis) {
    const Shot& S = shots[blockIdx.x];
    if (!active(S)) return;
    const int before = S.bc[2 * axis], after = S.bc[2 * axis + 1];
    if (!before && !after) return;
    float* un;
    const float *uc, *up;
    slot_ptrs(S, un, uc, up);
    const long long lines = boundary_lines(S.L, axis);
    for (long long t = threadIdx.x; t < lines; t += blockDim.x)
        boundary_line(un, S.L, axis, before, after, t);
}

__global__ void receivers_batched(const Shot* __restrict__ shots,
                                  const PairRef* __restrict__ pairs, int npairs) {
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= npairs) return;
    const PairRef pr = pairs[w];
    const Shot& S = shots[pr.shot];
    if (!active(S)) return;
    float* un;
    const float *uc, *up;
    slot_ptrs(S, un, uc, up);
    const size_t r = (size_t)pr.item;
    const float sum = gather_window<float, 2>(uc, S.L, S.rec.interval + r * 4,
                                              S.rec.values + S.rec.offsets[r], lane);
    if (lane == 0) S.receivers[(size_t)(S.n - 1) * S.rec.count + r] = sum;
}

__global__ void advance_batched(Shot* shots, int nshots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nshots && shots[s].n <= shots[s].end) shots[s].n++;
}

__global__ void swap_regions(float* __restrict__ a, float* __restrict__ b, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float t = a[i];
        a[i] = b[i];
        b[i] = t;
    }
}

// ---- host side -----------------------------------------------------------------

struct Failure {
    int code;
    std::string message;
};
[[noreturn]] static void fail(int code, const std::string& m) { throw Failure{code, m}; }
#define SB_CUDA(expr)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            ::sw::batch::fail(e_ == cudaErrorMemoryAllocation ? SIMWAVE_E_MEMORY          \
                                                              : SIMWAVE_E_CUDA,           \
                              std::string(#expr) + ": " + cudaGetErrorString(e_));        \
    } while (0)

struct HostShot {
    int id;
    Shot d;                  // descriptor (host copy; n tracked on the host too)
    float* cq = nullptr;     // engine-owned C and Q
    int* slots = nullptr;    // engine-owned schedule
    std::vector<int> perm;   // final logical -> physical slots
    long long grid = 0;      // elements of one pitched grid
    bool finished_restored = false;
};

template <int R, bool VD, int TZ>
static void set_smem_attr() {
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    cudaFuncSetAttribute(stencil2d_batched<R, VD, TZ>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(stencil2d_single<R, VD, TZ>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// configure (shared-memory size, outside any capture) or launch one group
template <int R, bool VD, int TZ>
static void launch_group_t(bool configure, const Shot* shots, const TileRef* tiles,
                           int ntiles, cudaStream_t st) {
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    if (configure) {
        set_smem_attr<R, VD, TZ>();
        return;
    }
    stencil2d_batched<R, VD, TZ><<<ntiles, kThreads, bytes, st>>>(shots, tiles);
}

template <int R, bool VD>
static void launch_group_r(bool configure, int tz, const Shot* shots, const TileRef* tiles,
                           int ntiles, cudaStream_t st) {
    if (tz == 8) launch_group_t<R, VD, 8>(configure, shots, tiles, ntiles, st);
    else if (tz == 32) launch_group_t<R, VD, 32>(configure, shots, tiles, ntiles, st);
    else launch_group_t<R, VD, 16>(configure, shots, tiles, ntiles, st);
}

static void launch_group(bool configure, int r, bool vd, int tz, const Shot* shots,
                         const TileRef* tiles, int ntiles, cudaStream_t st) {
#define SB_R(RR)                                                                          \
    case RR:                                                                              \
        if (vd) launch_group_r<RR, true>(configure, tz, shots, tiles, ntiles, st);        \
        else launch_group_r<RR, false>(configure, tz, shots, tiles, ntiles, st);          \
        break;
    switch (r) {
        SB_R(1) SB_R(2) SB_R(3) SB_R(4) SB_R(5) SB_R(6) SB_R(7) SB_R(8) SB_R(9) SB_R(10)
    }
#undef SB_R
}

// Single-shot tiled 2D stencil (16-row tiles) for the forward drivers.
template <int R, bool VD>
static void single_r(const Layout& L, float* un, const float* uc, const float* up,
                     const float* C, const float* Q, const float* den,
                     const Weights<float>& W, const int* box, cudaStream_t st) {
    constexpr int TZ = 16, HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (!configured[dev & 63]) {
        set_smem_attr<R, VD, TZ>();
        configured[dev & 63] = true;
    }
    dim3 grid((unsigned)((L.nx - 2 * R + 127) / 128), (unsigned)((L.nz - 2 * R + TZ - 1) / TZ));
    ZeroBox2 zb{{box[0], box[1], box[2], box[3]}};
    stencil2d_single<R, VD, TZ><<<grid, kThreads, bytes, st>>>(L, un, uc, up, C, Q, den, W, zb);
}

struct Engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<HostShot> shots;
    int next_id = 1;
    int tile_rows[kMaxRadius + 1];  // TZ per radius (tuning)
    // device tables (rebuilt when the shot set changes)
    Shot* d_shots = nullptr;
    size_t cap_shots = 0;
    TileRef* d_tiles = nullptr;
    size_t cap_tiles = 0;
    PairRef* d_src = nullptr;
    size_t cap_src = 0;
    PairRef* d_rec = nullptr;
    size_t cap_rec = 0;
    struct Group {
        int r;
        bool vd;
        int first, count;  // range in d_tiles
    };
    std::vector<Group> groups;
    int nsrc_pairs = 0, nrec_pairs = 0;
    bool dirty = true;
    // graph of `graph_steps` steps
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0;
    size_t kernel_launches = 0;

    Engine() {
        for (int r = 0; r <= kMaxRadius; r++) tile_rows[r] = 16;
    }

    template <typename P>
    void grow(P*& ptr, size_t& cap, size_t n) {
        if (n <= cap) return;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        SB_CUDA(cudaMalloc(&ptr, std::max<size_t>(n, 16) * sizeof(P)));
        cap = std::max<size_t>(n, 16);
    }

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        graph_steps = 0;
    }

    // rebuild the device tables from the host shots (descriptors keep the
    // host-tracked step counters, which equal the device ones between runs)
    void rebuild() {
        const size_t ns = shots.size();
        grow(d_shots, cap_shots, ns);
        std::vector<Shot> desc(ns);
        std::map<std::pair<int, int>, std::vector<TileRef>> byg;
        std::vector<PairRef> srcp, recp;
        for (size_t i = 0; i < ns; i++) {
            const HostShot& h = shots[i];
            desc[i] = h.d;
            const Layout& L = h.d.L;
            const int r = L.r;
            const int tz = tile_rows[r];
            const int nt_z = (int)((L.nz - 2 * r + tz - 1) / tz);
            const int nt_x = (int)((L.nx - 2 * r + 127) / 128);
            auto& v = byg[{r, h.d.den ? 1 : 0}];
            for (int a = 0; a < nt_z; a++)
                for (int b = 0; b < nt_x; b++) v.push_back({(int)i, a, b});
            for (size_t s = 0; s < h.d.src.count; s++) srcp.push_back({(int)i, (int)s});
            for (size_t s = 0; s < h.d.rec.count; s++) recp.push_back({(int)i, (int)s});
        }
        std::vector<TileRef> all;
        groups.clear();
        for (auto& kv : byg) {
            groups.push_back({kv.first.first, kv.first.second != 0, (int)all.size(),
                              (int)kv.second.size()});
            all.insert(all.end(), kv.second.begin(), kv.second.end());
        }
        grow(d_tiles, cap_tiles, all.size());
        grow(d_src, cap_src, srcp.size());
        grow(d_rec, cap_rec, recp.size());
        if (ns) SB_CUDA(cudaMemcpyAsync(d_shots, desc.data(), ns * sizeof(Shot),
                                        cudaMemcpyHostToDevice, stream));
        if (!all.empty())
            SB_CUDA(cudaMemcpyAsync(d_tiles, all.data(), all.size() * sizeof(TileRef),
                                    cudaMemcpyHostToDevice, stream));
        if (!srcp.empty())
            SB_CUDA(cudaMemcpyAsync(d_src, srcp.data(), srcp.size() * sizeof(PairRef),
                                    cudaMemcpyHostToDevice, stream));
        if (!recp.empty())
            SB_CUDA(cudaMemcpyAsync(d_rec, recp.data(), recp.size() * sizeof(PairRef),
                                    cudaMemcpyHostToDevice, stream));
        SB_CUDA(cudaStreamSynchronize(stream));
        nsrc_pairs = (int)srcp.size();
        nrec_pairs = (int)recp.size();
        for (const Group& g : groups)
            launch_group(true, g.r, g.vd, tile_rows[g.r], nullptr, nullptr, 0, stream);
        drop_graph();
        dirty = false;
    }

    // one step of every shot
    void enqueue_step(cudaStream_t st) {
        for (const Group& g : groups) {
            launch_group(false, g.r, g.vd, tile_rows[g.r], d_shots, d_tiles + g.first, g.count,
                         st);
            SB_CUDA(cudaGetLastError());
        }
        if (nsrc_pairs) sources_batched<<<nsrc_pairs, 128, 0, st>>>(d_shots, d_src);
        const int ns = (int)shots.size();
        edges_batched<<<ns, 256, 0, st>>>(d_shots, 1);
        edges_batched<<<ns, 256, 0, st>>>(d_shots, 0);
        if (nrec_pairs)
            receivers_batched<<<(nrec_pairs * 32 + 255) / 256, 256, 0, st>>>(d_shots, d_rec,
                                                                             nrec_pairs);
        advance_batched<<<(ns + 127) / 128, 128, 0, st>>>(d_shots, ns);
        SB_CUDA(cudaGetLastError());
    }

    void run(int steps, cudaStream_t user) {
        if (dirty) rebuild();
        if (shots.empty() || steps <= 0) return;
        // the longest remaining shot bounds the useful steps
        int most = 0;
        for (const HostShot& h : shots) most = std::max(most, h.d.end - h.d.n + 1);
        steps = std::min(steps, most);
        if (steps <= 0) return;
        const int K = 16;  // steps per graph
        if (!exec && steps >= K) {
            cudaGraph_t graph;
            SB_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                for (int k = 0; k < K; k++) enqueue_step(stream);
            } catch (...) {
                cudaStreamEndCapture(stream, &graph);
                throw;
            }
            SB_CUDA(cudaStreamEndCapture(stream, &graph));
            SB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            cudaGraphDestroy(graph);
            graph_steps = K;
        }
        // order the batch after the caller's prior work on `user`
        cudaEvent_t ev;
        SB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        SB_CUDA(cudaEventRecord(ev, user));
        SB_CUDA(cudaStreamWaitEvent(stream, ev, 0));
        int done = 0;
        const size_t per_step = groups.size() + (nsrc_pairs ? 1 : 0) + 3 + (nrec_pairs ? 1 : 0);
        while (steps - done >= K && exec) {
            SB_CUDA(cudaGraphLaunch(exec, stream));
            done += K;
            kernel_launches += K * per_step;
        }
        for (; done < steps; done++) {
            enqueue_step(stream);
            kernel_launches += per_step;
        }
        // the caller's stream waits for the batch
        SB_CUDA(cudaEventRecord(ev, stream));
        SB_CUDA(cudaStreamWaitEvent(user, ev, 0));
        SB_CUDA(cudaEventDestroy(ev));
        for (HostShot& h : shots) h.d.n = std::min(h.d.n + steps, h.d.end + 1);
    }
};

static std::mutex g_mutex;

static Engine* engine(simwave_batch* b) { return reinterpret_cast<Engine*>(b); }

// Validates a problem for the engine and builds its descriptor.
static void admit(Engine& E, const simwave_problem* P, int* id) {
    if (!P) fail(SIMWAVE_E_ARGUMENT, "null problem");
    if (P->dim != 2 || P->precision != 4)
        fail(SIMWAVE_E_ARGUMENT, "the batch engine takes 2D float32 shots");
    if (P->space_order < 2 || P->space_order > 20 || P->space_order % 2)
        fail(SIMWAVE_E_ARGUMENT, "space_order must be even in 2..20");
    const int r = P->space_order / 2;
    if (P->nz < (size_t)(2 * r + 1) || P->nx < (size_t)(2 * r + 1))
        fail(SIMWAVE_E_ARGUMENT, "every grid extent must be >= space_order + 1");
    if (P->pitch % 4 || (P->lead + r) % 4 || P->pitch < P->lead + P->nx)
        fail(SIMWAVE_E_ARGUMENT, "use simwave_layout() for the batch engine's grids");
    const bool vd = P->variable_density != 0;
    if (!P->u || !P->velocity || !P->damp || (vd && (!P->density || !P->coeff_order1)) ||
        !P->coeff_order2 || !P->boundary_conditions ||
        (P->num_receivers && !P->receivers) || (P->num_sources && !P->wavelet))
        fail(SIMWAVE_E_ARGUMENT, "null array argument");
    if (!(P->flags & SIMWAVE_FLAG_WINDOWS_CHECKED))
        fail(SIMWAVE_E_ARGUMENT, "validate the KWS windows and set SIMWAVE_FLAG_WINDOWS_CHECKED");
    for (int e = 0; e < 4; e++)
        if (P->boundary_conditions[e] > 2) fail(SIMWAVE_E_ARGUMENT, "boundary code must be 0..2");
    if (P->begin_timestep < 1 || P->end_timestep < P->begin_timestep || P->end_timestep > (1u << 30))
        fail(SIMWAVE_E_ARGUMENT, "invalid time range");
    if (P->num_sources) {
        const size_t need = P->wavelet_count > 1 ? P->end_timestep * P->num_sources
                                                 : P->end_timestep;
        if (P->wavelet_size * (P->wavelet_count ? P->wavelet_count : 1) < need)
            fail(SIMWAVE_E_ARGUMENT, "wavelet shorter than end_timestep");
    }
    const long long grid = (long long)P->nz * (long long)P->pitch;
    if (P->num_snapshots > 1 && P->slot_stride < (size_t)grid)
        fail(SIMWAVE_E_ARGUMENT, "slot_stride smaller than one grid");
    // slot schedule (the reference's bookkeeping; even-stride exchanges as
    // relabelling, undone when the shot is released)
    HostShot h;
    std::vector<int> table;
    std::vector<int> perm(P->num_snapshots);
    for (size_t i = 0; i < perm.size(); i++) perm[i] = (int)i;
    size_t prev = 0, cur = 1, next = 2;
    const size_t s = P->saving_stride, nsl = P->num_snapshots;
    for (size_t n = P->begin_timestep; n <= P->end_timestep; n++) {
        if (s == 0) {
            prev = (n - 1) % 3;
            cur = n % 3;
            next = (n + 1) % 3;
        } else if (s == 1) {
            prev = n - 1;
            cur = n;
            next = n + 1;
        }
        if (prev >= nsl || cur >= nsl || next >= nsl)
            fail(SIMWAVE_E_SCHEDULE, "the time range needs more wavefield slots");
        table.push_back(perm[prev]);
        table.push_back(perm[cur]);
        table.push_back(perm[next]);
        if (s > 1) {
            if (n % s == 1) {
                prev = cur;
                cur += 1;
                next += 1;
                if (s % 2 == 0 && n < P->end_timestep) {
                    std::swap(cur, next);
                    if (cur >= nsl || next >= nsl)
                        fail(SIMWAVE_E_SCHEDULE, "even-stride exchange needs more slots");
                    std::swap(perm[cur], perm[next]);
                }
            } else {
                prev = cur;
                cur = next;
                next = prev;
            }
        }
    }
    h.perm = perm;
    h.grid = grid;
    Shot& d = h.d;
    std::memset(&d, 0, sizeof(d));
    d.L.dim = 2;
    d.L.r = r;
    d.L.nz = (long long)P->nz;
    d.L.nx = (long long)P->nx;
    d.L.ny = 1;
    d.L.pitch = (long long)P->pitch;
    d.L.lead = (long long)P->lead;
    d.L.plane = d.L.pitch;
    d.L.slot = (long long)P->slot_stride;
    d.u = (float*)P->u;
    d.vel = (const float*)P->velocity;
    d.damp = (const float*)P->damp;
    d.den = vd ? (const float*)P->density : nullptr;
    d.W = make_weights<float>((const float*)P->coeff_order2,
                              vd ? (const float*)P->coeff_order1 : nullptr, r, P->dz,
                              P->dx, 1.0);
    d.src = Windows<float>{P->src_points_interval, (const float*)P->src_points_values,
                           P->src_points_values_offset, P->num_sources};
    d.rec = Windows<float>{P->rec_points_interval, (const float*)P->rec_points_values,
                           P->rec_points_values_offset, P->num_receivers};
    d.wavelet = (const float*)P->wavelet;
    d.wavelet_count = P->wavelet_count;
    d.receivers = (float*)P->receivers;
    d.dt = (float)P->dt;
    d.dt2 = d.dt * d.dt;
    d.begin = (int)P->begin_timestep;
    d.end = (int)P->end_timestep;
    d.n = d.begin;
    for (int e = 0; e < 4; e++) d.bc[e] = (int)P->boundary_conditions[e];
    // engine-owned: coefficients and schedule
    SB_CUDA(cudaMalloc(&h.cq, 2 * (size_t)grid * sizeof(float)));
    SB_CUDA(cudaMalloc(&h.slots, table.size() * sizeof(int)));
    SB_CUDA(cudaMemcpyAsync(h.slots, table.data(), table.size() * sizeof(int),
                            cudaMemcpyHostToDevice, E.stream));
    form_coefficients(d.vel, d.damp, h.cq, h.cq + grid, grid, d.dt, E.stream);
    SB_CUDA(cudaGetLastError());
    // box where Q is zero (its loads are skipped there)
    int* words = nullptr;
    SB_CUDA(cudaMalloc(&words, 8 * sizeof(int)));
    find_zero_box(h.cq + grid, d.L, words, E.stream);
    int box[7];
    const cudaError_t copied =
        cudaMemcpyAsync(box, words, sizeof(box), cudaMemcpyDeviceToHost, E.stream);
    const cudaError_t synced = cudaStreamSynchronize(E.stream);
    cudaFree(words);
    SB_CUDA(copied);
    SB_CUDA(synced);
    const bool good = box[6] == 0 && box[1] > box[0] && box[3] > box[2];
    for (int i = 0; i < 4; i++) d.zb[i] = good ? box[i] : 0;
    d.C = h.cq;
    d.Q = h.cq + grid;
    d.slots = h.slots;
    h.id = E.next_id++;
    *id = h.id;
    E.shots.push_back(h);
    E.dirty = true;
}

static void release(Engine& E, size_t i, bool restore) {
    HostShot& h = E.shots[i];
    if (restore) {
        // logical slot j ends in slot j, as in the reference
        const int nsl = (int)h.perm.size();
        std::vector<int> at(nsl), where(nsl);
        for (int j = 0; j < nsl; j++) {
            at[h.perm[j]] = j;
            where[j] = h.perm[j];
        }
        for (int j = 0; j < nsl; j++) {
            const int p = where[j];
            if (p == j) continue;
            swap_regions<<<256, 256, 0, E.stream>>>(h.d.u + (long long)j * h.d.L.slot,
                                                    h.d.u + (long long)p * h.d.L.slot, h.grid);
            const int other = at[j];
            at[p] = other;
            where[other] = p;
            at[j] = j;
            where[j] = j;
        }
        SB_CUDA(cudaGetLastError());
    }
    SB_CUDA(cudaStreamSynchronize(E.stream));
    cudaFree(h.cq);
    cudaFree(h.slots);
    E.shots.erase(E.shots.begin() + (long)i);
    E.dirty = true;
}

template <typename F>
static int guarded(F&& f) {
    try {
        record_error("");
        f();
        return SIMWAVE_OK;
    } catch (const Failure& e) {
        record_error(e.message);
        return e.code;
    } catch (const std::exception& e) {
        record_error(e.what());
        return SIMWAVE_E_ARGUMENT;
    }
}

// ---- persistent 2D forward: every step of one shot in one launch ----------
//
// Small 2D grids are bound by the start-up and drain of the six short
// kernels of each step, not by their work (a 513^2 order-4 shot spends
// about 20 us per step either way, with or without graph launches). One
// cooperative launch runs all steps instead: per step, the tiles of the
// stencil and the receiver gathers, then the sources, then the x and z
// boundary phases, each phase separated by a grid barrier. The barrier
// spins with a time limit: on expiry the block records SIMWAVE_E_TIMEOUT and
// the kernel ends (blocks still inside a barrier time out the same way).

struct Persist2D : Shot2D {
    float* u;                 // slot 0
    const int* slots;         // per step: next, cur, prev physical slots
    int steps;
    long long begin;
    unsigned* bar;            // [0] arrivals, [1] generation (zeroed before launch)
    int* err;
};

// Owner-computes part of a step for tile (tz, tx), after its stencil: the
// source points in the tile (points of the halo belong to the nearest edge
// tile), then the x edges of its rows if it is an x-edge tile, then the z
// edges of its columns if it is a z-edge tile. Exact when the first and last
// tiles hold at least r + 1 rows and columns (Shot2D::fused): every boundary
// operation then reads and writes points of one tile only, in the
// reference's order.
__device__ void tile_sources_edges(const Shot2D& P, float* un, long long n, int tz, int tx) {
    const Layout& L = P.L;
    const int r = L.r;
    const int nz = (int)L.nz, nx = (int)L.nx;
    const int z_lo = tz == 0 ? 0 : r + 16 * tz;
    const int z_hi = tz == P.tiles_z - 1 ? nz : r + 16 * (tz + 1);
    const int x_lo = tx == 0 ? 0 : r + 128 * tx;
    const int x_hi = tx == P.tiles_x - 1 ? nx : r + 128 * (tx + 1);
    const float dt2 = P.dt * P.dt;
    for (size_t s = 0; s < P.src.count; s++) {
        const float w = wavelet_at(P.wavelet, P.wavelet_count, (size_t)n, P.src.count, s);
        if (w == 0.f) continue;
        const size_t* b = P.src.interval + s * 4;
        if ((int)b[1] < z_lo || (int)b[0] >= z_hi || (int)b[3] < x_lo || (int)b[2] >= x_hi)
            continue;
        const float* v = P.src.values + P.src.offsets[s];
        const long long total = window_size<2>(b);
        for (long long t = threadIdx.x; t < total; t += blockDim.x) {
            long long iz, ix, iy;
            window_point<2>(b, t, iz, ix, iy);
            const int z = (int)(b[0] + iz), x = (int)(b[2] + ix);
            if (z < z_lo || z >= z_hi || x < x_lo || x >= x_hi) continue;
            const float kws = window_weight<float, 2>(b, v, iz, ix, iy);
            const long long p = L.at2(z, x);
            const float vv = P.vel[p] * P.vel[p];
            const float d = 1.f + P.damp[p] * P.dt * vv * 0.5f;
            atomicAdd(un + p, dt2 * vv * kws * w / d);
        }
    }
    __syncthreads();
    // x edges (rows of this tile), then z edges (columns of this tile)
    const int bx0 = P.bc[2], bx1 = P.bc[3], bz0 = P.bc[0], bz1 = P.bc[1];
    if ((bx0 && tx == 0) || (bx1 && tx == P.tiles_x - 1)) {
        const int r0 = max(z_lo, r), r1 = min(z_hi, nz - r);
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            if (tx == 0) apply_edge(un, L.at2(i, r), 1, r, bx0, -1);
            if (tx == P.tiles_x - 1) apply_edge(un, L.at2(i, nx - r - 1), 1, r, bx1, +1);
        }
    }
    __syncthreads();
    if ((bz0 && tz == 0) || (bz1 && tz == P.tiles_z - 1)) {
        const int c0 = max(x_lo, r), c1 = min(x_hi, nx - r);
        for (int j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
            if (tz == 0) apply_edge(un, L.at2(r, j), L.pitch, r, bz0, -1);
            if (tz == P.tiles_z - 1) apply_edge(un, L.at2(nz - r - 1, j), L.pitch, r, bz1, +1);
        }
    }
    __syncthreads();
}

constexpr long long kBarrierCycles = 4000000000LL;  // ~2 s at 2 GHz

// Grid-wide barrier of the cooperative launch; false when the wait expired
// (then the error word is set). Every block calls it the same number of
// times; the generation is read before arriving so a flip is never missed.
__device__ bool grid_barrier(unsigned* bar, int* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == g) {
                if (clock64() - t0 > kBarrierCycles || *(volatile int*)err) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (!ok) atomicCAS(err, 0, SIMWAVE_E_TIMEOUT);
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_persistent(const Persist2D P) {
    const Layout L = P.L;
    float* tile = reinterpret_cast<float*>(sw_batch_smem);
    const long long gthreads = (long long)gridDim.x * blockDim.x;
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const float dt2 = P.dt * P.dt;
    for (int i = 0; i < P.steps; i++) {
        const long long n = P.begin + i;
        float* un = P.u + (long long)P.slots[3 * i] * L.slot;
        const float* uc = P.u + (long long)P.slots[3 * i + 1] * L.slot;
        const float* up = P.u + (long long)P.slots[3 * i + 2] * L.slot;
        // stencil tiles, then the receivers (they read u_cur only)
        for (int t = blockIdx.x; t < P.ntiles; t += gridDim.x) {
            stencil2d_tile<R, VD, TZ>(tile, L, un, uc, up, P.C, P.Q, P.den, P.W, P.zb,
                                      t / P.tiles_x, t % P.tiles_x);
            __syncthreads();  // the tile buffer is restaged next
            if (P.fused) tile_sources_edges(P, un, n, t / P.tiles_x, t % P.tiles_x);
        }
        if (P.rec.count) {
            float* row = P.receivers + (n - 1) * (long long)P.rec.count;
            for (long long w = gtid >> 5; w < (long long)P.rec.count; w += gthreads >> 5) {
                const float sum = gather_window<float, 2>(
                    uc, L, P.rec.interval + w * 4, P.rec.values + P.rec.offsets[w], lane);
                if (lane == 0) row[w] = sum;
            }
        }
        if (!grid_barrier(P.bar, P.err)) return;
        if (P.fused) continue;  // sources and edges were applied per tile
        if (P.src.count) {
            for (size_t sidx = blockIdx.x; sidx < P.src.count; sidx += gridDim.x) {
                const float w = wavelet_at(P.wavelet, P.wavelet_count, (size_t)n, P.src.count,
                                           sidx);
                if (w != 0.f)
                    inject_window<float, 2>(un, P.vel, P.damp, L,
                                            P.src.interval + sidx * 4,
                                            P.src.values + P.src.offsets[sidx], w, P.dt, dt2,
                                            threadIdx.x, blockDim.x);
            }
            if (!grid_barrier(P.bar, P.err)) return;
        }
        // boundary phases in the reference's order: x edges, then z edges
        for (int a = 1; a >= 0; a--) {
            const int b0 = P.bc[2 * a], b1 = P.bc[2 * a + 1];
            if (!b0 && !b1) continue;
            const long long lines = boundary_lines(L, a);
            for (long long t = gtid; t < lines; t += gthreads) boundary_line(un, L, a, b0, b1, t);
            if (!grid_barrier(P.bar, P.err)) return;
        }
    }
}

// One time step of a 2D shot in one launch: blocks [0, ntiles) compute a
// tile each (stencil, then the sources and boundary edges the tile owns),
// the blocks after them gather the receivers (they read u_cur only).
template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_step(const Shot2D P, float* un, const float* uc, const float* up, long long n) {
    if ((int)blockIdx.x < P.ntiles) {
        const int t = blockIdx.x;
        stencil2d_tile<R, VD, TZ>(reinterpret_cast<float*>(sw_batch_smem), P.L, un, uc, up, P.C,
                                  P.Q, P.den, P.W, P.zb, t / P.tiles_x, t % P.tiles_x);
        __syncthreads();
        tile_sources_edges(P, un, n, t / P.tiles_x, t % P.tiles_x);
        return;
    }
    const long long w = ((long long)(blockIdx.x - P.ntiles) * blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)P.rec.count) return;
    const float sum = gather_window<float, 2>(uc, P.L, P.rec.interval + w * 4,
                                              P.rec.values + P.rec.offsets[w], threadIdx.x & 31);
    if ((threadIdx.x & 31) == 0) P.receivers[(n - 1) * (long long)P.rec.count + w] = sum;
}

template <int R, bool VD>
static void step_r(const Shot2D& P, float* un, const float* uc, const float* up, long long n,
                   cudaStream_t st) {
    constexpr int TZ = 16;
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    static bool configured[64] = {};
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        SB_CUDA(cudaFuncSetAttribute(stencil2d_step<R, VD, TZ>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        configured[dev & 63] = true;
    }
    const int rec_blocks = (int)((P.rec.count + kWarps - 1) / kWarps);
    stencil2d_step<R, VD, TZ><<<P.ntiles + rec_blocks, kThreads, bytes, st>>>(P, un, uc, up, n);
}

template <int R, bool VD>
static bool persistent_r(const Persist2D& P, cudaStream_t st) {
    constexpr int TZ = 16;
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    auto kernel = stencil2d_persistent<R, VD, TZ>;
    static bool configured[64] = {};
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     bytes));
        configured[dev & 63] = true;
    }
    int coop = 0, sms = 0, per_sm = 0;
    SB_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    SB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, bytes));
    if (!coop || per_sm < 1) return false;
    Persist2D A = P;
    const int grid = std::max(1, std::min(P.ntiles, per_sm * sms));
    void* args[] = {&A};
    SB_CUDA(cudaMemsetAsync(P.bar, 0, 2 * sizeof(unsigned), st));
    SB_CUDA(cudaLaunchCooperativeKernel((const void*)kernel, dim3(grid), dim3(kThreads), args,
                                        (size_t)bytes, st));
    return true;
}

}  // namespace batch

bool shot2d_prepare(Shot2D& S, const Layout& L, const float* C, const float* Q,
                    const float* den, const float* vel, const float* damp,
                    const Weights<float>& W, const int* zero_box, const Windows<float>& src,
                    const float* wavelet, size_t wavelet_count, float dt,
                    const Windows<float>& rec, float* receivers, const int* bc) {
    if (!tiled2d_supported(L)) return false;
    S.L = L;
    S.C = C;
    S.Q = Q;
    S.den = den;
    S.vel = vel;
    S.damp = damp;
    S.W = W;
    for (int i = 0; i < 4; i++) S.zb[i] = zero_box[i];
    S.src = src;
    S.wavelet = wavelet;
    S.wavelet_count = wavelet_count;
    S.dt = dt;
    S.rec = rec;
    S.receivers = receivers;
    for (int e = 0; e < 4; e++) S.bc[e] = bc[e];
    const int r = L.r;
    S.tiles_x = (int)((L.nx - 2 * r + 127) / 128);
    S.tiles_z = (int)((L.nz - 2 * r + 15) / 16);
    S.ntiles = S.tiles_x * S.tiles_z;
    // owner-computes sources and edges need r + 1 rows / columns in the first
    // and last tiles (the first hold min(extent, 16 or 128))
    const long long last_z = (L.nz - 2 * r) - 16LL * (S.tiles_z - 1);
    const long long last_x = (L.nx - 2 * r) - 128LL * (S.tiles_x - 1);
    const long long first_z = std::min<long long>(L.nz - 2 * r, 16);
    const long long first_x = std::min<long long>(L.nx - 2 * r, 128);
    S.fused = last_z >= r + 1 && last_x >= r + 1 && first_z >= r + 1 && first_x >= r + 1;
    return true;
}

void step2d_launch(const Shot2D& S, bool vd, float* un, const float* uc, const float* up,
                   long long n, cudaStream_t st) {
#define SB_ST(RR)                                                               \
    case RR:                                                                    \
        if (vd) batch::step_r<RR, true>(S, un, uc, up, n, st);                  \
        else batch::step_r<RR, false>(S, un, uc, up, n, st);                    \
        break;
    switch (S.L.r) {
        SB_ST(1) SB_ST(2) SB_ST(3) SB_ST(4) SB_ST(5) SB_ST(6) SB_ST(7) SB_ST(8) SB_ST(9) SB_ST(10)
    }
#undef SB_ST
}

bool persistent2d_launch(const Shot2D& S, bool vd, float* u, const int* slots, int steps,
                         long long begin, unsigned* bar, int* err, cudaStream_t st) {
    if (steps < 1) return false;
    batch::Persist2D P;
    static_cast<Shot2D&>(P) = S;
    P.u = u;
    P.slots = slots;
    P.steps = steps;
    P.begin = begin;
    P.bar = bar;
    P.err = err;
#define SB_P(RR)                                                                    \
    case RR:                                                                        \
        return vd ? batch::persistent_r<RR, true>(P, st) : batch::persistent_r<RR, false>(P, st);
    switch (S.L.r) {
        SB_P(1) SB_P(2) SB_P(3) SB_P(4) SB_P(5) SB_P(6) SB_P(7) SB_P(8) SB_P(9) SB_P(10)
    }
#undef SB_P
    return false;
}

bool tiled2d_supported(const Layout& L) {
    return L.dim == 2 && L.r >= 1 && L.r <= kMaxRadius && L.pitch % 4 == 0 &&
           (L.lead + L.r) % 4 == 0 && L.pitch >= L.lead + L.nx && L.nz * L.pitch < (1LL << 31);
}

void tiled2d_launch(const Layout& L, bool vd, float* un, const float* uc, const float* up,
                    const float* C, const float* Q, const float* den,
                    const Weights<float>& W, const int* zero_box, cudaStream_t st) {
#define SB_S(RR)                                                                          \
    case RR:                                                                              \
        if (vd) batch::single_r<RR, true>(L, un, uc, up, C, Q, den, W, zero_box, st);    \
        else batch::single_r<RR, false>(L, un, uc, up, C, Q, den, W, zero_box, st);      \
        break;
    switch (L.r) {
        SB_S(1) SB_S(2) SB_S(3) SB_S(4) SB_S(5) SB_S(6) SB_S(7) SB_S(8) SB_S(9) SB_S(10)
    }
#undef SB_S
}

}  // namespace sw

using sw::batch::Engine;

extern "C" int simwave_batch_create(simwave_batch** out) {
    return sw::batch::guarded([&] {
        if (!out) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null handle pointer");
        Engine* e = new Engine();
        SB_CUDA(cudaGetDevice(&e->device));
        SB_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        *out = reinterpret_cast<simwave_batch*>(e);
    });
}

extern "C" int simwave_batch_destroy(simwave_batch* b) {
    return sw::batch::guarded([&] {
        if (!b) return;
        Engine* e = sw::batch::engine(b);
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        while (!e->shots.empty()) sw::batch::release(*e, e->shots.size() - 1, false);
        e->drop_graph();
        cudaFree(e->d_shots);
        cudaFree(e->d_tiles);
        cudaFree(e->d_src);
        cudaFree(e->d_rec);
        cudaStreamDestroy(e->stream);
        delete e;
    });
}

extern "C" int simwave_batch_add(simwave_batch* b, const simwave_problem* problem, int* shot_id) {
    return sw::batch::guarded([&] {
        if (!b || !shot_id) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null argument");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        sw::batch::admit(*sw::batch::engine(b), problem, shot_id);
    });
}

extern "C" int simwave_batch_run(simwave_batch* b, int steps, void* stream) {
    return sw::batch::guarded([&] {
        if (!b) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null handle");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        sw::batch::engine(b)->run(steps, (cudaStream_t)stream);
    });
}

extern "C" int simwave_batch_remaining(simwave_batch* b, int shot_id, int* steps) {
    return sw::batch::guarded([&] {
        if (!b || !steps) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null argument");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        for (const auto& h : sw::batch::engine(b)->shots)
            if (h.id == shot_id) {
                *steps = h.d.end - h.d.n + 1;
                return;
            }
        sw::batch::fail(SIMWAVE_E_ARGUMENT, "unknown shot id");
    });
}

extern "C" int simwave_batch_release(simwave_batch* b, int shot_id) {
    return sw::batch::guarded([&] {
        if (!b) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null handle");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        Engine* e = sw::batch::engine(b);
        for (size_t i = 0; i < e->shots.size(); i++)
            if (e->shots[i].id == shot_id) {
                const bool done = e->shots[i].d.n > e->shots[i].d.end;
                sw::batch::release(*e, i, done);
                return;
            }
        sw::batch::fail(SIMWAVE_E_ARGUMENT, "unknown shot id");
    });
}

extern "C" int simwave_batch_set_tile_rows(simwave_batch* b, int space_order, int rows) {
    return sw::batch::guarded([&] {
        if (!b || space_order < 2 || space_order > 20 || space_order % 2 ||
            (rows != 8 && rows != 16 && rows != 32))
            sw::batch::fail(SIMWAVE_E_ARGUMENT, "space_order even in 2..20, rows 8, 16 or 32");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        Engine* e = sw::batch::engine(b);
        e->tile_rows[space_order / 2] = rows;
        e->dirty = true;
    });
}

extern "C" int simwave_batch_launches(simwave_batch* b, size_t* launches) {
    return sw::batch::guarded([&] {
        if (!b || !launches) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null argument");
        *launches = sw::batch::engine(b)->kernel_launches;
    });
}
