// sw_batch.cu -- many independent 2D shots advanced together.
//
// A shot is one forward problem (2D, float32, any order, density and saving
// stride) whose arrays are resident on the device (the caller owns u, the
// models, the KWS tables, the wavelet and the receivers; the engine owns the
// per-point coefficients C, Q and the shot's slot schedule). Each launch
// round of the batch is a fixed sequence of launches over *all* shots:
//   1. stencil   one launch per (radius, density, depth) group; a CTA is one
//                128 x TZ tile of one shot (tile list in device memory), or,
//                for time-blocked groups, one tile advanced `depth` steps
//                with its sources, edges and receiver copies
//   2. sources   one block per (shot, source)            } per-step shots
//   3. x edges, then z edges (the reference's order)     } only
//   4. receivers one warp per (shot, receiver); the time-blocked shots'
//                records are summed from their window copies
//   5. advance   each shot's step counter (by 1 or by its block)
// Every kernel reads the shot's current step and the run's stop step from
// its device descriptor and does nothing for a shot past them, so the
// sequence of 16 rounds is captured once into a CUDA graph and replayed
// until the set of shots changes (shots that finish simply go idle).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <string>
#include <vector>

#include "simwave_gb300.h"
#include "sw_kernels.cuh"
#include "sw_pairs.cuh"
#include "sw_tile2d.cuh"
#include "sw_tiled.h"

namespace sw {

void record_error(const std::string& message);

namespace batch {


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
    int stop;              // last step of the current run (<= end)
    int depth;             // steps per launch: 1 per-step kernels, > 1 time-blocked
    const unsigned char* keep;  // per step: its level is the last one written to its slot
    float* partial;        // time-blocked receivers: [rec][depth][win] window values
    int win;               // floats per receiver window in `partial`
    int halo_zero;         // every slot's halo is zero (no reloads needed)
    // time-blocked shots carry their latest two levels in two engine-owned
    // pairs of grids, [pair][prev, cur] (`grid` floats each): a launch
    // stages from pair *pairp and leaves its last two levels in the other,
    // so no tile reads a grid another tile of the launch writes
    float* ext;
    int* pairp;
    long long grid;
    int bc[4];
    int zb[4];             // z0, z1, x0, x1: box where Q is zero
};

struct ZeroBox2 {
    int b[4];
};

struct TileRef {
    int shot, tz, tx;
    int rec_first, rec_count;  // time-blocked tiles: their receiver-window parts
    int src_first, src_count;  // time-blocked tiles: sources whose window meets the region
};
struct PairRef {
    int shot, item;
};

__device__ __forceinline__ bool active(const Shot& s) { return s.n <= s.stop; }

// ---- time-blocked tiles ----------------------------------------------------------
// A time-blocked CTA owns OZ x OX interior points (plus the halo beyond them
// on the grid's edges) and stages a region of kTbRows rows around them: K R
// rows above and below, and 128 computed columns plus an HX halo, of which
// DX on each side are recomputed margin. After step k of the block the
// region's rows are exact k R rows further in and its computed columns
// (k - 1) R columns further in, so after K steps the owned points are.
constexpr int kTbRows = 104;

struct TbGeom {
    int mz, oz, dx, ox;
};

// Part of one receiver window inside one time-blocked tile's owned points.
struct TbRec {
    int rc;              // receiver
    int z0, z1, x0, x1;  // the part (grid indices, half-open)
    int b0, b2, lx;      // window origin and row length
};

__host__ __device__ constexpr TbGeom tb_geom(int r, int k) {
    // the staged HX columns beyond the 128 computed ones serve the first
    // step only, so k - 1 further steps eat (k - 1) r computed columns a side
    const int dx = ((k - 1) * r + 3) & ~3;
    return TbGeom{k * r, kTbRows - 2 * k * r, dx, 128 - 2 * dx};
}

__host__ __device__ constexpr bool tb_supported(int r, int k) {
    const TbGeom g = tb_geom(r, k);
    return k >= 2 && k <= 4 && g.oz >= 32 && g.ox >= 64;
}

__host__ __device__ __forceinline__ int tb_tiles(long long interior, int o) {
    return (int)((interior + o - 1) / o);
}

// Owned tile along an axis of n points (radius r, o owned points a tile).
__host__ __device__ __forceinline__ int tb_tile_of(long long p, int r, long long n, int o) {
    const int t = tb_tiles(n - 2 * r, o);
    if (p < r) return 0;
    const long long q = (p - r) / o;
    return (int)(q < t - 1 ? q : t - 1);
}

__device__ __forceinline__ void slot_ptrs(const Shot& s, float*& un, const float*& uc,
                                          const float*& up) {
    const int* sl = s.slots + 3 * (s.n - s.begin);
    up = s.u + (long long)sl[0] * s.L.slot;
    uc = s.u + (long long)sl[1] * s.L.slot;
    un = s.u + (long long)sl[2] * s.L.slot;
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

constexpr int kRing = 64;  // rows in the streamed stencil's ring

// 16-byte asynchronous copy global -> shared (zero-filled when !ok).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool ok) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src),
                 "r"(ok ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// ---- streamed 2D stencil (tall tiles) ----------------------------------------------
// A CTA owns 128 interior columns (a strip) of CH consecutive interior rows
// and streams down them: rows of u (and rho) with an HX column halo arrive
// by cp.async in a shared-memory ring of kRing = 64 rows (a power of two at
// least 2R + 2G, so a row's slot is one AND; G = 8 RW rows a group, RW rows
// per warp), one group ahead of the rows being computed, so each row is
// staged once per strip (plus the 2R rows where chunks meet) instead of
// once per overlapping 16-row tile. A warp computes two consecutive rows of
// a group, so they share their z neighbours (2R + 2 ring loads for the
// pair). Per group: a CTA barrier (the
// ring slots of the next group are free), the copies of the next group's
// rows, a wait for the current group's, a barrier, then each warp computes
// RW rows with the per-point arithmetic of stencil2d_tile, so the results
// are bit-identical to the staged tiles'.
template <int R, bool VD, int CH, int RW>
__device__ __forceinline__ void stencil2d_stream_body(float* ring, const Layout& L, float* un,
                                                      const float* uc, const float* up,
                                                      const float* C, const float* Q,
                                                      const float* den, const Weights<float>& W,
                                                      const int* zb, int tz, int tx) {
    constexpr int HX = (R + 3) & ~3;
    constexpr int TW = 128 + 2 * HX;
    constexpr int G = kWarps * RW;   // rows per group
    constexpr int NR = kRing;        // ring rows
    static_assert(2 * R + 2 * G <= NR && (NR & (NR - 1)) == 0, "ring size");
    constexpr int NC = (4 + 2 * HX) / 4;
    constexpr int CHK = TW / 4;  // 16-byte chunks per row
    static_assert(CH % G == 0, "chunk height");
    const int zbeg = R + tz * CH;
    const int zend = min(zbeg + CH, (int)L.nz - R);
    const int x0 = R + tx * 128;
    const int col0 = (int)L.lead + x0 - HX;
    const int pitch = (int)L.pitch;
    const int nz = (int)L.nz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = x0 + 4 * lane;
    const int xlim = (int)L.nx - R;
    const bool xbox = x >= zb[2] && x + 3 < zb[3];
    const int zlast = zend - 1 + R;  // last row any group needs
    float* rr = ring + (VD ? NR * TW : 0);  // density ring

    // rows [a, b) (clipped to zlast) into their ring slots, one commit group
    auto stage = [&](int a, int b) {
        b = min(b, zlast + 1);
        const int n = (b - a) * CHK;
        for (int i = threadIdx.x; i < n; i += kThreads) {
            const int row = a + i / CHK, ch = i - (i / CHK) * CHK;
            const int col = col0 + 4 * ch;
            const bool ok = row < nz && col + 3 < pitch;
            const long long o = ok ? (long long)row * pitch + col : 0;
            const int s = (int)((unsigned)row & (NR - 1)) * TW + 4 * ch;
            cp_async16(ring + s, uc + o, ok);
            if (VD) cp_async16(rr + s, den + o, ok);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    P2 w2[R + 1], w1[R + 1];
#pragma unroll
    for (int k = 0; k <= R; k++) {
        w2[k] = pk(W.c2[k], W.c2[k]);
        w1[k] = pk(W.c1[k], W.c1[k]);
    }
    const P2 ihx = pk(W.ih2[1], W.ih2[1]), ihz = pk(W.ih2[0], W.ih2[0]);
    const P2 one = pk(1.f, 1.f);

    auto row = [&](int zz) { return ring + (int)((unsigned)zz & (NR - 1)) * TW + 4 * lane; };
    auto rrow = [&](int zz) { return rr + (int)((unsigned)zz & (NR - 1)) * TW + 4 * lane; };
    // x axis, combine, update and store of row z from its z sums; tu / tr:
    // the row's lane window in the u / density ring
    auto finish = [&](int z, const float* tu, const float* tr, V4 u0, V4 sz, V4 gz, V4 rz, V4 cc,
                      V4 pv, V4 qq, bool qzero) {
        const long long p = (long long)z * pitch + L.lead + x;
        // x axis on pairs
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
            cross = {fma2(s1z, mul2(gz.lo, rz.lo), cross.lo),
                     fma2(s1z, mul2(gz.hi, rz.hi), cross.hi)};
            const float4 rr4 = to_f4(rho);
            const V4 inv = from_f4(make_float4(rcp_approx(rr4.x), rcp_approx(rr4.y),
                                               rcp_approx(rr4.z), rcp_approx(rr4.w)));
            lap = {fma2(sub2({0ull}, cross.lo), inv.lo, lap.lo),
                   fma2(sub2({0ull}, cross.hi), inv.hi, lap.hi)};
        }
        // a = 2 u - (1 - q) u_prev;  b = a / (1 + q);  u_next = b + C lap
        V4 av = {fma2(sub2(qq.lo, one), pv.lo, add2(u0.lo, u0.lo)),
                 fma2(sub2(qq.hi, one), pv.hi, add2(u0.hi, u0.hi))};
        if (!qzero) {
            const float4 q4 = to_f4(qq);
            const V4 rq = from_f4(make_float4(rcp_approx(1.f + q4.x), rcp_approx(1.f + q4.y),
                                              rcp_approx(1.f + q4.z), rcp_approx(1.f + q4.w)));
            av = {mul2(av.lo, rq.lo), mul2(av.hi, rq.hi)};
        }
        const V4 out = {fma2(lap.lo, cc.lo, av.lo), fma2(lap.hi, cc.hi, av.hi)};
        if (x + 3 < xlim) {
            *reinterpret_cast<ulonglong2*>(un + p) = make_ulonglong2(out.lo.v, out.hi.v);
        } else {
            const float4 o = to_f4(out);
            const float oa[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
            for (int v = 0; v < 4; v++)
                if (x + v < xlim) un[p + v] = oa[v];
        }
    };
    // per-point operands of row z
    auto fetch = [&](int z, V4& cc, V4& pv, V4& qq, bool& qz) {
        const bool ok = z < zend && x < xlim;
        const long long p = (long long)z * pitch + L.lead + x;
        qz = xbox && z >= zb[0] && z < zb[1];
        cc = ldg_v4(C + p, ok);
        pv = ld_v4(up + p, ok);
        qq = ldg_v4(Q + p, ok && !qz);
    };

    stage(zbeg - R, zbeg + G + R);
    for (int zr = zbeg; zr < zend; zr += G) {
        // this warp's rows: za and za + 1, sharing their z neighbours
        const int za = zr + 2 * warp;
        V4 cca, pva, qqa, ccb, pvb, qqb;
        bool qza, qzb;
        fetch(za, cca, pva, qqa, qza);
        fetch(za + 1, ccb, pvb, qqb, qzb);
        __syncthreads();  // the previous group's rows are read: their slots are free
        stage(zr + G + R, zr + 2 * G + R);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();  // every thread's copies of this group's rows have landed
        if (za >= zend || x >= xlim) continue;
        // z axis of both rows: at step k row za takes rows za + k and za - k,
        // row za + 1 takes za + 1 + k and za + 1 - k; za + k and za + 1 - k
        // were loaded at step k - 1 (the same sums as per row). at(j) / rat(j):
        // row za + j of the u / density ring (+ HX)
        V4 ua, ub, sza, szb, gza, gzb, rza, rzb;
        auto zsums = [&](auto at, auto rat) {
            ua = lds_v4(at(0));
            ub = lds_v4(at(1));
            sza = vmul(w2[0], ua);
            szb = vmul(w2[0], ub);
            V4 am = ua, bp = ub;
            V4 ram, rbp;
            if (VD) {
                ram = lds_v4(rat(0));
                rbp = lds_v4(rat(1));
            }
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const V4 Ap = bp, Bm = am;
                const V4 Am = lds_v4(at(-k)), Bp = lds_v4(at(1 + k));
                sza = vfma(w2[k], vadd(Ap, Am), sza);
                szb = vfma(w2[k], vadd(Bp, Bm), szb);
                if (VD) {
                    gza = k == 1 ? vmul(w1[k], vsub(Ap, Am)) : vfma(w1[k], vsub(Ap, Am), gza);
                    gzb = k == 1 ? vmul(w1[k], vsub(Bp, Bm)) : vfma(w1[k], vsub(Bp, Bm), gzb);
                    const V4 RAp = rbp, RBm = ram;
                    const V4 RAm = lds_v4(rat(-k)), RBp = lds_v4(rat(1 + k));
                    rza = k == 1 ? vmul(w1[k], vsub(RAp, RAm)) : vfma(w1[k], vsub(RAp, RAm), rza);
                    rzb = k == 1 ? vmul(w1[k], vsub(RBp, RBm)) : vfma(w1[k], vsub(RBp, RBm), rzb);
                    ram = RAm;
                    rbp = RBp;
                }
                am = Am;
                bp = Bp;
            }
        };
        // the pair's rows za - R .. za + 1 + R: when their slots do not wrap
        // around the ring's end (the same for the whole warp), one base
        // address and constant offsets; else a slot per row
        const int s0 = (int)((unsigned)(za - R) & (NR - 1));
        const float *tua, *tub, *tra, *trb;
        if (s0 + 2 * R + 1 < NR) {
            const float* wb = ring + s0 * TW + 4 * lane;
            const float* wr = rr + s0 * TW + 4 * lane;
            zsums([&](int j) { return wb + (R + j) * TW + HX; },
                  [&](int j) { return wr + (R + j) * TW + HX; });
            tua = wb + R * TW;
            tub = wb + (R + 1) * TW;
            tra = wr + R * TW;
            trb = wr + (R + 1) * TW;
        } else {
            zsums([&](int j) { return row(za + j) + HX; },
                  [&](int j) { return rrow(za + j) + HX; });
            tua = row(za);
            tub = row(za + 1);
            tra = rrow(za);
            trb = rrow(za + 1);
        }
        finish(za, tua, tra, ua, sza, gza, rza, cca, pva, qqa, qza);
        if (za + 1 < zend) finish(za + 1, tub, trb, ub, szb, gzb, rzb, ccb, pvb, qqb, qzb);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // nothing in flight at exit
}

// rows per warp a group
__host__ __device__ constexpr int stream_rw(int) { return 2; }

// three CTAs an SM with constant density (at most 85 registers), two with
// the density's ring and cross terms
template <int R, bool VD, int CH>
__global__ void __launch_bounds__(kThreads, VD ? 2 : 3)
stencil2d_streamed(const Shot* __restrict__ shots, const TileRef* __restrict__ tiles) {
    const TileRef t = tiles[blockIdx.x];
    const Shot& S = shots[t.shot];
    if (!active(S)) return;
    float* un;
    const float *uc, *up;
    slot_ptrs(S, un, uc, up);
    const Layout L = S.L;
    stencil2d_stream_body<R, VD, CH, stream_rw(CH)>(reinterpret_cast<float*>(sw_batch_smem), L,
                                                    un, uc, up, S.C, S.Q, S.den, S.W, S.zb,
                                                    t.tz, t.tx);
}

// ---- time-blocked 2D stencil (constant density) -----------------------------------
constexpr int kTbThreads = 512;
constexpr int kTbWarps = kTbThreads / 32;

// Copies the owned points [zlo, zhi) x [xlo, xhi) of a staged buffer (row
// pitch tw, region origin zr0, xc0) to the same points of grid g.
__device__ __forceinline__ void tb_copy_owned(const float* buf, float* g, int tw, int zr0,
                                              int xc0, int zlo, int zhi, int xlo, int xhi,
                                              int pitch, int lead, int warp, int lane) {
    const int xa = xlo - ((lead + xlo) & 3);  // 16-byte aligned start
    const int nch = (xhi - xa + 3) / 4;
    for (int zz = zlo + warp; zz < zhi; zz += kTbWarps) {
        const float* srow = buf + (zz - zr0) * tw - xc0;
        float* grow = g + (long long)zz * pitch + lead;
        for (int c = lane; c < nch; c += 32) {
            const int x4 = xa + 4 * c;
            if (x4 >= xlo && x4 + 3 < xhi) {
                *reinterpret_cast<float4*>(grow + x4) = *reinterpret_cast<const float4*>(srow + x4);
            } else {
                for (int v = 0; v < 4; v++)
                    if (x4 + v >= xlo && x4 + v < xhi) grow[x4 + v] = srow[x4 + v];
            }
        }
    }
}

// One CTA advances its tile K steps: u_cur and u_prev of the region are staged
// in shared memory once, then each step computes u_next in place of u_prev
// (each point's own previous value is the only one read there) and the two
// buffers swap roles. Per step, in the order of the per-step kernels: the
// stencil on the region's rows still exact after this step, the halo points
// of the new level as its slot holds them (skipped when every slot's halo is
// zero), the sources, x edges, z edges. The owned points of each receiver
// window are copied from each level before it is advanced (the sums are
// formed afterwards, in the per-step kernels' order). A level goes back to
// its slot only when it is one of the last two of the block (the next block
// starts from them) or the last write to its slot (snapshots, final slots).
template <int R, int K>
__global__ void __launch_bounds__(kTbThreads, 1)
stencil2d_tblock(const Shot* __restrict__ shots, const TileRef* __restrict__ tiles,
                 const TbRec* __restrict__ trec, const int* __restrict__ tsrc) {
    constexpr int HX = (R + 3) & ~3;
    constexpr int TW = 128 + 2 * HX;
    constexpr int TH = kTbRows;
    constexpr int CR = TH - 2 * R;  // rows with computed points (C and Q staged)
    constexpr int NC = (4 + 2 * HX) / 4;
    constexpr TbGeom G = tb_geom(R, K);
    constexpr int MZ = G.mz, OZ = G.oz, DX = G.dx, OX = G.ox;
    static_assert(tb_supported(R, K), "time-block depth too large for the radius");
    const TileRef t = tiles[blockIdx.x];
    const Shot& S = shots[t.shot];
    if (S.n > S.stop) return;
    const int n0 = S.n;
    const int kk = min(K, S.stop - n0 + 1);
    const Layout L = S.L;
    const int nz = (int)L.nz, nx = (int)L.nx, pitch = (int)L.pitch, lead = (int)L.lead;
    const int tiles_z = tb_tiles(nz - 2 * R, OZ), tiles_x = tb_tiles(nx - 2 * R, OX);
    const int zr0 = R + t.tz * OZ - MZ;  // grid row of region row 0
    const int xr0 = R + t.tx * OX - DX;  // first computed column
    const int xc0 = xr0 - HX;            // grid column of region column 0
    const int zlo = t.tz == 0 ? 0 : R + t.tz * OZ;
    const int zhi = t.tz == tiles_z - 1 ? nz : R + (t.tz + 1) * OZ;
    const int xlo = t.tx == 0 ? 0 : R + t.tx * OX;
    const int xhi = t.tx == tiles_x - 1 ? nx : R + (t.tx + 1) * OX;
    float* U = reinterpret_cast<float*>(sw_batch_smem);
    float* P = U + TH * TW;
    float* Cs = P + TH * TW;  // [CR][128]: C of region rows R .. TH - R - 1
    float* Qs = Cs + CR * 128;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int pair = *S.pairp;
    {
        // u_prev, u_cur (region), C and Q (computed rows and columns), all
        // in flight at once; points off the grid read as zero
        const float* up = S.ext + (long long)(2 * pair) * S.grid;
        const float* uc = up + S.grid;
        constexpr int CH = TW / 4;
        for (int i = threadIdx.x; i < TH * CH; i += kTbThreads) {
            const int row = i / CH, ch = i - row * CH;
            const int z = zr0 + row;
            const int col = lead + xc0 + 4 * ch;
            const bool ok = z >= 0 && z < nz && col >= 0 && col + 3 < pitch;
            const long long p = ok ? (long long)z * pitch + col : 0;
            cp_async16(U + row * TW + 4 * ch, uc + p, ok);
            cp_async16(P + row * TW + 4 * ch, up + p, ok);
        }
        for (int i = threadIdx.x; i < CR * 32; i += kTbThreads) {
            const int row = i >> 5, ch = i & 31;
            const int z = zr0 + R + row;
            const int col = lead + xr0 + 4 * ch;
            const bool ok = z >= R && z < nz - R && col >= 0 && col + 3 < pitch;
            const long long p = ok ? (long long)z * pitch + col : 0;
            cp_async16(Cs + row * 128 + 4 * ch, S.C + p, ok);
            cp_async16(Qs + row * 128 + 4 * ch, S.Q + p, ok);
        }
        cp_async_wait_all();
    }
    P2 w2[R + 1];
#pragma unroll
    for (int k = 0; k <= R; k++) w2[k] = pk(S.W.c2[k], S.W.c2[k]);
    const P2 ihx = pk(S.W.ih2[1], S.W.ih2[1]), ihz = pk(S.W.ih2[0], S.W.ih2[0]);
    const P2 one = pk(1.f, 1.f);
    const int x = xr0 + 4 * lane;  // this lane's first column
    const bool xbox = x >= S.zb[2] && x + 3 < S.zb[3];
    const bool xany = x + 3 >= R && x < nx - R && lead + x >= 0;
    const bool xfull = x >= R && x + 3 < nx - R;
    // the region holds an edge line or halo points of the grid
    const bool edge = zr0 <= R || zr0 + TH > nz - R - 1 || xc0 <= R || xc0 + TW > nx - R - 1;
    const bool reload = edge && !S.halo_zero;
    const int bz0 = S.bc[0], bz1 = S.bc[1], bx0 = S.bc[2], bx1 = S.bc[3];
    // descriptor fields the loops read, held in registers (the shared-memory
    // accesses are compiler barriers: fields read through S would be
    // re-fetched from global memory on every row)
    const int zbox0 = S.zb[0], zbox1 = S.zb[1];
    float* const partial = S.partial;
    const int win = S.win;
    const unsigned char* const keep = S.keep + (n0 - S.begin);
    const int* const next_slot = S.slots + 3 * (n0 - S.begin) + 2;
    float* const u0 = S.u;
    const long long slot = L.slot;
    float* const ext_out = S.ext + (long long)(2 * (pair ^ 1)) * S.grid;
    const long long grid = S.grid;
    const Windows<float> src = S.src;
    const float* const wavelet = S.wavelet;
    const size_t wcount = (size_t)S.wavelet_count;
    const float* const vel = S.vel;
    const float* const damp = S.damp;
    const float dt = S.dt, dt2 = S.dt2;
    __syncthreads();
    if (kk == 1)  // the block's last two levels: the staged u_cur and the one it computes
        tb_copy_owned(U, ext_out, TW, zr0, xc0, zlo, zhi, xlo, xhi, pitch, lead, warp, lane);
    for (int j = 0; j < kk; j++) {
        const int n = n0 + j;
        // receivers: this tile's part of each window of level n, to scratch
        for (int e = warp; e < t.rec_count; e += kTbWarps) {
            const TbRec q = trec[t.rec_first + e];
            const int w = q.x1 - q.x0;
            const int cnt = (q.z1 - q.z0) * w;
            float* dst = partial + ((size_t)q.rc * K + j) * win;
            for (int i = lane; i < cnt; i += 32) {
                const int z = q.z0 + i / w, xx = q.x0 + i % w;
                dst[(z - q.b0) * q.lx + (xx - q.b2)] = U[(z - zr0) * TW + (xx - xc0)];
            }
        }
        // stencil over the rows that stay exact after this step
        const int rlo = (j + 1) * R, rhi = TH - (j + 1) * R;
        for (int rr = rlo + warp; rr < rhi; rr += kTbWarps) {
            const int z = zr0 + rr;
            if (z < R || z >= nz - R || !xany) continue;
            const bool qzero = xbox && z >= zbox0 && z < zbox1;
            const V4 cc = lds_v4(Cs + (rr - R) * 128 + 4 * lane);
            const V4 qq = lds_v4(Qs + (rr - R) * 128 + 4 * lane);
            const float* tu = U + rr * TW + 4 * lane;
            const V4 u0 = lds_v4(tu + HX);
            V4 sz = vmul(w2[0], u0);
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const V4 a = lds_v4(tu + k * TW + HX);
                const V4 b = lds_v4(tu - k * TW + HX);
                sz = vfma(w2[k], vadd(a, b), sz);
            }
            V4 sx;
            {
                P2 ev[2 * NC], od[2 * NC - 1];
                YWindow<NC>::load(tu, ev, od);
                P2 sh[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    sh[h] = mul2(w2[0], h ? u0.hi : u0.lo);
#pragma unroll
                    for (int k = 1; k <= R; k++) {
                        const P2 a = YWindow<NC>::at(ev, od, HX + 2 * h + k);
                        const P2 b = YWindow<NC>::at(ev, od, HX + 2 * h - k);
                        sh[h] = fma2(w2[k], add2(a, b), sh[h]);
                    }
                }
                sx = {sh[0], sh[1]};
            }
            const V4 lap = vfma(ihz, sz, vmul(ihx, sx));
            float* dst = P + rr * TW + HX + 4 * lane;
            const V4 pv = lds_v4(dst);
            V4 av = {fma2(sub2(qq.lo, one), pv.lo, add2(u0.lo, u0.lo)),
                     fma2(sub2(qq.hi, one), pv.hi, add2(u0.hi, u0.hi))};
            if (!qzero) {
                const float4 q4 = to_f4(qq);
                const V4 rq = from_f4(make_float4(rcp_approx(1.f + q4.x), rcp_approx(1.f + q4.y),
                                                  rcp_approx(1.f + q4.z), rcp_approx(1.f + q4.w)));
                av = {mul2(av.lo, rq.lo), mul2(av.hi, rq.hi)};
            }
            const V4 out = {fma2(lap.lo, cc.lo, av.lo), fma2(lap.hi, cc.hi, av.hi)};
            if (xfull) {
                sts_v4(dst, out);
            } else {
                const float4 o = to_f4(out);
                const float oa[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
                for (int v = 0; v < 4; v++)
                    if (x + v >= R && x + v < nx - R) dst[v] = oa[v];
            }
        }
        __syncthreads();
        float* un = u0 + (long long)next_slot[3 * j] * slot;
        if (reload) {
            // halo points of the new level: what its slot holds (the per-step
            // kernels never write them before the boundary phases); halo rows
            // of the region first, then the halo columns of its interior rows
            const int ra = max(zr0, 0), rb = min(zr0 + TH, nz);
            const int ca = max(xc0, 0), cb = min(xc0 + TW, nx);
            const int w = max(0, cb - ca);
            const int top = max(0, min(R, rb) - ra);
            const int bot0 = max(nz - R, ra), bot = max(0, rb - bot0);
            const int m0 = max(ra, R), m1 = min(rb, nz - R), nm = max(0, m1 - m0);
            const int nl = max(0, min(R, cb) - ca), right0 = max(nx - R, ca);
            const int nr = max(0, cb - right0), per = nl + nr;
            const int A = (top + bot) * w, B = nm * per;
#pragma unroll 4
            for (int i = threadIdx.x; i < A + B; i += kTbThreads) {
                int zz, xx;
                if (i < A) {
                    const int row = i / w;
                    zz = row < top ? ra + row : bot0 + (row - top);
                    xx = ca + (i - row * w);
                } else {
                    const int k = i - A, row = k / per, c = k - row * per;
                    zz = m0 + row;
                    xx = c < nl ? ca + c : right0 + (c - nl);
                }
                P[(zz - zr0) * TW + (xx - xc0)] = un[L.at2(zz, xx)];
            }
            __syncthreads();
        }
        if (t.src_count) {
            for (int q = 0; q < t.src_count; q++) {
                const size_t s = (size_t)tsrc[t.src_first + q];
                const float w = wavelet_at(wavelet, wcount, (size_t)n, src.count, s);
                if (w == 0.f) continue;
                const size_t* b = src.interval + 4 * s;
                const float* v = src.values + src.offsets[s];
                const long long total = window_size<2>(b);
                for (long long i = threadIdx.x; i < total; i += kTbThreads) {
                    long long iz, ix, iy;
                    window_point<2>(b, i, iz, ix, iy);
                    const int z = (int)(b[0] + iz), xx = (int)(b[2] + ix);
                    if (z < zr0 || z >= zr0 + TH || xx < xc0 || xx >= xc0 + TW) continue;
                    const float kws = window_weight<float, 2>(b, v, iz, ix, iy);
                    const long long p = L.at2(z, xx);
                    const float vv = vel[p] * vel[p];
                    const float d = 1.f + damp[p] * dt * vv * 0.5f;
                    atomicAdd(P + (z - zr0) * TW + (xx - xc0), dt2 * vv * kws * w / d);
                }
            }
            __syncthreads();
        }
        if (edge) {
            // x edges on the interior rows, then z edges on the interior columns
            const int r0 = max(zr0, R), r1 = min(zr0 + TH, nz - R);
            const bool left = bx0 && R >= xc0 && R < xc0 + TW;
            const bool right = bx1 && nx - R - 1 >= xc0 && nx - R - 1 < xc0 + TW;
            if (left || right) {
                for (int i = r0 + threadIdx.x; i < r1; i += kTbThreads) {
                    float* row = P + (i - zr0) * TW - xc0;  // indexed by grid column
                    if (left) {
                        if (bx0 == 1) row[R] = 0.f;
                        else
                            for (int q = 1; q <= R; q++)
                                if (R - q >= xc0) row[R - q] = row[R + q];
                    }
                    if (right) {
                        const int e = nx - R - 1;
                        if (bx1 == 1) row[e] = 0.f;
                        else
                            for (int q = 1; q <= R; q++)
                                if (e + q < xc0 + TW) row[e + q] = row[e - q];
                    }
                }
            }
            __syncthreads();
            const int c0 = max(xc0, R), c1 = min(xc0 + TW, nx - R);
            const bool top = bz0 && R >= zr0 && R < zr0 + TH;
            const bool bottom = bz1 && nz - R - 1 >= zr0 && nz - R - 1 < zr0 + TH;
            if (top || bottom) {
                for (int c = c0 + threadIdx.x; c < c1; c += kTbThreads) {
                    float* col = P + (c - xc0) - zr0 * TW;  // indexed by grid row * TW
                    if (top) {
                        if (bz0 == 1) col[R * TW] = 0.f;
                        else
                            for (int q = 1; q <= R; q++)
                                if (R - q >= zr0) col[(R - q) * TW] = col[(R + q) * TW];
                    }
                    if (bottom) {
                        const int e = nz - R - 1;
                        if (bz1 == 1) col[e * TW] = 0.f;
                        else
                            for (int q = 1; q <= R; q++)
                                if (e + q < zr0 + TH) col[(e + q) * TW] = col[(e - q) * TW];
                    }
                }
            }
            __syncthreads();
        }
        // owned points of the level: every one to the other pair when it is
        // one of the block's last two; to its slot, as the per-step kernels
        // write it (interior and Neumann mirrors), when that is the slot's
        // last write
        if (j >= kk - 2)
            tb_copy_owned(P, ext_out + (j - (kk - 2)) * grid, TW, zr0, xc0, zlo, zhi, xlo, xhi,
                          pitch, lead, warp, lane);
        if (keep[j]) {
            const int xa = xlo - ((lead + xlo) & 3);  // 16-byte aligned start
            const int nch = (xhi - xa + 3) / 4;
            for (int zz = zlo + warp; zz < zhi; zz += kTbWarps) {
                const bool zin = zz >= R && zz < nz - R;
                const float* srow = P + (zz - zr0) * TW - xc0;
                float* grow = un + (long long)zz * pitch + lead;
                for (int c = lane; c < nch; c += 32) {
                    const int x4 = xa + 4 * c;
                    if (zin && x4 >= max(xlo, R) && x4 + 3 < min(xhi, nx - R)) {
                        *reinterpret_cast<float4*>(grow + x4) =
                            *reinterpret_cast<const float4*>(srow + x4);
                        continue;
                    }
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const int xx = x4 + v;
                        if (xx < xlo || xx >= xhi) continue;
                        const bool xin = xx >= R && xx < nx - R;
                        bool st = zin && xin;
                        if (!st && zin != xin)  // halo of one axis: Neumann mirrors only
                            st = xin ? S.bc[zz < R ? 0 : 1] == 2 : S.bc[xx < R ? 2 : 3] == 2;
                        if (st) grow[xx] = srow[xx];
                    }
                }
            }
        }
        float* tmp = U;
        U = P;
        P = tmp;
    }
}

// Receiver records of the time-blocked shots from the window copies: one
// warp per receiver, each level summed in the per-step gather's order (the
// records equal the per-step kernels' bit for bit).
__global__ void receivers_tblock(const Shot* __restrict__ shots,
                                 const PairRef* __restrict__ pairs, int npairs) {
    const int wid = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (wid >= npairs) return;
    const PairRef pr = pairs[wid];
    const Shot& S = shots[pr.shot];
    if (!active(S)) return;
    const int K = S.depth;
    const int kk = min(K, S.stop - S.n + 1);
    const size_t* b = S.rec.interval + 4 * (size_t)pr.item;
    const float* v = S.rec.values + S.rec.offsets[pr.item];
    const int lz = (int)(b[1] - b[0] + 1), lx = (int)(b[3] - b[2] + 1);
    const float* vf = v + lz;
    const int sub = lane & 7, grp = lane >> 3;
    for (int j = 0; j < kk; j++) {
        const float* win = S.partial + ((size_t)pr.item * K + j) * S.win;
        float sum = 0.f;
        for (int f = sub; f - sub < lx; f += 8) {
            if (f >= lx) continue;
            const float wf = vf[f];
            for (int row = grp; row < lz; row += 4) sum += win[row * lx + f] * (v[row] * wf);
        }
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) S.receivers[(size_t)(S.n + j - 1) * S.rec.count + pr.item] = sum;
    }
}

// Flags (word 0) a nonzero halo value in slots [0, nslots) of a 2D grid.
__global__ void halo_nonzero(const float* __restrict__ u, Layout L, int nslots,
                             int* __restrict__ flag) {
    const int r = L.r;
    const long long nz = L.nz, nx = L.nx;
    const long long per = 2LL * r * nx + 2LL * r * (nz - 2 * r);  // halo points a slot
    const long long total = per * nslots;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long s = i / per, k = i - s * per;
        long long z, x;
        if (k < 2LL * r * nx) {
            const long long row = k / nx;
            z = row < r ? row : nz - 2 * r + row;
            x = k - row * nx;
        } else {
            const long long m = k - 2LL * r * nx, row = m / (2 * r), c = m - row * (2 * r);
            z = r + row;
            x = c < r ? c : nx - 2 * r + c;
        }
        if (u[s * L.slot + L.at2(z, x)] != 0.f) atomicOr(flag, 1);
    }
}

__global__ void set_stops(Shot* shots, int nshots, int steps) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nshots) {
        const long long stop = (long long)shots[s].n + steps - 1;
        shots[s].stop = (int)(stop < shots[s].end ? stop : shots[s].end);
    }
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
    if (!active(S) || S.depth > 1) return;  // time-blocked shots apply their own
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
    if (s < nshots && shots[s].n <= shots[s].stop) {
        const int k = shots[s].depth;
        const int left = shots[s].stop - shots[s].n + 1;
        shots[s].n += k > 1 ? (k < left ? k : left) : 1;
        if (k > 1) *shots[s].pairp ^= 1;  // the launch left its levels in the other pair
    }
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
    unsigned char* keep = nullptr;  // engine-owned per-step last-write flags
    float* partial = nullptr;       // engine-owned receiver partials (time-blocked)
    size_t partial_cap = 0;
    std::vector<int> perm;   // final logical -> physical slots
    std::vector<int> table;  // per step: prev, cur, next physical slots
    std::vector<size_t> rec_iv;  // receiver windows (host copy)
    std::vector<size_t> src_iv;  // source windows (host copy)
    float* ext = nullptr;    // engine-owned level pairs (time-blocked)
    int* pairp = nullptr;
    bool in_pairs = false;   // the latest levels live in `ext`, not the slots
    long long grid = 0;      // elements of one pitched grid
    // time blocking needs: constant density, each step reading the levels
    // the two steps before it wrote, source windows off the halo
    bool blockable = false;
    bool finished_restored = false;
};

// Steps per launch for shot `h` when its radius asks for `k`: k where the
// shot allows time blocking (and its interior is wide enough for the edge
// rules to stay within one side), else 1.
static int effective_depth(const HostShot& h, int k) {
    const Layout& L = h.d.L;
    const int r = L.r;
    if (k <= 1 || !h.blockable || !tb_supported(r, k)) return 1;
    if (L.nz - 2 * r < 4 * r + 2 || L.nx - 2 * r < 4 * r + 2) return 1;
    return k;
}

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

// streamed tiles of CH rows (ring of kRing rows)
template <int R, bool VD, int CH>
static void launch_stream_t(bool configure, const Shot* shots, const TileRef* tiles,
                            int ntiles, cudaStream_t st) {
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * kRing * (128 + 2 * HX) * 4;
    if (configure) {
        cudaFuncSetAttribute(stencil2d_streamed<R, VD, CH>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        return;
    }
    stencil2d_streamed<R, VD, CH><<<ntiles, kThreads, bytes, st>>>(shots, tiles);
}

template <int R, bool VD>
static void launch_group_r(bool configure, int tz, const Shot* shots, const TileRef* tiles,
                           int ntiles, cudaStream_t st) {
    if (tz == 8) launch_group_t<R, VD, 8>(configure, shots, tiles, ntiles, st);
    else if (tz == 32) launch_group_t<R, VD, 32>(configure, shots, tiles, ntiles, st);
    else if (tz == 64) launch_stream_t<R, VD, 64>(configure, shots, tiles, ntiles, st);
    else if (tz == 128) launch_stream_t<R, VD, 128>(configure, shots, tiles, ntiles, st);
    else if (tz == 256) launch_stream_t<R, VD, 256>(configure, shots, tiles, ntiles, st);
    else launch_group_t<R, VD, 16>(configure, shots, tiles, ntiles, st);
}

template <int R, int K>
static void launch_tblock_t(bool configure, const Shot* shots, const TileRef* tiles,
                            const TbRec* trec, const int* tsrc, int ntiles, cudaStream_t st) {
    if constexpr (tb_supported(R, K)) {
        constexpr int HX = (R + 3) & ~3;
        const int bytes = (2 * kTbRows * (128 + 2 * HX) + 2 * (kTbRows - 2 * R) * 128) * 4;
        if (configure) {
            cudaFuncSetAttribute(stencil2d_tblock<R, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 bytes);
            return;
        }
        stencil2d_tblock<R, K><<<ntiles, kTbThreads, bytes, st>>>(shots, tiles, trec, tsrc);
    } else {
        fail(SIMWAVE_E_ARGUMENT, "time-block depth too large for the space order");
    }
}

template <int R>
static void launch_tblock_r(bool configure, int k, const Shot* shots, const TileRef* tiles,
                            const TbRec* trec, const int* tsrc, int ntiles, cudaStream_t st) {
    if (k == 2) launch_tblock_t<R, 2>(configure, shots, tiles, trec, tsrc, ntiles, st);
    else if (k == 3) launch_tblock_t<R, 3>(configure, shots, tiles, trec, tsrc, ntiles, st);
    else launch_tblock_t<R, 4>(configure, shots, tiles, trec, tsrc, ntiles, st);
}

static void launch_tblock(bool configure, int r, int k, const Shot* shots, const TileRef* tiles,
                          const TbRec* trec, const int* tsrc, int ntiles, cudaStream_t st) {
#define SB_T(RR)                                                                          \
    case RR:                                                                              \
        launch_tblock_r<RR>(configure, k, shots, tiles, trec, tsrc, ntiles, st);          \
        break;
    switch (r) {
        SB_T(1) SB_T(2) SB_T(3) SB_T(4) SB_T(5) SB_T(6) SB_T(7) SB_T(8) SB_T(9) SB_T(10)
    }
#undef SB_T
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
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
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
    int depth[kMaxRadius + 1];      // steps per launch per radius (tuning; 1 = per step)
    // device tables (rebuilt when the shot set changes)
    Shot* d_shots = nullptr;
    size_t cap_shots = 0;
    TileRef* d_tiles = nullptr;
    size_t cap_tiles = 0;
    PairRef* d_src = nullptr;
    size_t cap_src = 0;
    PairRef* d_rec = nullptr;
    size_t cap_rec = 0;
    TbRec* d_trec = nullptr;     // receiver-window parts of time-blocked tiles
    size_t cap_trec = 0;
    PairRef* d_tbrec = nullptr;  // receivers of time-blocked shots
    size_t cap_tbrec = 0;
    int* d_tsrc = nullptr;       // sources meeting each time-blocked tile's region
    size_t cap_tsrc = 0;
    struct Group {
        int r;
        bool vd;
        int depth;
        int first, count;  // range in d_tiles
    };
    std::vector<Group> groups;
    int nsrc_pairs = 0, nrec_pairs = 0, ntb_rec = 0;
    bool any_stepwise = false;
    bool dirty = true;
    // graph of `graph_steps` steps
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0;
    size_t kernel_launches = 0;

    int* words = nullptr;  // device scratch for admission results

    int* scratch_words() {
        if (!words) SB_CUDA(cudaMalloc(&words, 16 * sizeof(int)));
        return words;
    }

    Engine() {
        for (int r = 0; r <= kMaxRadius; r++) {
            tile_rows[r] = 16;
            depth[r] = 1;
        }
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

    // Puts the shot's latest two levels where its next launches read them:
    // into pair 0 of its level pairs (time-blocked) or back into the
    // schedule's slots (per step). Runs between launches, on the engine
    // stream.
    void move_levels(HostShot& h, bool blocked) {
        const size_t bytes = (size_t)h.grid * sizeof(float);
        const bool running = h.d.n <= h.d.end;
        const size_t i = (size_t)(h.d.n - h.d.begin);
        if (blocked && !h.in_pairs) {
            if (!h.ext) {
                SB_CUDA(cudaMallocAsync(&h.ext, 4 * bytes, stream));
                SB_CUDA(cudaMallocAsync(&h.pairp, sizeof(int), stream));
            }
            SB_CUDA(cudaMemsetAsync(h.pairp, 0, sizeof(int), stream));
            if (running) {
                for (int l = 0; l < 2; l++)
                    SB_CUDA(cudaMemcpyAsync(h.ext + l * h.grid,
                                            h.d.u + (long long)h.table[3 * i + l] * h.d.L.slot,
                                            bytes, cudaMemcpyDeviceToDevice, stream));
            }
            h.in_pairs = true;
        } else if (!blocked && h.in_pairs) {
            int pair = 0;
            SB_CUDA(cudaMemcpyAsync(&pair, h.pairp, sizeof(int), cudaMemcpyDeviceToHost, stream));
            SB_CUDA(cudaStreamSynchronize(stream));
            if (running) {
                for (int l = 0; l < 2; l++)
                    SB_CUDA(cudaMemcpyAsync(h.d.u + (long long)h.table[3 * i + l] * h.d.L.slot,
                                            h.ext + (2 * pair + l) * h.grid, bytes,
                                            cudaMemcpyDeviceToDevice, stream));
            }
            h.in_pairs = false;
        }
        h.d.ext = h.ext;
        h.d.pairp = h.pairp;
        h.d.grid = h.grid;
    }

    // rebuild the device tables from the host shots (descriptors keep the
    // host-tracked step counters, which equal the device ones between runs)
    void rebuild() {
        const size_t ns = shots.size();
        grow(d_shots, cap_shots, ns);
        std::vector<Shot> desc(ns);
        std::map<std::tuple<int, int, int>, std::vector<TileRef>> byg;
        std::vector<PairRef> srcp, recp, tbrecp;
        std::vector<TbRec> trec;
        std::vector<int> tsrc;
        any_stepwise = false;
        for (size_t i = 0; i < ns; i++) {
            HostShot& h = shots[i];
            const Layout& L = h.d.L;
            const int r = L.r;
            const int k = effective_depth(h, depth[r]);
            h.d.depth = k;
            move_levels(h, k > 1);
            if (k > 1) {
                int win = 1;
                for (size_t q = 0; q < h.d.rec.count; q++) {
                    const size_t* b = &h.rec_iv[4 * q];
                    win = std::max(win, (int)((b[1] - b[0] + 1) * (b[3] - b[2] + 1)));
                }
                const size_t need = h.d.rec.count * (size_t)k * win;
                if (need > h.partial_cap) {
                    if (h.partial) SB_CUDA(cudaFreeAsync(h.partial, stream));
                    h.partial = nullptr;
                    h.partial_cap = 0;
                    SB_CUDA(cudaMallocAsync(&h.partial, std::max<size_t>(need, 4) * sizeof(float),
                                            stream));
                    h.partial_cap = std::max<size_t>(need, 4);
                }
                h.d.partial = h.partial;
                h.d.win = win;
                const TbGeom g = tb_geom(r, k);
                const int nt_z = tb_tiles(L.nz - 2 * r, g.oz);
                const int nt_x = tb_tiles(L.nx - 2 * r, g.ox);
                // each window point is copied by the tile that owns it
                std::vector<std::vector<TbRec>> per(nt_z * nt_x);
                for (size_t q = 0; q < h.d.rec.count; q++) {
                    const size_t* b = &h.rec_iv[4 * q];
                    const int z0 = tb_tile_of((long long)b[0], r, L.nz, g.oz);
                    const int z1 = tb_tile_of((long long)b[1], r, L.nz, g.oz);
                    const int x0 = tb_tile_of((long long)b[2], r, L.nx, g.ox);
                    const int x1 = tb_tile_of((long long)b[3], r, L.nx, g.ox);
                    for (int a = z0; a <= z1; a++)
                        for (int c = x0; c <= x1; c++) {
                            const int lo_z = a == 0 ? 0 : r + a * g.oz;
                            const int hi_z = a == nt_z - 1 ? (int)L.nz : r + (a + 1) * g.oz;
                            const int lo_x = c == 0 ? 0 : r + c * g.ox;
                            const int hi_x = c == nt_x - 1 ? (int)L.nx : r + (c + 1) * g.ox;
                            TbRec e;
                            e.rc = (int)q;
                            e.z0 = std::max(lo_z, (int)b[0]);
                            e.z1 = std::min(hi_z, (int)b[1] + 1);
                            e.x0 = std::max(lo_x, (int)b[2]);
                            e.x1 = std::min(hi_x, (int)b[3] + 1);
                            e.b0 = (int)b[0];
                            e.b2 = (int)b[2];
                            e.lx = (int)(b[3] - b[2] + 1);
                            if (e.z1 > e.z0 && e.x1 > e.x0) per[a * nt_x + c].push_back(e);
                        }
                    tbrecp.push_back({(int)i, (int)q});
                }
                auto& v = byg[{r, 0, k}];
                const int hx = (r + 3) & ~3;
                for (int a = 0; a < nt_z; a++)
                    for (int c = 0; c < nt_x; c++) {
                        const auto& e = per[a * nt_x + c];
                        // the staged region: kTbRows rows from zr0, 128 + 2 hx columns from xc0
                        const long long zr0 = r + (long long)a * g.oz - g.mz;
                        const long long xc0 = r + (long long)c * g.ox - g.dx - hx;
                        const int first_src = (int)tsrc.size();
                        for (size_t q = 0; q < h.d.src.count; q++) {
                            const size_t* b = &h.src_iv[4 * q];
                            if ((long long)b[1] >= zr0 && (long long)b[0] < zr0 + kTbRows &&
                                (long long)b[3] >= xc0 && (long long)b[2] < xc0 + 128 + 2 * hx)
                                tsrc.push_back((int)q);
                        }
                        v.push_back({(int)i, a, c, (int)trec.size(), (int)e.size(), first_src,
                                     (int)tsrc.size() - first_src});
                        trec.insert(trec.end(), e.begin(), e.end());
                    }
            } else {
                any_stepwise = true;
                const int tz = tile_rows[r];
                const int nt_z = (int)((L.nz - 2 * r + tz - 1) / tz);
                const int nt_x = (int)((L.nx - 2 * r + 127) / 128);
                auto& v = byg[{r, h.d.den ? 1 : 0, 1}];
                for (int a = 0; a < nt_z; a++)
                    for (int b = 0; b < nt_x; b++) v.push_back({(int)i, a, b, 0, 0, 0, 0});
                for (size_t q = 0; q < h.d.src.count; q++) srcp.push_back({(int)i, (int)q});
                for (size_t q = 0; q < h.d.rec.count; q++) recp.push_back({(int)i, (int)q});
            }
            desc[i] = h.d;
        }
        std::vector<TileRef> all;
        groups.clear();
        for (auto& kv : byg) {
            groups.push_back({std::get<0>(kv.first), std::get<1>(kv.first) != 0,
                              std::get<2>(kv.first), (int)all.size(), (int)kv.second.size()});
            all.insert(all.end(), kv.second.begin(), kv.second.end());
        }
        grow(d_tiles, cap_tiles, all.size());
        grow(d_src, cap_src, srcp.size());
        grow(d_rec, cap_rec, recp.size());
        grow(d_trec, cap_trec, trec.size());
        grow(d_tbrec, cap_tbrec, tbrecp.size());
        grow(d_tsrc, cap_tsrc, tsrc.size());
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
        if (!trec.empty())
            SB_CUDA(cudaMemcpyAsync(d_trec, trec.data(), trec.size() * sizeof(TbRec),
                                    cudaMemcpyHostToDevice, stream));
        if (!tbrecp.empty())
            SB_CUDA(cudaMemcpyAsync(d_tbrec, tbrecp.data(), tbrecp.size() * sizeof(PairRef),
                                    cudaMemcpyHostToDevice, stream));
        if (!tsrc.empty())
            SB_CUDA(cudaMemcpyAsync(d_tsrc, tsrc.data(), tsrc.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, stream));
        SB_CUDA(cudaStreamSynchronize(stream));
        nsrc_pairs = (int)srcp.size();
        nrec_pairs = (int)recp.size();
        ntb_rec = (int)tbrecp.size();
        for (const Group& g : groups) {
            if (g.depth > 1)
                launch_tblock(true, g.r, g.depth, nullptr, nullptr, nullptr, nullptr, 0, stream);
            else
                launch_group(true, g.r, g.vd, tile_rows[g.r], nullptr, nullptr, 0, stream);
        }
        drop_graph();
        dirty = false;
    }

    // kernels of one step (one block of steps for the time-blocked shots)
    size_t step_launches() const {
        return groups.size() + (nsrc_pairs ? 1 : 0) + (any_stepwise ? 2 : 0) +
               (nrec_pairs ? 1 : 0) + (ntb_rec ? 1 : 0) + 1;
    }

    // one step of every per-step shot, one block of steps of every
    // time-blocked shot
    void enqueue_step(cudaStream_t st) {
        for (const Group& g : groups) {
            if (g.depth > 1)
                launch_tblock(false, g.r, g.depth, d_shots, d_tiles + g.first, d_trec, d_tsrc,
                              g.count, st);
            else
                launch_group(false, g.r, g.vd, tile_rows[g.r], d_shots, d_tiles + g.first,
                             g.count, st);
            SB_CUDA(cudaGetLastError());
        }
        if (nsrc_pairs) sources_batched<<<nsrc_pairs, 128, 0, st>>>(d_shots, d_src);
        const int ns = (int)shots.size();
        if (any_stepwise) {
            edges_batched<<<ns, 256, 0, st>>>(d_shots, 1);
            edges_batched<<<ns, 256, 0, st>>>(d_shots, 0);
        }
        if (nrec_pairs)
            receivers_batched<<<(nrec_pairs * 32 + 255) / 256, 256, 0, st>>>(d_shots, d_rec,
                                                                             nrec_pairs);
        if (ntb_rec)
            receivers_tblock<<<(ntb_rec * 32 + 255) / 256, 256, 0, st>>>(d_shots, d_tbrec,
                                                                          ntb_rec);
        advance_batched<<<(ns + 127) / 128, 128, 0, st>>>(d_shots, ns);
        SB_CUDA(cudaGetLastError());
    }

    // Advances every shot by `steps` time steps (or to its end).
    void run(int steps, cudaStream_t user) {
        if (dirty) rebuild();
        if (shots.empty() || steps <= 0) return;
        // launches needed: the most blocks any shot needs for its steps
        int blocks = 0;
        for (const HostShot& h : shots) {
            const int left = std::min(steps, h.d.end - h.d.n + 1);
            if (left > 0) blocks = std::max(blocks, (left + h.d.depth - 1) / h.d.depth);
        }
        if (blocks <= 0) return;
        const int K = 16;  // steps per graph
        if (!exec && blocks >= K) {
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
        // each shot stops after `steps` more steps, however many launches run
        const int ns = (int)shots.size();
        set_stops<<<(ns + 127) / 128, 128, 0, stream>>>(d_shots, ns, steps);
        SB_CUDA(cudaGetLastError());
        kernel_launches += 1;
        int done = 0;
        const size_t per_step = step_launches();
        while (blocks - done >= K && exec) {
            SB_CUDA(cudaGraphLaunch(exec, stream));
            done += K;
            kernel_launches += K * per_step;
        }
        for (; done < blocks; done++) {
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
    h.table = table;
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
    d.stop = d.end;
    d.depth = 1;
    // last-write flags (a level of a time block goes back to its slot when no
    // later step overwrites that slot) and the level chain time blocking
    // relies on: each step reads the levels the two steps before it wrote
    const size_t nsteps = table.size() / 3;
    std::vector<unsigned char> keep(nsteps, 0);
    {
        std::vector<char> seen(nsl + 1, 0);
        for (size_t i = nsteps; i-- > 0;) {
            const int slot = table[3 * i + 2];
            if (!seen[slot]) keep[i] = 1;
            seen[slot] = 1;
        }
    }
    bool chain = true;
    for (size_t i = 1; i < nsteps; i++)
        chain = chain && table[3 * i] == table[3 * (i - 1) + 1] &&
                table[3 * i + 1] == table[3 * (i - 1) + 2];
    // engine-owned: coefficients, schedule, last-write flags (stream-ordered
    // allocations: admission runs while other shots step)
    SB_CUDA(cudaMallocAsync(&h.cq, 2 * (size_t)grid * sizeof(float), E.stream));
    SB_CUDA(cudaMallocAsync(&h.slots, table.size() * sizeof(int), E.stream));
    SB_CUDA(cudaMallocAsync(&h.keep, std::max<size_t>(nsteps, 1), E.stream));
    SB_CUDA(cudaMemcpyAsync(h.slots, table.data(), table.size() * sizeof(int),
                            cudaMemcpyHostToDevice, E.stream));
    SB_CUDA(cudaMemcpyAsync(h.keep, keep.data(), nsteps, cudaMemcpyHostToDevice, E.stream));
    d.keep = h.keep;
    form_coefficients(d.vel, d.damp, h.cq, h.cq + grid, grid, d.dt, E.stream);
    SB_CUDA(cudaGetLastError());
    // the box where Q is zero (its loads are skipped there), whether every
    // slot's halo is zero, and the window tables (receivers for the tile
    // lists, sources for the halo test) -- then one wait
    int* words = E.scratch_words();
    find_zero_box(h.cq + grid, d.L, words, E.stream);
    SB_CUDA(cudaMemsetAsync(words + 8, 0, sizeof(int), E.stream));
    halo_nonzero<<<256, 256, 0, E.stream>>>(d.u, d.L, (int)nsl, words + 8);
    SB_CUDA(cudaGetLastError());
    int box[9];
    SB_CUDA(cudaMemcpyAsync(box, words, sizeof(box), cudaMemcpyDeviceToHost, E.stream));
    h.rec_iv.assign(4 * P->num_receivers, 0);
    h.src_iv.assign(4 * P->num_sources, 0);
    std::vector<size_t>& src_iv = h.src_iv;
    if (P->num_receivers)
        SB_CUDA(cudaMemcpyAsync(h.rec_iv.data(), P->rec_points_interval,
                                h.rec_iv.size() * sizeof(size_t), cudaMemcpyDeviceToHost,
                                E.stream));
    if (P->num_sources)
        SB_CUDA(cudaMemcpyAsync(src_iv.data(), P->src_points_interval,
                                src_iv.size() * sizeof(size_t), cudaMemcpyDeviceToHost,
                                E.stream));
    SB_CUDA(cudaStreamSynchronize(E.stream));
    const bool good = box[6] == 0 && box[1] > box[0] && box[3] > box[2];
    for (int i = 0; i < 4; i++) d.zb[i] = good ? box[i] : 0;
    d.halo_zero = box[8] == 0;
    bool src_inside = true;
    for (size_t q = 0; q < P->num_sources; q++) {
        const size_t* b = &src_iv[4 * q];
        src_inside = src_inside && b[0] >= (size_t)r && b[1] < P->nz - r && b[2] >= (size_t)r &&
                     b[3] < P->nx - r;
    }
    h.blockable = !vd && chain && src_inside;
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
    E.move_levels(h, false);  // an unfinished time-blocked shot's levels go back to its slots
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
    cudaFreeAsync(h.cq, E.stream);
    cudaFreeAsync(h.slots, E.stream);
    cudaFreeAsync(h.keep, E.stream);
    if (h.partial) cudaFreeAsync(h.partial, E.stream);
    if (h.ext) cudaFreeAsync(h.ext, E.stream);
    if (h.pairp) cudaFreeAsync(h.pairp, E.stream);
    SB_CUDA(cudaStreamSynchronize(E.stream));
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
// reference's order. With `ring`, the tile also saves its points of the
// four interior edge lines between the sources and the boundary conditions
// (rows r and nz - r - 1, then columns r and nx - r - 1 without the corner
// rows: the layout of the adjoint's boundary ring).
__device__ void tile_sources_edges(const Shot2D& P, float* un, long long n, int tz, int tx,
                                   float* ring = nullptr) {
    const Layout& L = P.L;
    const int r = L.r;
    const int nz = (int)L.nz, nx = (int)L.nx;
    const int z_lo = tz == 0 ? 0 : r + 16 * tz - P.zoff;
    const int z_hi = tz == P.tiles_z - 1 ? nz : r + 16 * (tz + 1) - P.zoff;
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
    if (ring) {
        const int w = nx - 2 * r, h = nz - 2 * r - 2;
        const int c0 = max(x_lo, r), c1 = min(x_hi, nx - r);
        if (tz == 0)
            for (int j = c0 + threadIdx.x; j < c1; j += blockDim.x) ring[j - r] = un[L.at2(r, j)];
        if (tz == P.tiles_z - 1)
            for (int j = c0 + threadIdx.x; j < c1; j += blockDim.x)
                ring[w + j - r] = un[L.at2(nz - r - 1, j)];
        const int i0 = max(z_lo, r + 1), i1 = min(z_hi, nz - r - 1);
        if (tx == 0)
            for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
                ring[2 * w + i - r - 1] = un[L.at2(i, r)];
        if (tx == P.tiles_x - 1)
            for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
                ring[2 * w + h + i - r - 1] = un[L.at2(i, nx - r - 1)];
        __syncthreads();
    }
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
                                      t / P.tiles_x, t % P.tiles_x, P.zoff);
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
// `ring` (optional) receives the interior edge lines before the boundary
// conditions.
template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_step(const Shot2D P, float* un, const float* uc, const float* up, long long n,
               float* ring) {
    if ((int)blockIdx.x < P.ntiles) {
        const int t = blockIdx.x;
        stencil2d_tile<R, VD, TZ>(reinterpret_cast<float*>(sw_batch_smem), P.L, un, uc, up, P.C,
                                  P.Q, P.den, P.W, P.zb, t / P.tiles_x, t % P.tiles_x, P.zoff);
        __syncthreads();
        tile_sources_edges(P, un, n, t / P.tiles_x, t % P.tiles_x, ring);
        return;
    }
    const long long w = ((long long)(blockIdx.x - P.ntiles) * blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)P.rec.count) return;
    const float sum = gather_window<float, 2>(uc, P.L, P.rec.interval + w * 4,
                                              P.rec.values + P.rec.offsets[w], threadIdx.x & 31);
    if ((threadIdx.x & 31) == 0) P.receivers[(n - 1) * (long long)P.rec.count + w] = sum;
}

// One time step of several 2D shots of one layout in one launch (the
// gradient's lockstep passes): `per_shot` blocks a shot, the shot's tiles
// (stencil, sources, edges, and its ring row when it has a ring) then, with
// `record`, its receiver blocks. Levels i_un, i_uc, i_up of the shot's level
// array (`G` elements each); ring row at element `ring_off`.
template <int R, bool VD, int TZ>
__global__ void __launch_bounds__(kThreads)
stencil2d_step_shots(const StepShot* __restrict__ shots, int per_shot, long long G, int i_un,
                     int i_uc, int i_up, long long n, long long ring_off, int record) {
    const int s = blockIdx.x / per_shot, b = blockIdx.x - s * per_shot;
    const StepShot& Q = shots[s];
    const Shot2D& P = Q.S;
    float* un = Q.lev + i_un * G;
    const float* uc = Q.lev + i_uc * G;
    const float* up = Q.lev + i_up * G;
    if (b < P.ntiles) {
        stencil2d_tile<R, VD, TZ>(reinterpret_cast<float*>(sw_batch_smem), P.L, un, uc, up, P.C,
                                  P.Q, P.den, P.W, P.zb, b / P.tiles_x, b % P.tiles_x, P.zoff);
        __syncthreads();
        tile_sources_edges(P, un, n, b / P.tiles_x, b % P.tiles_x,
                           Q.ring ? Q.ring + ring_off : nullptr);
        return;
    }
    if (!record) return;
    const long long w = ((long long)(b - P.ntiles) * blockDim.x + threadIdx.x) >> 5;
    if (w >= (long long)P.rec.count) return;
    const float sum = gather_window<float, 2>(uc, P.L, P.rec.interval + w * 4,
                                              P.rec.values + P.rec.offsets[w], threadIdx.x & 31);
    if ((threadIdx.x & 31) == 0) P.receivers[(n - 1) * (long long)P.rec.count + w] = sum;
}

template <int R, bool VD>
static void step_shots_r(const StepShot* shots, int nshots, int per_shot, long long G, int i_un,
                         int i_uc, int i_up, long long n, long long ring_off, bool record,
                         cudaStream_t st) {
    constexpr int TZ = 16;
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        SB_CUDA(cudaFuncSetAttribute(stencil2d_step_shots<R, VD, TZ>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        configured[dev & 63] = true;
    }
    stencil2d_step_shots<R, VD, TZ><<<nshots * per_shot, kThreads, bytes, st>>>(
        shots, per_shot, G, i_un, i_uc, i_up, n, ring_off, record ? 1 : 0);
}

template <int R, bool VD>
static void step_r(const Shot2D& P, float* un, const float* uc, const float* up, long long n,
                   float* ring, cudaStream_t st) {
    constexpr int TZ = 16;
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    if (!configured[dev & 63]) {
        SB_CUDA(cudaFuncSetAttribute(stencil2d_step<R, VD, TZ>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        configured[dev & 63] = true;
    }
    const int rec_blocks = (int)((P.rec.count + kWarps - 1) / kWarps);
    stencil2d_step<R, VD, TZ><<<P.ntiles + rec_blocks, kThreads, bytes, st>>>(P, un, uc, up, n,
                                                                               ring);
}

template <int R, bool VD>
static bool persistent_r(const Persist2D& P, cudaStream_t st) {
    constexpr int TZ = 16;
    constexpr int HX = (R + 3) & ~3;
    const int bytes = (VD ? 2 : 1) * (TZ + 2 * R) * (128 + 2 * HX) * 4;
    auto kernel = stencil2d_persistent<R, VD, TZ>;
    static std::atomic<bool> configured[64];  // zero (false) at start; set once per device
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

void step2d_launch_shots(const StepShot* shots, int nshots, int per_shot, int r, bool vd,
                         long long G, int i_un, int i_uc, int i_up, long long n,
                         long long ring_off, bool record, cudaStream_t st) {
#define SB_M(RR)                                                                             \
    case RR:                                                                                 \
        if (vd) batch::step_shots_r<RR, true>(shots, nshots, per_shot, G, i_un, i_uc, i_up, n, \
                                       ring_off, record, st);                                \
        else batch::step_shots_r<RR, false>(shots, nshots, per_shot, G, i_un, i_uc, i_up, n,  \
                                     ring_off, record, st);                                  \
        break;
    switch (r) { SB_M(1) SB_M(2) SB_M(3) SB_M(4) SB_M(5) SB_M(6) SB_M(7) SB_M(8) SB_M(9) SB_M(10) }
#undef SB_M
}

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
    const long long nzi = L.nz - 2 * r;
    // owner-computes sources and edges need r + 1 rows / columns in the first
    // and last tiles: the 16-row tiles start zoff rows above the interior,
    // the smallest offset that leaves both edge tiles r + 1 rows (the rows
    // of the grid's interior are the same whatever the offset)
    S.zoff = 0;
    for (int o = 0; o <= 15 - (r + 1) && nzi > 16; o++) {
        const long long last = (nzi + o) % 16;
        if (last == 0 || last >= r + 1) {
            S.zoff = o;
            break;
        }
    }
    S.tiles_x = (int)((L.nx - 2 * r + 127) / 128);
    S.tiles_z = (int)((nzi + S.zoff + 15) / 16);
    S.ntiles = S.tiles_x * S.tiles_z;
    const long long last_z = nzi + S.zoff - 16LL * (S.tiles_z - 1);
    const long long last_x = (L.nx - 2 * r) - 128LL * (S.tiles_x - 1);
    const long long first_z = std::min<long long>(nzi, 16 - S.zoff);
    const long long first_x = std::min<long long>(L.nx - 2 * r, 128);
    S.fused = last_z >= r + 1 && last_x >= r + 1 && first_z >= r + 1 && first_x >= r + 1;
    return true;
}

void step2d_launch(const Shot2D& S, bool vd, float* un, const float* uc, const float* up,
                   long long n, cudaStream_t st, float* ring) {
#define SB_ST(RR)                                                               \
    case RR:                                                                    \
        if (vd) batch::step_r<RR, true>(S, un, uc, up, n, ring, st);            \
        else batch::step_r<RR, false>(S, un, uc, up, n, ring, st);              \
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
        cudaFree(e->d_trec);
        cudaFree(e->d_tbrec);
        cudaFree(e->d_tsrc);
        cudaFree(e->words);
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
            (rows != 8 && rows != 16 && rows != 32 && rows != 64 && rows != 128 &&
             rows != 256))
            sw::batch::fail(SIMWAVE_E_ARGUMENT,
                            "space_order even in 2..20, rows 8, 16, 32, 64, 128 or 256");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        Engine* e = sw::batch::engine(b);
        e->tile_rows[space_order / 2] = rows;
        e->dirty = true;
    });
}

extern "C" int simwave_batch_set_depth(simwave_batch* b, int space_order, int depth) {
    return sw::batch::guarded([&] {
        if (!b || space_order < 2 || space_order > 20 || space_order % 2 || depth < 1 ||
            depth > 4 || (depth > 1 && !sw::batch::tb_supported(space_order / 2, depth)))
            sw::batch::fail(SIMWAVE_E_ARGUMENT,
                            "space_order even in 2..20; depth 1, or 2..4 with the tile "
                            "keeping >= 32 owned rows (depth x space_order / 2 <= 36) and "
                            ">= 64 owned columns");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        Engine* e = sw::batch::engine(b);
        e->depth[space_order / 2] = depth;
        e->dirty = true;
    });
}

extern "C" int simwave_batch_depth(simwave_batch* b, int shot_id, int* depth) {
    return sw::batch::guarded([&] {
        if (!b || !depth) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null argument");
        std::lock_guard<std::mutex> lock(sw::batch::g_mutex);
        Engine* e = sw::batch::engine(b);
        if (e->dirty) e->rebuild();
        for (const auto& h : e->shots)
            if (h.id == shot_id) {
                *depth = h.d.depth;
                return;
            }
        sw::batch::fail(SIMWAVE_E_ARGUMENT, "unknown shot id");
    });
}

extern "C" int simwave_batch_launches(simwave_batch* b, size_t* launches) {
    return sw::batch::guarded([&] {
        if (!b || !launches) sw::batch::fail(SIMWAVE_E_ARGUMENT, "null argument");
        *launches = sw::batch::engine(b)->kernel_launches;
    });
}
