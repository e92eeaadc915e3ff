// sw_tile2d.cuh -- the 2D tiled stencil body shared by the single-shot,
// batch and gradient kernels.
#pragma once

#include "sw_kernels.cuh"
#include "sw_pairs.cuh"

namespace sw {
namespace batch {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

// ---- tiled 2D stencil -------------------------------------------------------------
// Tile: 128 x-points (32 lanes x float4) by TZ rows; u (and rho) with an R
// halo staged in shared memory by plain 16-byte loads; each warp computes
// TZ / 8 rows. Same arithmetic as the 3D tiled kernels: unscaled half
// weights, per-axis 1/h^2, per-point C and Q coefficients. The tiles start
// `zoff` rows above the interior (the first one holds TZ - zoff rows), so
// that the first and last tiles of a shot can both be made tall enough.
template <int R, bool VD, int TZ>
__device__ __forceinline__ void stencil2d_tile(float* tile, const Layout& L, float* un,
                                               const float* uc, const float* up,
                                               const float* C, const float* Q,
                                               const float* den, const Weights<float>& W,
                                               const int* zb, int tz, int tx, int zoff = 0) {
    constexpr int HX = (R + 3) & ~3;
    constexpr int TW = 128 + 2 * HX;   // floats per tile row
    constexpr int TH = TZ + 2 * R;     // tile rows
    constexpr int NF = VD ? 2 : 1;
    constexpr int NC = (4 + 2 * HX) / 4;             // 16-byte chunks of an x window
    constexpr int RPW = (TZ + kWarps - 1) / kWarps;  // rows per warp
    const int z0 = R + tz * TZ - zoff;      // first row of the tile
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
        const bool ok = warp + j * kWarps < TZ && z >= R && z < nz - R && x < xlim;
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
            if (z >= 0 && z < nz && col + 3 < pitch)
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
        if (rr >= TZ || z < R || z >= nz - R || x >= xlim) continue;
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

// ---- adjoint of the variable-density 2D operator -------------------------------
// The adjoint update of the velocity gradient (sw_gradient.cu) with variable
// density: the forward's A u = L u - sum_a G_a fd_a(u) (G_a = fd_a(rho) /
// (4 h_a^2 rho) at interior points, zero elsewhere; fd_a the first
// difference with the c1 weights) has the transpose
//   A^T nu = L nu + sum_a fd_a(G_a nu)
// for nu supported on the interior (zero halo). The tile stages nu and the
// products Gz nu, Gx nu with an R halo, then writes
//   nu_next = (2 nu - N nu_prev) / D + C A^T nu
// in the forward tile's arithmetic (C, Q per point, Q skipped in the box).
template <int R, int TZ>
__device__ __forceinline__ void adjoint2d_density_tile(float* tile, const Layout& L, float* un,
                                                       const float* uc, const float* up,
                                                       const float* C, const float* Q,
                                                       const float* Gz, const float* Gx,
                                                       const Weights<float>& W, const int* zb,
                                                       int tz, int tx, int zoff = 0) {
    constexpr int HX = (R + 3) & ~3;
    constexpr int TW = 128 + 2 * HX;
    constexpr int TH = TZ + 2 * R;
    constexpr int NC = (4 + 2 * HX) / 4;
    constexpr int RPW = (TZ + kWarps - 1) / kWarps;
    const int z0 = R + tz * TZ - zoff;
    const int x0 = R + tx * 128;
    const int col0 = (int)L.lead + x0 - HX;
    const int pitch = (int)L.pitch;
    const int nz = (int)L.nz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = x0 + 4 * lane;
    const int xlim = (int)L.nx - R;
    const bool xbox = x >= zb[2] && x + 3 < zb[3];

    V4 cc[RPW], pv[RPW], qq[RPW];
    bool qzero[RPW];
#pragma unroll
    for (int j = 0; j < RPW; j++) {
        const int z = z0 + warp + j * kWarps;
        const bool ok = warp + j * kWarps < TZ && z >= R && z < nz - R && x < xlim;
        const long long p = (long long)z * pitch + L.lead + x;
        qzero[j] = xbox && z >= zb[0] && z < zb[1];
        cc[j] = ldg_v4(C + p, ok);
        pv[j] = ld_v4(up + p, ok);
        qq[j] = ldg_v4(Q + p, ok && !qzero[j]);
    }

    // stage nu, Gz nu and Gx nu: rows z0-R .. z0+TZ+R-1 (guarded)
    constexpr int CH = TW / 4;
    float* tn = tile;
    float* tpz = tile + TH * TW;
    float* tpx = tile + 2 * TH * TW;
    for (int i = threadIdx.x; i < TH * CH; i += kThreads) {
        const int row = i / CH, ch = i - row * CH;
        const int z = z0 - R + row;
        const int col = col0 + 4 * ch;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f), gz = v, gx = v;
        if (z >= 0 && z < nz && col + 3 < pitch) {
            const long long o = (long long)z * pitch + col;
            v = *reinterpret_cast<const float4*>(uc + o);
            gz = __ldg(reinterpret_cast<const float4*>(Gz + o));
            gx = __ldg(reinterpret_cast<const float4*>(Gx + o));
        }
        *reinterpret_cast<float4*>(tn + row * TW + 4 * ch) = v;
        *reinterpret_cast<float4*>(tpz + row * TW + 4 * ch) =
            make_float4(gz.x * v.x, gz.y * v.y, gz.z * v.z, gz.w * v.w);
        *reinterpret_cast<float4*>(tpx + row * TW + 4 * ch) =
            make_float4(gx.x * v.x, gx.y * v.y, gx.z * v.z, gx.w * v.w);
    }
    __syncthreads();

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
        if (rr >= TZ || z < R || z >= nz - R || x >= xlim) continue;
        const int o = (rr + R) * TW + 4 * lane;  // row z, chunk start
        const long long p = (long long)z * pitch + L.lead + x;
        // z axis: L on nu, fd of Gz nu
        const V4 u0 = lds_v4(tn + o + HX);
        V4 sz = vmul(w2[0], u0), dz;
#pragma unroll
        for (int k = 1; k <= R; k++) {
            sz = vfma(w2[k], vadd(lds_v4(tn + o + k * TW + HX), lds_v4(tn + o - k * TW + HX)), sz);
            const V4 d = vsub(lds_v4(tpz + o + k * TW + HX), lds_v4(tpz + o - k * TW + HX));
            dz = k == 1 ? vmul(w1[k], d) : vfma(w1[k], d, dz);
        }
        // x axis: L on nu, fd of Gx nu (window pairs as in the forward tile)
        V4 sx, dx;
        {
            P2 ev[2 * NC], od[2 * NC - 1];
            YWindow<NC>::load(tn + o, ev, od);
            P2 sh[2], gh[2];
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
            YWindow<NC>::load(tpx + o, ev, od);
#pragma unroll
            for (int h = 0; h < 2; h++) {
#pragma unroll
                for (int k = 1; k <= R; k++) {
                    const P2 a = YWindow<NC>::at(ev, od, HX + 2 * h + k);
                    const P2 b = YWindow<NC>::at(ev, od, HX + 2 * h - k);
                    gh[h] = k == 1 ? mul2(w1[k], sub2(a, b)) : fma2(w1[k], sub2(a, b), gh[h]);
                }
            }
            dx = {gh[0], gh[1]};
        }
        // A^T nu = L nu + fd_x(Gx nu) + fd_z(Gz nu)
        V4 lap = vfma(ihz, sz, vmul(ihx, sx));
        lap = vadd(lap, vadd(dx, dz));
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
            const float4 ov = to_f4(out);
            const float oa[4] = {ov.x, ov.y, ov.z, ov.w};
#pragma unroll
            for (int v = 0; v < 4; v++)
                if (x + v < xlim) un[p + v] = oa[v];
        }
    }
}

}  // namespace batch
}  // namespace sw
