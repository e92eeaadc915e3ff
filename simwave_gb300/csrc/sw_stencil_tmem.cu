// sw_stencil_tmem.cu -- 3D float32 stencils for orders 2..8 that stream
// along z with their planes staged by TMA, in two configurations:
//
//   SIMWAVE_POLICY_TMEM: the z queues in tensor memory. The thread's TMEM
//     lane keeps a ring of the 2R+1 planes z-R .. z+R of u and one of the
//     density (tcgen05.ld every plane, the ring head written with
//     tcgen05.st into the slot plane z-R leaves), so the rings cost no
//     registers and the density's z term needs no per-point array; the
//     damping mask comes from per-axis tables (below). 8 x rows per CTA, two
//     CTAs per SM. Least DRAM traffic of the 3D kernels: 23.3 B per point
//     update at order 8 with variable density (20 B algorithmic).
//   SIMWAVE_POLICY_STAGE_RELEASE: u queue in registers, density z term from
//     the per-point array gz formed once per run, damping from Q = damp dt /
//     (2 s); 12 x rows per CTA (up to 168 registers a thread), one CTA per SM,
//     six planes in flight, and no CTA barrier per plane: the last warp to
//     finish reading a stage loads the plane six ahead into it (shared-memory
//     acquire/release count, async-proxy fence), so warps drift by up to
//     five planes. The default for order 8 with variable density.
//
// Common tiling (as the packed kernel of sw_stencil_tiled.cu): a CTA of XW
// warps owns 128 (y) x XW (x) interior points and streams them along z over a
// chunk of planes; lane l of warp w holds the y points y0 .. y0+3 (y0 = R +
// 128 bx + 4 l) of the x row R + XW by + w. Per plane z the u tile and, with
// variable density, the density tile, each with an R-wide x/y halo, arrive in
// shared memory by TMA (cp.async.bulk.tensor, mbarrier completion): x and y
// derivatives; arithmetic on 64-bit pairs (.f32x2), the derivative sums in
// the reference's order (c0 u first, then k = 1 .. R), the combine in the
// order y, x, z.
//
// Damping from tables (TMEM policy): where the mask is nonzero, its value
// comes from per-axis tables at points with exactly one axis outside the box
// where the mask is zero (tables taken from the mask's centre lines and
// checked on the device against every such point), and from the mask itself
// where two or three axes are outside (the layer's edges and corners); a mask
// that fails the check is read at every point outside the box. The update is
// written with t = damp C / dt:
//   u_next = (2 - t) u - (1 - t) u_prev + C lap,
// the reference's 2/D u - N/D u_prev + value (dt^2/s)/D (D = 1 + q, N = 1 - q,
// q = damp dt / (2 s), C = (dt^2/s)/D, so 2/D = 2 - t and N/D = 1 - t); inside
// the box t = 0 and the arithmetic is the scalar update's.
//
// Every mbarrier wait is bounded; on expiry the CTA records an error code,
// drains its outstanding copies (also bounded), frees its TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <atomic>

#include "simwave_gb300.h"
#include "sw_pairs.cuh"
#include "sw_tiled.h"
#include "sw_tma.cuh"

namespace sw {

namespace {

__host__ __device__ constexpr int pow2_at_least(int n) {
    int p = 32;
    while (p < n) p *= 2;
    return p;
}

template <int R, bool VD, int XW, int UQ, int RZ, int ST>
struct TmTile {
    static constexpr int HY = round4(R);
    static constexpr int TW = 128 + 2 * HY;  // floats per tile row
    static constexpr int TH = XW + 2 * R;    // tile rows
    static constexpr int ELEMS = TW * TH;
    static constexpr int BYTES = ELEMS * 4;  // one TMA box
    static constexpr int STRIDE = (ELEMS + 31) & ~31;
    static constexpr int NC = (2 * HY) / 4 + 1;  // float4 chunks of a y window
    static constexpr int QN = 2 * R + 1;         // planes in a ring
    static constexpr int QC = 4 * QN;            // TMEM columns of one ring
    // TMEM columns of one warp: the u ring and / or the density ring
    static constexpr int WC = (UQ == 1 ? QC : 0) + ((VD && RZ == 0) ? QC : 0);
    static constexpr int NCOLS = pow2_at_least((XW / 4) * WC);  // per CTA
    static constexpr int NF = VD ? 2 : 1;
    static constexpr int SF = NF * STRIDE;  // floats per stage
    static constexpr size_t SMEM = (size_t)ST * SF * 4 + 256;
};

struct TmBox {  // interior box where the damping mask is zero
    int z0, z1, x0, x1, y0, y1;
};

// The mask outside the zero box: per-axis tables (valid at points with one
// axis outside the box when `ok`) and the mask itself.
struct TmDamp {
    const float* tz;
    const float* tx;
    const float* ty;
    const float* damp;
    int ok;
};

__device__ __forceinline__ P2 pair_of(unsigned a, unsigned b) {
    P2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ void halves(P2 p, unsigned& a, unsigned& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(a), "=r"(b) : "l"(p.v));
}
__device__ __forceinline__ void tmem_st_v4(unsigned taddr, V4 v) {
    unsigned a, b, c, d;
    halves(v.lo, a, b);
    halves(v.hi, c, d);
    tmem_st4(taddr, a, b, c, d);
}
// plane slot s of a ring loaded into r
__device__ __forceinline__ V4 ring_at(const unsigned* r, int s) {
    return {pair_of(r[4 * s], r[4 * s + 1]), pair_of(r[4 * s + 2], r[4 * s + 3])};
}

// Template switches of the kernel:
//   UQ  u queue: 0 registers (slots static in the unrolled plane loop),
//       1 a ring in tensor memory;
//   RZ  density z term: 0 a ring in tensor memory, 2 the per-point array
//       gz = s1_z sum_k c1_k (rho(z+k) - rho(z-k)) formed once per run;
//   DM  damping: 0 the per-axis tables, 1 the per-point Q;
//   SY  stage release: 0 a CTA barrier per plane, 1 the last warp to finish
//       a stage refills it;
//   ST  stages (planes in flight).
template <int R, bool VD, int XW, int MINB, int UQ, int RZ, int DM, int SY, int ST>
__global__ void __launch_bounds__(32 * XW, MINB)
stencil3d_tmem(const __grid_constant__ CUtensorMap map_u,
               const __grid_constant__ CUtensorMap map_rho, float* un,
               const float* __restrict__ uc, const float* up,
               const float* __restrict__ coefC, const float* __restrict__ den,
               const float* __restrict__ gz, const float* __restrict__ coefQ, TmDamp F, Layout L,
               PairWeights PW, float inv_dt, int slot_cur, int zchunk, TmBox zb,
               int* __restrict__ err) {
    using TT = TmTile<R, VD, XW, UQ, RZ, ST>;
    static_assert(RZ == 0 || RZ == 2, "density z term");
    constexpr int S = ST;  // stages (planes in flight per field)
    constexpr int HY = TT::HY, TW = TT::TW, NC = TT::NC, QN = TT::QN, QC = TT::QC;
    constexpr int NF = TT::NF;
    constexpr bool TM_U = UQ == 1;
    constexpr bool TM_R = VD && RZ == 0;
    constexpr bool GZ_R = VD && RZ == 2;
    constexpr bool USE_TMEM = TM_U || TM_R;
    // stages: the u tile, then the density tile
    float* tiles = reinterpret_cast<float*>(sw_dyn_smem);  // [stages][SF]
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(tiles + S * TT::SF);
    int* words = reinterpret_cast<int*>(bars + S);
    int& s_abort = words[0];
    unsigned& s_tmem = *reinterpret_cast<unsigned*>(words + 1);
    // stage release without a CTA barrier (SY): per stage, the count of warps
    // that finished reading it and the plane index last loaded into it
    unsigned* rel = reinterpret_cast<unsigned*>(words + 2);
    int* last_it = words + 2 + S;
    if (smem_addr(tiles) & 127) {  // layout assumption broken: refuse
        if (threadIdx.x == 0) atomicExch(err, SIMWAVE_E_ARGUMENT);
        return;
    }
    // an earlier launch already failed: read once, so every warp of the CTA
    // leaves together (the TMEM allocation below is the CTA's)
    if (threadIdx.x == 0) s_abort = *(volatile int*)err;
    __syncthreads();
    if (s_abort) return;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int yb = R + blockIdx.x * 128;
    const int y0 = yb + 4 * lane;
    const int x = R + blockIdx.y * XW + warp;
    const int zbeg = R + blockIdx.z * zchunk;
    const int zend = min(zbeg + zchunk, (int)L.nz - R);
    if (zbeg >= zend) return;  // uniform over the CTA, before any allocation
    const int ylim = (int)L.ny - R;
    const bool any = x < (int)L.nx - R && y0 < ylim;
    const bool full = any && y0 + 3 < ylim;
    // threads past the interior load from the last interior row / chunk
    // (inside the grid) instead of selecting zeros; only their stores are
    // masked
    const int xl = min(x, (int)L.nx - R - 1);
    const int yl = min(y0, R + 4 * ((ylim - 1 - R) / 4));
    const int offl = xl * (int)L.pitch + (int)L.lead + yl;
    const int dstore = (x * (int)L.pitch + (int)L.lead + y0) - offl;  // store offset
    const int col0 = (int)L.lead + yb - HY;
    const int row0 = blockIdx.y * XW;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&bars[s], 1);
            rel[s] = 0;
            last_it[s] = -1;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (USE_TMEM && warp == 0) tmem_alloc(&s_tmem, TT::NCOLS);
    if (USE_TMEM) tmem_fence_before_sync();
    __syncthreads();
    if (USE_TMEM) tmem_fence_after_sync();
    // this warp's columns in its lane quadrant: the u ring, then the density ring
    const unsigned tbase = USE_TMEM ? s_tmem : 0u;
    const unsigned tu =
        tbase + ((unsigned)(32 * (warp & 3)) << 16) + (unsigned)((warp >> 2) * TT::WC);
    const unsigned tr = tu + (TM_U ? QC : 0);

    auto issue = [&](int plane, int stage) {
        last_it[stage] = plane - zbeg;
        float* sb = tiles + stage * TT::SF;
        mbar_expect_tx(&bars[stage], NF * TT::BYTES);
        tma_load_4d(sb, &map_u, &bars[stage], col0, row0, plane, slot_cur);
        if (VD) tma_load_4d(sb + TT::STRIDE, &map_rho, &bars[stage], col0, row0, plane, 0);
    };
    if (threadIdx.x == 0)
        for (int i = 0; i < S && zbeg + i < zend; i++) issue(zbeg + i, i);

    P2 w2[R + 1], w1[R + 1];
#pragma unroll
    for (int k = 0; k <= R; k++) {
        w2[k].v = PW.c2[k];
        w1[k].v = PW.c1[k];
    }
    auto vs = [&](int k, V4 a, V4 acc) -> V4 { return vfma(w2[k], a, acc); };
    auto vw = [&](bool first, int k, V4 a, V4 acc) -> V4 {
        return first ? vmul(w1[k], a) : vfma(w1[k], a, acc);
    };

    // queues and rings: plane p sits in slot (p - zbeg + R) mod QN
    V4 qu[TM_U ? 1 : QN];
    {
        const float* pu = uc + (long long)(zbeg - R) * L.plane + offl;
        const float* pr = den + (long long)(zbeg - R) * L.plane + offl;
#pragma unroll
        for (int j = 0; j < QN; j++) {
            const V4 a = ldg_v4(pu, true);
            if (TM_U) tmem_st_v4(tu + 4 * j, a);
            else qu[j] = a;
            if (TM_R) tmem_st_v4(tr + 4 * j, ldg_v4(pr, true));
            pu += L.plane;
            pr += L.plane;
        }
    }
    if (USE_TMEM) tmem_wait_st();

    // damping of the thread's points outside the zero box, looked up when a
    // plane needs it: with z inside the box, from the x or y table where
    // exactly one of x, y is outside, from the mask where both are (gzi);
    // with z outside, from the z table, or from the mask where x or y is
    // outside too (gzo). A mask that failed the table check is read at every
    // point outside the box.
    const bool xin = x >= zb.x0 && x < zb.x1;
    unsigned yinm = 0, gzi = 0, gzo = 0;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        const int yy = min(y0 + v, (int)L.ny - 1);
        const bool yo = !(yy >= zb.y0 && yy < zb.y1), xo = !xin;
        yinm |= (unsigned)!yo << v;
        gzi |= (unsigned)((xo && yo) || ((xo != yo) && !F.ok)) << v;
        gzo |= (unsigned)(xo || yo || !F.ok) << v;
    }
    const bool colin = xin && yinm == 15u;
    const unsigned flags = yinm | (gzi << 4) | (gzo << 8) | ((unsigned)xin << 12);

    // per-point operands of the next plane, fetched a plane ahead (p: the
    // plane's element offset of this thread's first point)
    V4 nprev, ncoef, ngz = vzero(), nq = vzero();
    bool nbox = true;
    auto fetch = [&](int zz, long long p) {
        nprev = ld_v4(up + p, true);
        ncoef = ldg_v4(coefC + p, true);
        if (GZ_R) ngz = ldg_v4(gz + p, true);
        nbox = colin && zz >= zb.z0 && zz < zb.z1;
        if (DM == 1) nq = ldg_v4(coefQ + p, !nbox);
    };
    long long zoff = (long long)zbeg * L.plane + offl;  // this plane's offset
    fetch(zbeg, zoff);
    int aborted_at = -1;

    auto plane_step = [&](const int z, const int J, const int m) -> bool {
        constexpr bool kStatic = QN % S == 0;
        const int it = QN * m + J;
        const int stage = kStatic ? J % S : it % S;
        const unsigned parity = kStatic ? (unsigned)(((QN / S) * m + J / S) & 1)
                                        : (unsigned)((it / S) & 1);
        auto slot = [&](int d) { return (J + R + d) % QN; };  // plane z + d
        if (SY && *(volatile int*)&s_abort) {  // another warp gave up
            aborted_at = it;
            return false;
        }
        const V4 vprev = nprev, vcoef = ncoef, vq = nq, vgz = ngz;
        const bool inbox = nbox;

        unsigned ur[TM_U ? QC : 1];
        if (TM_U) tmem_ld_cols<QC>(tu, ur);  // u ring (asynchronous)
        V4 hu = vzero(), hr = vzero();
        const bool more = z + 1 < zend;
        const long long pz = zoff;
        zoff += L.plane;
        if (more) {  // queue heads (plane z+R+1) and the next plane's operands
            const long long ph = pz + (long long)(R + 1) * L.plane;
            hu = ldg_v4(uc + ph, true);
            if (TM_R) hr = ldg_v4(den + ph, true);
            fetch(z + 1, zoff);
        }

        // z axis of u (c0 u first, then k = 1 .. R)
        if (TM_U) tmem_wait_ld<QC>(ur);
        auto uq = [&](int d) -> V4 { return TM_U ? ring_at(ur, slot(d)) : qu[slot(d)]; };
        const V4 u0 = uq(0);
        V4 sdz = vmul(w2[0], u0), fuz = vzero();
#pragma unroll
        for (int k = 1; k <= R; k++) {
            const V4 a = uq(k), b = uq(-k);
            sdz = vs(k, vadd(a, b), sdz);
            if (VD) fuz = vw(k == 1, k, vsub(a, b), fuz);
        }

        // warp-uniform, so the warp's tcgen05 operations stay converged
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&bars[stage], parity));
        if (!ok) s_abort = 1;
        if (ok) {
            const float* sb = tiles + stage * TT::SF;
            const float* tus = sb + (warp + R) * TW + 4 * lane;
            const float* trs = sb + TT::STRIDE + (warp + R) * TW + 4 * lane;
            // y axis of u on pairs: even offsets straight from the 16-byte
            // loads, odd offsets repacked once
            V4 sdy, fuy;
            {
                P2 ev[2 * NC], od[2 * NC - 1];
                YWindow<NC>::load(tus, ev, od);
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
                if (VD) fuy = {g[0], g[1]};
            }
            // x axis of u: rows x +- k of the tile
            V4 sdx = vmul(w2[0], u0), fux = vzero();
#pragma unroll
            for (int k = 1; k <= R; k++) {
                const V4 a = lds_v4(tus + k * TW + HY);
                const V4 b = lds_v4(tus - k * TW + HY);
                sdx = vs(k, vadd(a, b), sdx);
                if (VD) fux = vw(k == 1, k, vsub(a, b), fux);
            }
            // lap = y / hy^2 + x / hx^2 + z / hz^2
            V4 lap = vmul({PW.ih2[2]}, sdy);
            lap = vfma({PW.ih2[1]}, sdx, lap);
            lap = vfma({PW.ih2[0]}, sdz, lap);
            if (VD) {
                unsigned rr[TM_R ? QC : 1];
                if (TM_R) tmem_ld_cols<QC>(tr, rr);  // density ring (asynchronous)
                V4 rho0, fry, frx = vzero();
                {
                    P2 ev[2 * NC], od[2 * NC - 1];
                    YWindow<NC>::load(trs, ev, od);
                    rho0 = {ev[HY / 2], ev[HY / 2 + 1]};
                    P2 g[2];
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
#pragma unroll
                for (int k = 1; k <= R; k++) {
                    const V4 a = lds_v4(trs + k * TW + HY);
                    const V4 b = lds_v4(trs - k * TW + HY);
                    frx = vw(k == 1, k, vsub(a, b), frx);
                }
                // cross = fy gy / (4 hy^2) + fx gx / (4 hx^2) + fz gz / (4 hz^2)
                V4 cross = vmul({PW.s1[2]}, {mul2(fuy.lo, fry.lo), mul2(fuy.hi, fry.hi)});
                cross = vfma({PW.s1[1]}, {mul2(fux.lo, frx.lo), mul2(fux.hi, frx.hi)}, cross);
                if (GZ_R) {
                    cross = {fma2(fuz.lo, vgz.lo, cross.lo), fma2(fuz.hi, vgz.hi, cross.hi)};
                } else {
                    if (TM_R) tmem_wait_ld<QC>(rr);
                    auto rq = [&](int d) -> V4 { return ring_at(rr, slot(d)); };
                    V4 frz = vzero();
#pragma unroll
                    for (int k = 1; k <= R; k++) frz = vw(k == 1, k, vsub(rq(k), rq(-k)), frz);
                    cross = vfma({PW.s1[0]}, {mul2(fuz.lo, frz.lo), mul2(fuz.hi, frz.hi)}, cross);
                }
                const float4 rr4 = to_f4(rho0);
                const V4 inv = from_f4(make_float4(rcp_approx(rr4.x), rcp_approx(rr4.y),
                                                   rcp_approx(rr4.z), rcp_approx(rr4.w)));
                // lap -= cross / rho
                lap = {fma2(sub2({0ull}, cross.lo), inv.lo, lap.lo),
                       fma2(sub2({0ull}, cross.hi), inv.hi, lap.hi)};
            }
            // a = (2 - t) u - (1 - t) u_prev, t = damp C / dt (0 in the box)
            V4 a;
            if (DM == 1) {
                // with Q: a = 2 u - (1 - q) u_prev, divided by 1 + q off the box
                const P2 one{PW.one};
                a = {fma2(sub2(vq.lo, one), vprev.lo, add2(u0.lo, u0.lo)),
                     fma2(sub2(vq.hi, one), vprev.hi, add2(u0.hi, u0.hi))};
                if (!inbox) {
                    const float4 qq = to_f4(vq);
                    const V4 rq = from_f4(make_float4(rcp_approx(1.f + qq.x), rcp_approx(1.f + qq.y),
                                                      rcp_approx(1.f + qq.z), rcp_approx(1.f + qq.w)));
                    a = {mul2(a.lo, rq.lo), mul2(a.hi, rq.hi)};
                }
            } else if (inbox) {
                const P2 m1{PW.minus_one};
                a = {fma2(m1, vprev.lo, add2(u0.lo, u0.lo)), fma2(m1, vprev.hi, add2(u0.hi, u0.hi))};
            } else {
                const bool zin = z >= zb.z0 && z < zb.z1;
                const unsigned need = (flags >> (zin ? 4 : 8)) & 15u;
                const V4 gm = ldg_v4(F.damp + pz, need != 0);
                const float4 g4 = to_f4(gm);
                const float gg[4] = {g4.x, g4.y, g4.z, g4.w};
                const bool xin_ = (flags >> 12) & 1u;
                const float tzv = (!zin && F.ok) ? __ldg(F.tz + z) : 0.f;
                const float txv = (zin && !xin_ && F.ok) ? __ldg(F.tx + xl) : 0.f;
                float d[4];
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const bool yo = !((flags >> v) & 1u);
                    const float face =
                        !zin ? tzv
                             : (!xin_ ? txv
                                      : ((yo && F.ok) ? __ldg(F.ty + min(y0 + v, (int)L.ny - 1))
                                                      : 0.f));
                    d[v] = ((need >> v) & 1u) ? gg[v] : face;
                }
                const V4 dv = from_f4(make_float4(d[0], d[1], d[2], d[3]));
                const P2 idt = pk(inv_dt, inv_dt);
                const V4 t = {mul2(mul2(dv.lo, vcoef.lo), idt), mul2(mul2(dv.hi, vcoef.hi), idt)};
                const P2 one{PW.one}, two{PW.two};
                a = {fma2(sub2(t.lo, one), vprev.lo, mul2(sub2(two, t.lo), u0.lo)),
                     fma2(sub2(t.hi, one), vprev.hi, mul2(sub2(two, t.hi), u0.hi))};
            }
            const V4 out = {fma2(lap.lo, vcoef.lo, a.lo), fma2(lap.hi, vcoef.hi, a.hi)};
            float* po = un + pz + dstore;
            if (full) {
                *reinterpret_cast<ulonglong2*>(po) = make_ulonglong2(out.lo.v, out.hi.v);
            } else if (any) {
                const float4 o = to_f4(out);
                const float ov[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
                for (int v = 0; v < 4; v++)
                    if (y0 + v < ylim) po[v] = ov[v];
            }
        }
        // queue heads into the slot plane z - R leaves
        if (more) {
            if (TM_U) tmem_st_v4(tu + 4 * slot(-R), hu);
            else qu[slot(-R)] = hu;
            if (TM_R) tmem_st_v4(tr + 4 * slot(-R), hr);
        }
        if (SY) {
            // the warp is done with the stage: the last warp to finish it
            // loads plane z + S into it
            __syncwarp();
            if (!ok) {
                aborted_at = it;
                return false;
            }
            if (lane == 0) {
                unsigned old;
                asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;"
                             : "=r"(old)
                             : "r"(smem_addr(&rel[stage]))
                             : "memory");
                if ((old + 1) % XW == 0 && z + S < zend) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue(z + S, stage);
                }
            }
        } else {
            __syncthreads();  // the stage is free again; abort is uniform here
            if (s_abort) {
                aborted_at = it;
                return false;
            }
            if (threadIdx.x == 0 && z + S < zend) issue(z + S, stage);
        }
        if (USE_TMEM) tmem_wait_st();  // the next plane's ring loads see the heads
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
    if (SY) __syncthreads();  // every warp has left the plane loop
    if (threadIdx.x == 0 && (s_abort || aborted_at >= 0)) {
        atomicExch(err, SIMWAVE_E_TIMEOUT);
        // drain the copies still in flight into this CTA's shared memory
        for (int s = 0; s < S; s++)
            if (last_it[s] >= 0) mbar_wait(&bars[s], (unsigned)((last_it[s] / S) & 1));
    }
    if (USE_TMEM) {
        // every warp is done with TMEM before the allocating warp frees it
        tmem_wait_st();
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        if (warp == 0) tmem_dealloc(tbase, TT::NCOLS);
    }
}

// ---- damping tables ------------------------------------------------------------

// tz[i] = damp(i, xc, yc), tx[j] = damp(zc, j, yc), ty[k] = damp(zc, xc, k) at
// the centre (zc, xc, yc) of the zero box `box` (device words z0, z1, x0, x1,
// y0, y1).
__global__ void damp_tables(const float* __restrict__ damp, Layout L, const int* box,
                            float* tz, float* tx, float* ty) {
    const int zc = (box[0] + box[1]) / 2, xc = (box[2] + box[3]) / 2, yc = (box[4] + box[5]) / 2;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
         t < L.nz + L.nx + L.ny; t += (long long)gridDim.x * blockDim.x) {
        if (t < L.nz)
            tz[t] = damp[L.at3(t, xc, yc)];
        else if (t < L.nz + L.nx)
            tx[t - L.nz] = damp[L.at3(zc, t - L.nz, yc)];
        else
            ty[t - L.nz - L.nx] = damp[L.at3(zc, xc, t - L.nz - L.nx)];
    }
}

// Checks every interior point with exactly one axis outside the zero box
// against that axis' table; a mismatch sets *bad.
__global__ void damp_tables_verify(const float* __restrict__ damp, Layout L, const int* box,
                                   const float* __restrict__ tz, const float* __restrict__ tx,
                                   const float* __restrict__ ty, int* bad) {
    const int r = L.r;
    const long long ny = L.ny - 2 * r, nx = L.nx - 2 * r, nz = L.nz - 2 * r;
    const long long total = nz * nx * ny;
    int mismatch = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = r + (int)(t % ny), j = r + (int)((t / ny) % nx), i = r + (int)(t / (ny * nx));
        const bool zo = i < box[0] || i >= box[1], xo = j < box[2] || j >= box[3],
                   yo = k < box[4] || k >= box[5];
        if ((int)zo + (int)xo + (int)yo != 1) continue;
        const float want = zo ? tz[i] : (xo ? tx[j] : ty[k]);
        mismatch |= damp[L.at3(i, j, k)] != want;
    }
    if (__syncthreads_or(mismatch) && threadIdx.x == 0) atomicOr(bad, 1);
}

int tm_sms() {
    static std::atomic<int> sms[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!sms[dev & 63]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms[dev & 63] = std::max(v, 1);
    }
    return sms[dev & 63];
}

// z chunk length: fill the machine in whole waves, counting the 2R-plane
// warm-up of every chunk as the cost of splitting, with chunks of at most
// kMaxChunk planes. Long chunks lose more than their warm-up saves: columns
// in the damping layer run slower than those inside, so over a long chunk
// neighbouring columns drift apart in z and the halo rows each reads of the
// other are no longer in L2. Measured on the 472^3 order-8 grid with
// variable density (ms per launch, 2 .. 64 chunks of 464 planes): 0.724,
// 0.606, 0.563, 0.545, 0.527 (12 chunks of 39 planes), 0.528, 0.530, 0.542,
// 0.570, 0.591; a wave of whole columns streaming all 464 planes, 0.640.
constexpr int kMaxChunk = 40;

int tm_chunk(int ty, int tx, int nzi, int R, int per_sm) {
    const long long slots = (long long)std::max(per_sm, 1) * tm_sms();
    const int zs_min = std::min((nzi + kMaxChunk - 1) / kMaxChunk, 64);
    int best = std::max(zs_min, 1);
    double best_cost = 1e300;
    for (int zs = std::max(zs_min, 1); zs <= std::max(32, zs_min) && zs <= nzi; zs++) {
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

// Shared memory of a CTA: the tiles, padded so that no more than MINB CTAs
// fit on an SM when they hold TMEM (their allocations must fit the SM's 512
// columns).
template <int R, bool VD, int XW, int MINB, int UQ, int RZ, int ST>
size_t tm_smem() {
    using TT = TmTile<R, VD, XW, UQ, RZ, ST>;
    static_assert(TT::WC == 0 || MINB * TT::NCOLS <= 512, "TMEM columns of the resident CTAs");
    if (TT::WC == 0) return TT::SMEM;
    const size_t per_sm = 228 * 1024;
    const size_t floor = per_sm / (MINB + 1) + 1024;
    return std::max(TT::SMEM, floor);
}

template <int R, bool VD, int XW, int MINB, int UQ, int RZ, int DM, int SY, int ST>
void launch_tm(float* un, const float* uc, const float* up, const float* coefC,
               const float* den, const Layout& L, const Weights<float>& W,
               const TiledContext& ctx, cudaStream_t st) {
    auto kernel = stencil3d_tmem<R, VD, XW, MINB, UQ, RZ, DM, SY, ST>;
    static std::atomic<bool> configured[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t smem = tm_smem<R, VD, XW, MINB, UQ, RZ, ST>();
    if (!configured[dev & 63]) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured[dev & 63] = true;
    }
    const int ty = (int)((L.ny - 2 * R + 127) / 128);
    const int tx = (int)((L.nx - 2 * R + XW - 1) / XW);
    const int nzi = (int)(L.nz - 2 * R);
    const int chunk = tm_chunk(ty, tx, nzi, R, MINB);
    const int zsplit = (nzi + chunk - 1) / chunk;
    const long long cur_slot = (uc - ctx.u_base) / ctx.slot_stride;
    TmBox zb{ctx.zero_box[0], ctx.zero_box[1], ctx.zero_box[2],
             ctx.zero_box[3], ctx.zero_box[4], ctx.zero_box[5]};
    TmDamp F{ctx.damp_tz, ctx.damp_tx, ctx.damp_ty, ctx.damp, ctx.damp_faces_ok};
    PairWeights PW = pair_weights(W);
    dim3 grid(ty, tx, zsplit);
    kernel<<<grid, 32 * XW, smem, st>>>(
        *reinterpret_cast<const CUtensorMap*>(ctx.map_u_tm),
        *reinterpret_cast<const CUtensorMap*>(ctx.map_rho_tm), un, uc, up, coefC, den,
        ctx.coefGz, ctx.coefQ, F, L, PW, ctx.inv_dt, (int)cur_slot, chunk, zb, ctx.err);
}

}  // namespace

int tmem_rows(int policy) { return policy == SIMWAVE_POLICY_STAGE_RELEASE ? 12 : 8; }

void damp_face_tables(const float* damp, const Layout& L, const int* box, float* tz,
                      float* tx, float* ty, int* bad, cudaStream_t st) {
    cudaMemsetAsync(bad, 0, sizeof(int), st);
    damp_tables<<<(unsigned)((L.nz + L.nx + L.ny + 255) / 256), 256, 0, st>>>(damp, L, box, tz,
                                                                            tx, ty);
    damp_tables_verify<<<tm_sms() * 4, 256, 0, st>>>(damp, L, box, tz, tx, ty, bad);
}

bool tmem_launch(const TiledContext& ctx, int policy, bool vd, float* un, const float* uc,
                 const float* up, const float* coefC, const float* den, const Layout& L,
                 const Weights<float>& W, cudaStream_t st) {
    if (!ctx.tm || L.r > 4 || ctx.tm_rows != tmem_rows(policy)) return false;
    if (policy == SIMWAVE_POLICY_STAGE_RELEASE) {
        if (vd && !ctx.coefGz) return false;  // the run formed no gz
#define SW_SR(RR)                                                                          \
    case RR:                                                                               \
        if (vd) launch_tm<RR, true, 12, 1, 0, 2, 1, 1, 6>(un, uc, up, coefC, den, L, W, ctx, st);  \
        else launch_tm<RR, false, 12, 1, 0, 2, 1, 1, 6>(un, uc, up, coefC, den, L, W, ctx, st);    \
        return true;
        switch (L.r) { SW_SR(1) SW_SR(2) SW_SR(3) SW_SR(4) }
#undef SW_SR
        return false;
    }
    if (!ctx.damp || !ctx.damp_tz) return false;
#define SW_TM(RR)                                                                          \
    case RR:                                                                               \
        if (vd) launch_tm<RR, true, 8, 2, 1, 0, 0, 0, 3>(un, uc, up, coefC, den, L, W, ctx, st);   \
        else launch_tm<RR, false, 8, 2, 1, 0, 0, 0, 3>(un, uc, up, coefC, den, L, W, ctx, st);     \
        return true;
    switch (L.r) { SW_TM(1) SW_TM(2) SW_TM(3) SW_TM(4) }
#undef SW_TM
    return false;
}

}  // namespace sw
