// sw_pairs.cuh -- packed float pairs for the f32 stencils on sm_100 and later.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include "sw_common.cuh"

namespace sw {

// ---- packed-pair arithmetic (.f32x2, sm_100 and later) -----------------------
//
// Two consecutive y points share one 64-bit register pair; add, sub, mul and
// fma on .f32x2 round each half exactly like the scalar instruction, so a
// kernel written on pairs computes what the float4 kernel computes with half
// the arithmetic instructions. Weights are passed pre-duplicated ({w, w}).

struct P2 {
    unsigned long long v;
};
struct V4 {  // points y0, y0+1 (lo) and y0+2, y0+3 (hi)
    P2 lo, hi;
};

__device__ __forceinline__ P2 pk(float a, float b) {
    P2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpk(P2 p, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(p.v));
}
__device__ __forceinline__ P2 add2(P2 a, P2 b) {
    P2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ P2 sub2(P2 a, P2 b) {
    P2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ P2 mul2(P2 a, P2 b) {
    P2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ P2 fma2(P2 a, P2 b, P2 c) {
    P2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ V4 vadd(V4 a, V4 b) { return {add2(a.lo, b.lo), add2(a.hi, b.hi)}; }
__device__ __forceinline__ V4 vsub(V4 a, V4 b) { return {sub2(a.lo, b.lo), sub2(a.hi, b.hi)}; }
__device__ __forceinline__ V4 vmul(P2 w, V4 a) { return {mul2(w, a.lo), mul2(w, a.hi)}; }
__device__ __forceinline__ V4 vfma(P2 w, V4 a, V4 c) {
    return {fma2(w, a.lo, c.lo), fma2(w, a.hi, c.hi)};
}
__device__ __forceinline__ V4 vzero() { return {{0ull}, {0ull}}; }

// 16-byte loads and stores of 4 consecutive points as two pairs
__device__ __forceinline__ V4 ldg_v4(const float* p, bool any) {
    if (!any) return vzero();
    const ulonglong2 t = __ldg(reinterpret_cast<const ulonglong2*>(p));
    return {{t.x}, {t.y}};
}
__device__ __forceinline__ V4 ld_v4(const float* p, bool any) {
    if (!any) return vzero();
    const ulonglong2 t = *reinterpret_cast<const ulonglong2*>(p);
    return {{t.x}, {t.y}};
}
__device__ __forceinline__ V4 lds_v4(const void* p) {
    V4 r;
    asm volatile("ld.shared.v2.b64 {%0, %1}, [%2];"
                 : "=l"(r.lo.v), "=l"(r.hi.v)
                 : "r"(static_cast<unsigned>(__cvta_generic_to_shared(p)))
                 : "memory");
    return r;
}
__device__ __forceinline__ void sts_v4(void* p, V4 v) {
    asm volatile("st.shared.v2.b64 [%0], {%1, %2};" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(p))), "l"(v.lo.v),
                 "l"(v.hi.v)
                 : "memory");
}
__device__ __forceinline__ float4 to_f4(V4 v) {
    float4 r;
    unpk(v.lo, r.x, r.y);
    unpk(v.hi, r.z, r.w);
    return r;
}
__device__ __forceinline__ V4 from_f4(float4 f) { return {pk(f.x, f.y), pk(f.z, f.w)}; }

// The y window of a thread (4 * NC values from the tile row) as 64-bit
// pairs: ev[j] = (w[2j], w[2j+1]) straight from the 16-byte loads, od[j] =
// (w[2j+1], w[2j+2]) repacked. at(s) is the pair starting at offset s.
template <int NC>
struct YWindow {
    __device__ __forceinline__ static void load(const float* t, P2* ev, P2* od) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const V4 q = lds_v4(t + 4 * c);
            ev[2 * c] = q.lo;
            ev[2 * c + 1] = q.hi;
        }
#pragma unroll
        for (int j = 0; j < 2 * NC - 1; j++) {
            float a, b, c, d;
            unpk(ev[j], a, b);
            unpk(ev[j + 1], c, d);
            od[j] = pk(b, c);
        }
    }
    __device__ __forceinline__ static P2 at(const P2* ev, const P2* od, int s) {
        return (s & 1) ? od[s >> 1] : ev[s >> 1];
    }
};

// Approximate reciprocal (the value __fdividef(1, x) uses, without its
// range test); for the density and 1 + q, both far from the range limits.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Weights duplicated into pairs (kernel parameters).
struct PairWeights {
    unsigned long long c2[kMaxRadius + 1], c1[kMaxRadius + 1], ih2[3], s1[3], one, two,
        minus_one;
};

inline PairWeights pair_weights(const Weights<float>& W) {
    auto dup = [](float w) {
        unsigned u;
        std::memcpy(&u, &w, 4);
        return ((unsigned long long)u << 32) | u;
    };
    PairWeights P;
    for (int k = 0; k <= kMaxRadius; k++) {
        P.c2[k] = dup(W.c2[k]);
        P.c1[k] = dup(W.c1[k]);
    }
    for (int a = 0; a < 3; a++) {
        P.ih2[a] = dup(W.ih2[a]);
        P.s1[a] = dup(W.s1[a]);
    }
    P.one = dup(1.0f);
    P.two = dup(2.0f);
    P.minus_one = dup(-1.0f);
    return P;
}

}  // namespace sw
