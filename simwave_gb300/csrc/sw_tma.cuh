// sw_tma.cuh -- PTX helpers of the tiled 3D stencils: mbarriers, TMA tensor
// loads and tensor-memory (TMEM) allocation, loads and stores (sm_100 and
// later, "a" targets). Internal linkage: each kernel file has its own copy.
#pragma once

#include <cuda.h>

namespace sw {
namespace {

constexpr unsigned kSpinLimit = 1u << 20;  // mbarrier polls before giving up

__host__ __device__ constexpr int round4(int r) { return (r + 3) & ~3; }

// The kernels' only shared memory: one dynamic region per CTA.
extern __shared__ __align__(128) float4 sw_dyn_smem[];

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

// ---- tensor memory ------------------------------------------------------------
//
// A CTA allocates a power-of-two number of TMEM columns (32..512) with one
// warp, publishes the base address through shared memory and frees the
// columns with the same warp before it exits. Warp w of the CTA reaches TMEM
// lanes 32 (w % 4) .. 32 (w % 4) + 31; with the 32x32b shape every thread
// reads and writes columns of its own lane, so a lane's columns serve as
// per-thread storage beside the register file.

// Whole warp: allocate `ncols` columns; the base address goes to *dst.
__device__ __forceinline__ void tmem_alloc(unsigned* dst, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// Whole warp (the allocating one): free the columns.
__device__ __forceinline__ void tmem_dealloc(unsigned base, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Loads of N consecutive columns of the thread's lane starting at `taddr`
// (asynchronous: the registers are valid after tmem_wait_ld).
template <int N>
__device__ __forceinline__ void tmem_ld(unsigned taddr, unsigned* r);

template <>
__device__ __forceinline__ void tmem_ld<4>(unsigned taddr, unsigned* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr)
                 : "memory");
}
template <>
__device__ __forceinline__ void tmem_ld<8>(unsigned taddr, unsigned* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}
template <>
__device__ __forceinline__ void tmem_ld<16>(unsigned taddr, unsigned* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
template <>
__device__ __forceinline__ void tmem_ld<32>(unsigned taddr, unsigned* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// Loads of N columns (N a multiple of 4, at most 60) in power-of-two pieces.
template <int N>
__device__ __forceinline__ void tmem_ld_cols(unsigned taddr, unsigned* r) {
    static_assert(N % 4 == 0 && N <= 60, "column count");
    constexpr int A = N >= 32 ? 32 : 0;
    constexpr int B = (N - A) >= 16 ? 16 : 0;
    constexpr int C = (N - A - B) >= 8 ? 8 : 0;
    constexpr int D = N - A - B - C;
    static_assert(D == 0 || D == 4, "pieces");
    if constexpr (A) tmem_ld<32>(taddr, r);
    if constexpr (B) tmem_ld<16>(taddr + A, r + A);
    if constexpr (C) tmem_ld<8>(taddr + A + B, r + A + B);
    if constexpr (D) tmem_ld<4>(taddr + A + B + C, r + A + B + C);
}

// Wait for the thread's outstanding TMEM loads; the registers of `r` are
// passed through so no use of them is scheduled before the wait.
template <int N>
__device__ __forceinline__ void tmem_wait_ld(unsigned* r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; i++) asm volatile("" : "+r"(r[i]));
}

__device__ __forceinline__ void tmem_st4(unsigned taddr, unsigned a, unsigned b, unsigned c,
                                         unsigned d) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr),
                 "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

__device__ __forceinline__ void tmem_wait_st() {
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace
}  // namespace sw
