// sw_common.cuh -- shared types of the simwave GB300 library.
//
// Grid layout on the device (the "pitched" layout): z slowest, the fastest
// axis (x in 2D, y in 3D) contiguous with a row pitch and a leading offset so
// that the first interior point of every row (index r) is 128-byte aligned:
//   2D: (i, j)    -> i * pitch + lead + j
//   3D: (i, j, k) -> i * plane + j * pitch + lead + k,  plane = nx * pitch
// A dense C-order array is the special case pitch = fastest extent, lead = 0.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>

namespace sw {

constexpr int kMaxRadius = 10;  // space order 20

struct Layout {
    int dim;        // 2 or 3
    int r;          // stencil radius = space_order / 2
    long long nz, nx, ny;  // extended shape (ny = 1 in 2D)
    long long pitch, lead;
    long long plane;  // elements per z-plane in 3D (nx * pitch); pitch in 2D
    long long slot;   // elements between wavefield slots

    __host__ __device__ long long nfast() const { return dim == 3 ? ny : nx; }
    __host__ __device__ long long nmid() const { return dim == 3 ? nx : nz; }
    __host__ __device__ long long nslow() const { return dim == 3 ? nz : 1; }
    // offset of (slow, mid, fast) indices
    __host__ __device__ long long at(long long s, long long m, long long f) const {
        return s * plane + m * pitch + lead + f;
    }
    // 3D (i=z, j=x, k=y); 2D (i=z, j=x)
    __host__ __device__ long long at3(long long i, long long j, long long k) const {
        return i * plane + j * pitch + lead + k;
    }
    __host__ __device__ long long at2(long long i, long long j) const {
        return i * pitch + lead + j;
    }
    // element stride of axis a (0 z, 1 x, 2 y)
    __host__ __device__ long long stride(int a) const {
        if (dim == 3) return a == 0 ? plane : (a == 1 ? pitch : 1);
        return a == 0 ? pitch : 1;
    }
    __host__ __device__ long long extent(int a) const {
        return a == 0 ? nz : (a == 1 ? nx : ny);
    }
    __host__ __device__ long long interior_points() const {
        long long p = (nz - 2 * r) * (nx - 2 * r);
        return dim == 3 ? p * (ny - 2 * r) : p;
    }
};

// Stencil weights. The weights are kept as given and each axis sum is scaled
// by 1/h^2 afterwards, like the reference's `sum / h^2`: folding 1/h^2 into
// every weight would round each weight differently, break the zero sum of
// the second-derivative weights and bias every point the same way
// (measured: 1.1e-4 relative L2 drift after 362 steps on the reference's
// 2D order-8 golden case, against 3e-6 for per-axis scaling).
template <typename T>
struct Weights {
    T c2[kMaxRadius + 1];  // second-derivative half weights [c0..cr]
    T c1[kMaxRadius + 1];  // first-derivative half weights (variable density)
    T ih2[3];              // per axis (z, x, y): 1 / h^2
    T s1[3];               // per axis 1 / (4 h^2) (variable density cross term)
};

// Weights of one problem: the half weights as given (c1 only for variable
// density) and, per axis, 1/h^2 and 1/(4 h^2) with h^2 formed in the model
// precision like the reference's `dz * dz`.
template <typename T>
inline Weights<T> make_weights(const T* c2, const T* c1, int r, double dz, double dx,
                               double dy) {
    Weights<T> W;
    std::memset(&W, 0, sizeof(W));
    const double h[3] = {dz, dx, dy};
    for (int k = 0; k <= r; k++) {
        W.c2[k] = c2[k];
        W.c1[k] = c1 ? c1[k] : T(0);
    }
    for (int a = 0; a < 3; a++) {
        const T h2 = (T)h[a] * (T)h[a];
        W.ih2[a] = (T)(1.0 / (double)h2);
        W.s1[a] = (T)(1.0 / (4.0 * (double)h2));
    }
    return W;
}

// Ragged KWS windows of a set of sources or receivers, in the reference's
// layout (source.py:123-159): per entry 2*dim interval ends, concatenated
// per-axis values, offsets[n+1].
template <typename T>
struct Windows {
    const size_t* interval;
    const T* values;
    const size_t* offsets;
    size_t count;
};

}  // namespace sw
