// sw_tiled.h -- entry points of the tiled stencil kernels (sw_stencil_tiled.cu).
#pragma once

#include "sw_common.cuh"

namespace sw {

// True when the tiled kernel handles this (precision, dimension, density,
// layout); otherwise the generic kernel runs.
template <typename T, int DIM, bool VD>
bool tiled_supported(const Layout& L);

template <typename T, int DIM, bool VD>
void launch_tiled(T* un, const T* uc, const T* up, const T* vel, const T* den,
                  const T* damp, const Layout& L, const Weights<T>& W, T dt,
                  T dt2, cudaStream_t st);

}  // namespace sw
