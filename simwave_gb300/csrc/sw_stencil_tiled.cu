// sw_stencil_tiled.cu -- tiled stencil kernels (placeholder: generic path only).
#include "sw_tiled.h"

namespace sw {

template <typename T, int DIM, bool VD>
bool tiled_supported(const Layout&) { return false; }

template <typename T, int DIM, bool VD>
void launch_tiled(T*, const T*, const T*, const T*, const T*, const T*,
                  const Layout&, const Weights<T>&, T, T, cudaStream_t) {}

#define SW_INST(T, D, V)                                                      \
    template bool tiled_supported<T, D, V>(const Layout&);                    \
    template void launch_tiled<T, D, V>(T*, const T*, const T*, const T*,    \
                                        const T*, const T*, const Layout&,    \
                                        const Weights<T>&, T, T, cudaStream_t);
SW_INST(float, 2, false) SW_INST(float, 2, true) SW_INST(float, 3, false) SW_INST(float, 3, true)
SW_INST(double, 2, false) SW_INST(double, 2, true) SW_INST(double, 3, false) SW_INST(double, 3, true)

}  // namespace sw
