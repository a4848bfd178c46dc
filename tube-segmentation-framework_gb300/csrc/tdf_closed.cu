// tdf_closed.cu -- the circle-fitting TDF with the closed-form eigensolver
// (eigen mode 1, eigen_closed.cuh): the instantiation of the sweep kernels of
// tdf_kernels.cuh for it, in its own translation unit.
#include "tdf_kernels.cuh"

namespace tsf {

int launch_tdf_kernels_closed(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                              const CircleTable &tab, void *d_T, int unorm, float *d_R, cudaStream_t s, int kernel,
                              const uint4 *P, int fast_ok) {
    return launch_tdf_kernels<1>(d_field4, X, Y, Z, st, rmin, rmax, rstep, tab, d_T, unorm, d_R, s, kernel, P, fast_ok);
}

}  // namespace tsf
