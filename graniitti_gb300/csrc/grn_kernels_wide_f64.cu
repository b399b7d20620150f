// grn_kernels_wide_f64.cu — the FP64 loop-stage kernels for hypercubes of more than 8
// dimensions (cascades, 4- and 6-body central states, forward excitation), instantiated in a
// translation unit of their own so that they compile in parallel with grn_kernels.cu. The
// same source is included with its launchers and its other kernels left out
// (GRN_KERNELS_WIDE); the launchers in grn_kernels.cu reach these instantiations through
// explicit instantiation declarations.
#define GRN_KERNELS_WIDE
#include "grn_kernels.cu"

namespace grn {

template __global__ void k_weights_loop<double, kMaxDim>(
    const KArgs, const double *__restrict__, int, const int64_t *__restrict__,
    const unsigned long long *__restrict__, double *__restrict__, uint8_t *__restrict__,
    int64_t *__restrict__, unsigned long long *__restrict__);
template __global__ void k_vegas_loop<double, kMaxDim>(
    const KArgs, int, int, int, double *__restrict__, unsigned long long *__restrict__,
    const int64_t *__restrict__, const double *__restrict__, const double *__restrict__, int64_t,
    int64_t *__restrict__, const int64_t *__restrict__);

}  // namespace grn
