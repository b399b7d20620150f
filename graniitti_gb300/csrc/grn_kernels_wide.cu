// grn_kernels_wide.cu — the stage-A, record-build and histogram kernels for hypercubes of more
// than 8 dimensions (cascades, 4- and 6-body central states, forward excitation), instantiated in a
// translation unit of their own so that they compile in parallel with grn_kernels.cu. The
// same source is included with its launchers and its other kernels left out
// (GRN_KERNELS_WIDE); the launchers in grn_kernels.cu reach these instantiations through
// explicit instantiation declarations.
#define GRN_KERNELS_WIDE
#include "grn_kernels.cu"

namespace grn {

template __global__ void k_weights_born<kMaxDim>(
    const KArgs, const double *__restrict__, int64_t, int, double *__restrict__,
    uint8_t *__restrict__, int64_t *__restrict__, unsigned long long *__restrict__);
template __global__ void k_weights_born_rec<kMaxDim>(
    const KArgs, const double *__restrict__, int64_t, int, double *__restrict__,
    uint8_t *__restrict__, int64_t *__restrict__, float *__restrict__, double *__restrict__,
    unsigned long long *__restrict__);
template __global__ void k_hist_fill<kMaxDim>(
    const KArgs, const double *__restrict__, int, int, int64_t, uint64_t, uint32_t,
    const float *__restrict__, const double *__restrict__, const grn_hist_spec *__restrict__,
    const int *__restrict__, int, double *__restrict__, double *__restrict__,
    unsigned long long *__restrict__, unsigned long long *__restrict__);
template __global__ void k_vegas_born<kMaxDim>(
    const KArgs, const double *__restrict__, int, int, int64_t, uint64_t, uint32_t, int,
    double *__restrict__, unsigned long long *__restrict__, int64_t *__restrict__,
    double *__restrict__, double *__restrict__, int64_t, float *__restrict__,
    double *__restrict__, const float *__restrict__, const float *__restrict__);

}  // namespace grn
