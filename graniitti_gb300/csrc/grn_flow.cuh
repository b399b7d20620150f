// grn_flow.cuh — launch interface of the coupling-layer spline flow (grn_flow.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace grn {
namespace flow {

constexpr int kDim   = 8;                  // hypercube dimension
constexpr int kDA    = kDim / 2;           // conditioning / transformed coordinates per layer
constexpr int kBins  = 16;                 // spline bins
constexpr int kRaw   = 3 * kBins + 1;      // widths, heights, knot derivatives
constexpr int kRawP  = 56;                 // padded to whole 8-column MMA tiles
constexpr int kHid   = 128;                // MLP width
constexpr int kNOut  = kDA * kRaw;         // 196
constexpr int kNOutP = kDA * kRawP;        // 224
constexpr int kLayerParams = kDA * kHid + kHid + kHid * kHid + kHid + kHid * kNOut + kNOut;
constexpr int kMaxLayers   = 12;

}  // namespace flow

size_t      flow_w2p_elems(int layers);  // BF16 elements of the padded W2 copies (backward)
size_t      flow_w3p_elems(int layers);  // BF16 elements of the padded W3 copies (backward)
size_t      flow_w2c_elems(int layers);  // BF16 elements of the canonical W2^T copies (forward)
size_t      flow_w3c_elems(int layers);  // BF16 elements of the canonical W3^T copies (forward)
cudaError_t launch_flow_pack(const float *theta, int layers, void *w2p, void *w3p, void *w2c,
                             void *w3c, cudaStream_t st);
// mode 0: density direction (xin = points x, xout = z); mode 1: sampling direction
// (xin = z or, when null, Philox uniforms of points first..first+n-1 with key seed and
// stream id `stream`; xout = x). Arrays are dimension-major with leading dimension
// ld_in / ld_out. lq receives log q(x). xs_store (density mode, may be null) receives
// each layer's input, layers x 8 x n. err: device int set to 1 when a bounded wait of
// the kernel gave up (its outputs are then invalid). first_wait_polls >= 0: the poll limit
// of each CTA's first wait (on its first weight copy) instead of the default.
cudaError_t launch_flow_forward(int mode, const float *theta, const void *w2c, const void *w3c,
                                int layers, const float *xin, int64_t ld_in, int64_t n,
                                uint64_t seed, uint32_t stream, int64_t first, float *xout,
                                int64_t ld_out, float *lq, float *xs_store, int *err,
                                cudaStream_t st, int first_wait_polls = -1);
// Loss over n points and its gradient: grad <- d(sum_i l_i / n)/d theta and loss_sum <-
// sum_i l_i, both deterministic (each backward block accumulates a private slice of part,
// flow_backward_slices() x parameters floats, and loss_part, flow_backward_slices()
// doubles; the slices are summed in block order). kind 1: l = coef exp(-log q);
// kind 0: l = -coef log q.
int         flow_backward_slices();
cudaError_t launch_flow_backward(const float *theta, const void *w2p, const void *w3p, int layers,
                                 const float *xs, const float *lq, const float *coef, int64_t n,
                                 int kind, float *part, double *loss_part, float *grad,
                                 double *loss_sum, cudaStream_t st);
cudaError_t launch_flow_adam(float *theta, float *m, float *v, const float *grad, int64_t n,
                             float lr_t, float b1, float b2, float eps_t, cudaStream_t st);
// Training coefficients from the weights f of a pass and the sampling log density
// lq0 (null = uniform): kind 1: coef = f^2 exp(lq0) / norm; kind 0: coef = f / norm.
cudaError_t launch_flow_coef(const double *f, const float *lq0, int64_t n, int kind, double norm,
                             float *coef, cudaStream_t st);
// Philox uniforms of points first..first+n-1 as FP32, rounded down (dimension-major,
// leading dimension ld); lq (may be null) <- 0.
cudaError_t launch_flow_uniform(uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                                int64_t ld, float *u, float *lq, cudaStream_t st);
// lq <- log(alpha + (1 - alpha) exp(lq)): the defensive mixture with the uniform density.
cudaError_t launch_flow_mix(float *lq, int64_t n, double alpha, cudaStream_t st);
// grad[i] = sum of the nslices slices of part (np floats each) in slice order; loss = sum of
// loss_part[0..nslices).
cudaError_t launch_flow_grad_reduce(const float *part, int nslices, int64_t np, float *grad,
                                    const double *loss_part, double *loss, cudaStream_t st);

// ---------------------------------------------------------------------------
// The same flow for other shapes (grn_flow_wide.cu): dimension D = 8 or 14, MLP width H = 128
// or 256 ((8, 128) is served by the kernels above). Parameters per layer
// flow_layer_params(D, H), same layout. BF16 operand copies (element counts for all layers):
struct FlowWideSizes {
  size_t w2c, w3c;       // forward: 64-column chunks in the K-major canonical layout
  size_t w2t, w2r;       // backward: W2 as [out][in] and [in][out] row-major
  size_t w3t, w3r;       // backward: W3 as [56 j + r][h] and [h][o] row-major
};
struct FlowWideBufs {
  void *w2c, *w3c, *w2t, *w2r, *w3t, *w3r;
};
bool          flow_wide_supported(int dim, int hidden);
int64_t       flow_layer_params(int dim, int hidden);
FlowWideSizes flow_wide_sizes(int dim, int hidden, int layers);
cudaError_t   launch_wflow_pack(int dim, int hidden, const float *theta, int layers,
                                const FlowWideBufs &b, cudaStream_t st);
// Same contract as launch_flow_forward (xs_store: layers x D x n).
cudaError_t   launch_wflow_forward(int dim, int hidden, int mode, const float *theta,
                                   const FlowWideBufs &b, int layers, const float *xin,
                                   int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream,
                                   int64_t first, float *xout, int64_t ld_out, float *lq,
                                   float *xs_store, int *err, cudaStream_t st);
// Same contract as launch_flow_backward (part: flow_backward_slices() slices).
cudaError_t   launch_wflow_backward(int dim, int hidden, const float *theta,
                                    const FlowWideBufs &b, int layers, const float *xs,
                                    const float *lq, const float *coef, int64_t n, int kind,
                                    float *part, double *loss_part, float *grad, double *loss,
                                    cudaStream_t st);
// launch_flow_uniform for D = 8 or 14.
cudaError_t   launch_flow_uniform_dim(int dim, uint64_t seed, uint32_t stream, int64_t first,
                                      int64_t n, int64_t ld, float *u, float *lq,
                                      cudaStream_t st);

}  // namespace grn
