// grn_noalloc.cu — allocation-free event weights.
//
// grn_event_weights keeps its screened work list in engine-owned device buffers
// that grow with the batch (cudaMalloc on first use of a larger batch). Some
// callers cannot allow that: an application whose device memory is owned by its
// own pool allocator and must not see foreign cudaMalloc/cudaFree calls, a
// service that sizes its memory once at start-up and must never hit an
// out-of-memory error (or the implicit device synchronisation of cudaFree) in the
// middle of a run. grn_event_weights_noalloc serves them: its scratch is a fixed
// file-scope device array of this library, so the call itself allocates nothing.
//
// Scratch layout: one 256-byte slot holding the counters of the screened work list and
// of the FP64 refinement list, then GRN_NOALLOC_MAX_POINTS 64-bit point indices for each
// list (16 MiB in total, resident on every device that loads the library until the
// process exits).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "grn_internal.cuh"

namespace {

constexpr size_t kCounterSlot = 256;
constexpr size_t kListBytes = static_cast<size_t>(GRN_NOALLOC_MAX_POINTS) * sizeof(int64_t);
constexpr size_t kScratchBytes = kCounterSlot + 2 * kListBytes;

// The scratch itself. Device code may name it directly; host code only ever uses
// the device address obtained from cudaGetSymbolAddress (the host-side symbol is
// a stand-in, not a device address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 128;
std::mutex    g_setup_mutex;
void         *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (the first call on a device does this set-up; it should come before any
// stream capture). The address stays valid for the life of the device's primary
// context: the library must not be used across a cudaDeviceReset.
cudaError_t scratch_address(int device, void **addr) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void             *p  = nullptr;
    const cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess) return ce;
    g_scratch_addr[device] = p;
  }
  *addr = g_scratch_addr[device];
  return cudaSuccess;
}

// A device (or managed) pointer of `device` itself: memory of another GPU would be read
// through peer addressing that nothing here enables.
bool on_device(const void *ptr, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace

namespace grn {
// Engine accessors implemented in grn_api.cu.
grn_status engine_noalloc_view(grn_engine *e, KArgs *args, int *device, cudaStream_t *stream,
                               int *loop_blocks, int *dim);
grn_status set_error(grn_status st, const char *msg);
}  // namespace grn

extern "C" grn_status grn_event_weights_noalloc(grn_engine *e, const double *u, int64_t n,
                                                int32_t dim, double *w_out, uint8_t *flags,
                                                int32_t prec) {
  grn::KArgs   args{};
  int          device = 0, loop_blocks = 0, edim = 0;
  cudaStream_t stream = nullptr;
  const grn_status st = grn::engine_noalloc_view(e, &args, &device, &stream, &loop_blocks, &edim);
  if (st != GRN_OK) return st;
  if (!u || !w_out) return grn::set_error(GRN_ERR_INVALID, "null argument");
  if (dim != edim)
    return grn::set_error(GRN_ERR_INVALID, ("grn_event_weights_noalloc: dim must equal "
                                            "grn_dim() = " + std::to_string(edim)).c_str());
  if (prec != GRN_PREC_FP64 && prec != GRN_PREC_MIXED)
    return grn::set_error(GRN_ERR_INVALID, "bad prec");
  if (n < 0 || n > GRN_NOALLOC_MAX_POINTS)
    return grn::set_error(GRN_ERR_INVALID,
                          "grn_event_weights_noalloc: n exceeds GRN_NOALLOC_MAX_POINTS "
                          "(1048576); split the batch or use grn_event_weights");
  if (n == 0) return GRN_OK;
  cudaError_t ce = cudaSetDevice(device);
  if (ce != cudaSuccess) return grn::set_error(GRN_ERR_CUDA, cudaGetErrorString(ce));
  if (!on_device(u, device) || !on_device(w_out, device) || (flags && !on_device(flags, device)))
    return grn::set_error(GRN_ERR_INVALID,
                          "grn_event_weights_noalloc: u, w_out and flags must be device "
                          "pointers on the engine's device (host staging would allocate)");
  void *base = nullptr;
  ce = scratch_address(device, &base);
  if (ce != cudaSuccess)
    return grn::set_error(GRN_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") +
                                         cudaGetErrorString(ce)).c_str());
  auto *count = static_cast<unsigned long long *>(base);
  auto *list  = reinterpret_cast<int64_t *>(static_cast<unsigned char *>(base) + kCounterSlot);
  auto *rlist = reinterpret_cast<int64_t *>(static_cast<unsigned char *>(base) + kCounterSlot +
                                            kListBytes);
  // launch_event_weights clears both counters (cudaMemsetAsync) before stage A. It is the
  // generic two-stage path (FP32 loop with FP64 refinement in MIXED) for every process;
  // grn_event_weights takes the record-mode loop for screened single-trajectory Regge
  // processes in MIXED, so there the two agree to the FP32-loop tolerance (1e-5), and
  // exactly in FP64.
  ce = grn::launch_event_weights(args, prec, u, n, dim, w_out, flags, list, rlist, count,
                                 loop_blocks, stream);
  if (ce != cudaSuccess) return grn::set_error(GRN_ERR_CUDA, cudaGetErrorString(ce));
  return GRN_OK;
}
