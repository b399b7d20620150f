// grn_internal.cuh — kernel launch interface shared by grn_kernels.cu and grn_api.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "grn_physics.cuh"

namespace grn {

// Everything a weight kernel needs, passed by value (kernel parameter space).
struct KArgs {
  grn_process_params P;
  Consts             K;
  // kt-loop node tables (device): per kt node j (kt_j, Re c_j, Im c_j) with
  // c_j = V_j * kt_j * A_eik(kt_j^2); per phi node i (cos phi_i, sin phi_i, U_i).
  const double *lc_kt;
  const double *lc_phi;
  int           n_kt_nodes;
  int           n_phi_nodes;
  double        loop_norm_re, loop_norm_im;  // i/(8 pi^2 s) * 9 h_phi h_kt / 64
  int           loop_pair;  // record-mode loop: 0 one event per thread, 1 two (packed FP32x2)
  // FP32 generic loop: an event whose estimated relative weight error exceeds refine_tol is
  // listed for the FP64 loop (0: never)
  double        refine_tol;
  int           born_blocks;  // grid of the VEGAS stage A (0: the default)
  int           gen_blocks;   // grid of the FP32 generic loop stage (0: one resident wave)
};

// Error estimate of the FP32 generic loop: |error of the loop sum| ~ kRefineKappa u
// sum_ij |U_i c_j| |A_ij| (u = 2^-24), calibrated on the tensor-pomeron structures, whose
// phi-rings cancel by up to 10^12 at small forward pT.
constexpr double kRefineKappa = 8.0;
constexpr double kRefineTol   = 1e-5;

constexpr int kMaxLoopNodes = 256;  // per axis
constexpr int kMaxDim       = 20;   // hypercube dimensions: 8 (2-body), 10 (excitation), 12, 14
                                    // (cascades, 4-body), 20 (6-body)

// Scalars accumulated per block by the VEGAS sampling kernel.
enum VegasScalar {
  VS_FSUM = 0,
  VS_F2SUM,
  VS_MAXF,
  VS_MAXW,
  VS_EVAL,
  VS_AMP_OK,
  VS_KIN_OK,
  VS_FID_OK,
  VS_VETO_OK,
  VS_NAN,
  VS_REFINED,  // events of the FP32 loop recomputed in FP64
  VS_COUNT
};
// acc layout: the VegasScalar accumulators, then the screened work-list length
// (acc[VS_COUNT]) and the length of the FP64 refinement list (acc[kAccRefine]).
constexpr int kAccRefine = VS_COUNT + 1;
constexpr int kAccSlots  = VS_COUNT + 2;

// Launchers (all stream-ordered, return cudaGetLastError of the launch).
// count: two counters (screened work list, FP64 refinement list rlist; both capacity n).
cudaError_t launch_event_weights(const KArgs &a, int prec, const double *u, int64_t n, int dim,
                                 double *w, uint8_t *flags, int64_t *list, int64_t *rlist,
                                 unsigned long long *count, int loop_blocks, cudaStream_t st);
int         loop_grid_blocks(int device);
cudaError_t launch_event_kinematics(const KArgs &a, const double *u, int64_t n, int dim,
                                    double *p4, double *ts, uint8_t *flags, cudaStream_t st);
cudaError_t launch_event_daughters(const KArgs &a, const double *u, int64_t n, int dim,
                                   double *pd, cudaStream_t st);
cudaError_t launch_uniforms(uint64_t seed, uint32_t stream, int64_t first, int64_t n, int dim,
                            double *out, cudaStream_t st);

cudaError_t launch_eikonal_density(const grn_soft_params &sp, double s, int n_bt, double2 *amp,
                                   double *mbt, cudaStream_t st);
cudaError_t launch_eikonal_screening(double s, int n_bt, const double *mbt, int n_kt2, double2 *g,
                                     double *msa, double *xs, cudaStream_t st);

cudaError_t launch_eikonal_xs(const double *mbt, int n_bt, double *xs, cudaStream_t st);

// VEGAS
int         vegas_grid_blocks(int device);
cudaError_t launch_vegas_grid_init(double *xmat, int bins, int dim, cudaStream_t st);
// One VEGAS pass in two stages; acc holds kAccSlots unsigned long long
// accumulators (see kAccRefine); the list arrays have
// capacity ncall (l_x: dim x ncall, dimension-major).
// rf/rd: loop records (record mode, see record_mode()); null for the point mode,
// in which stage B recomputes the tree level from the mapped points l_x. Record mode stores
// l_x too unless it is null (then its loop hands no events to the FP64 loop).
cudaError_t launch_vegas_born(const KArgs &a, const double *xmat, int bins, int dim, int64_t ncall,
                              uint64_t seed, uint32_t stream, int track_max, double *f_out,
                              unsigned long long *acc, int64_t *l_idx, double *l_x, double *l_vw,
                              float *rf, double *rd, cudaStream_t st, const float *fu = nullptr,
                              const float *flq = nullptr);
// fu / flq: points drawn from the flow (dimension-major, leading dimension ncall) and
// their log density; the VEGAS weight of a point is then vw(u) / q(u).
// The FP64 loop over the listed events an FP32 loop handed over (sel = r_list, its length
// acc[kAccRefine] read on the device; l_x the events' mapped points).
cudaError_t launch_vegas_loop_fp64(const KArgs &a, int bins, int dim, int64_t ncall,
                                   int track_max, double *f_out, unsigned long long *acc,
                                   const int64_t *l_idx, const double *l_x, const double *l_vw,
                                   const int64_t *r_list, cudaStream_t st);
// Stage B (nblocks: the record loop's grid; the generic loops size theirs from their own
// occupancy). r_list (capacity ncall): slots of the FP32 loop (generic, or record mode when l_x
// is stored) whose error estimate exceeds a.refine_tol, finished by an FP64 pass over them in
// the same call; in record mode fp64_pass = false leaves that pass to the caller
// (launch_vegas_loop_fp64 with the same arguments).
cudaError_t launch_vegas_loop(const KArgs &a, int prec, int bins, int dim, int64_t ncall,
                              int track_max, double *f_out, unsigned long long *acc,
                              const int64_t *l_idx, const double *l_x, const double *l_vw,
                              const float *rf, const double *rd, int64_t *r_list, int nblocks,
                              cudaStream_t st, bool fp64_pass = true);
// The f^2 histogram of a finished pass (bins x dim, the input of launch_vegas_refine) from its
// f array and its points (Philox (seed, stream), or the flow points fu with leading dimension
// ncall), summed in a fixed order: equal f arrays give equal histograms bit for bit.
// part: kHistBlocks * bins * dim doubles of scratch. vegas_hist_prepare() (once per device,
// outside stream capture) allows the shared memory of the largest histograms.
constexpr int kHistBlocks = 256;
cudaError_t vegas_hist_prepare();
cudaError_t launch_vegas_hist(int bins, int dim, int64_t ncall, uint64_t seed, uint32_t stream,
                              const float *fu, const double *f, double *part, double *f2mat,
                              cudaStream_t st);
// Record mode: screened, FP32 loop, single active trajectory.
bool        record_mode(const KArgs &a, int prec);
constexpr int kRecordDoubles = 4;
// The two stages of launch_event_weights_rec separately (the loop stage reads the list
// length from *count and may be re-run on the same records).
cudaError_t launch_weights_born_rec(const KArgs &a, const double *u, int64_t n, int dim, double *w,
                                    uint8_t *flags, int64_t *list, float *rf, double *rd,
                                    unsigned long long *count, cudaStream_t st);
// rlist non-null (capacity n, with u and dim): points whose error estimate exceeds
// a.refine_tol go to rlist (length count[1]) and get their weights from the FP64 loop.
cudaError_t launch_weights_loop_rec(const KArgs &a, int64_t n, double *w, uint8_t *flags,
                                    const int64_t *list, const float *rf, const double *rd,
                                    unsigned long long *count, int loop_blocks, cudaStream_t st,
                                    int64_t *rlist = nullptr, const double *u = nullptr,
                                    int dim = 0);
int         loop_rec_blocks_per_sm(int pair);
cudaError_t launch_event_weights_rec(const KArgs &a, const double *u, int64_t n, int dim,
                                     double *w, uint8_t *flags, int64_t *list, float *rf,
                                     double *rd, unsigned long long *count, int loop_blocks,
                                     cudaStream_t st, int64_t *rlist = nullptr);
constexpr int kVegasSumParts = 256;
cudaError_t launch_vegas_reduce(const double *f_out, int64_t ncall,
                                const unsigned long long *acc, double *part, double *sc,
                                cudaStream_t st);
cudaError_t launch_vegas_refine(double *xmat, double *f2mat, int bins, int dim, double lambda,
                                cudaStream_t st);
cudaError_t launch_vegas_points(const double *xmat, int bins, int dim, uint64_t seed,
                                uint32_t stream, const int64_t *idx, int64_t n, double *u_out,
                                cudaStream_t st, const float *fu = nullptr, int64_t fu_ld = 0);

// Unweighting
cudaError_t launch_unweight(const double *f, int64_t n, double fmax, uint64_t seed,
                            uint32_t stream, int *blk_counts, unsigned long long *overflow,
                            int64_t *idx_out, int64_t cap, int64_t *n_acc_dev, int nblocks,
                            cudaStream_t st);
int unweight_blocks(int64_t n);

// Several processes in one pass (grn_batch): one entry per process, in device memory.
constexpr int kMaxBatch = 8;
struct BatchProc {
  KArgs               A;
  const double       *xmat;
  int                 bins, dim;
  int64_t             ncall;
  uint64_t            seed;
  uint32_t            stream;     // Philox stream id of the pass (updated every pass)
  int                 track_max;  // integration pass: track the maximum weight
  double             *f_out, *hpart;  // f array; partial f^2 histograms (kHistBlocks x nh)
  unsigned long long *acc;
  int64_t            *l_idx;
  double             *l_x, *l_vw;
  float              *rf;
  double             *rd;
  int64_t            *r_list;      // record mode with refinement: events for the FP64 loop
  const float        *fu, *flq;    // flow points of the pass and their log density (or null)
  int                 blk0, blk1;  // stage-A blocks of this process: [blk0, blk1)
};
// The process table of a batch, copied into constant memory (stream-ordered).
cudaError_t upload_batch_procs(const BatchProc *h_procs, int np, cudaStream_t st);
// Stage A of every process in one launch (block b serves the process whose range holds b).
// max_dim / max_nh: largest hypercube dimension / bins * dim of the batch's processes.
cudaError_t launch_batch_born(int np, int nblocks, int max_dim, int max_nh, cudaStream_t st);
// Stage B of the record-mode processes in one persistent launch (two events per thread):
// blocks take chunks of work from the counter (zeroed by the caller) over the listed events
// of those processes.
cudaError_t launch_batch_loop(int np, unsigned long long *counter, int nblocks, int max_nh,
                              cudaStream_t st);
// The f^2 histogram of member p of the uploaded table into f2mat (part: its q.hpart).
cudaError_t launch_batch_hist(int p, int bins, int dim, const double *part, double *f2mat,
                              cudaStream_t st);
// Resident blocks per SM of the VEGAS stage-A kernel and of the FP32 generic loop kernel for
// a hypercube dimension (bins x dim doubles of shared memory for stage A).
int vegas_born_blocks_per_sm(int dim, int bins);
int generic_loop_blocks_per_sm(int dim);
int         batch_loop_blocks(int device, int max_nh);

// On-the-fly histograms: every point e < ncall of the last pass with f[e] > 0 (its point from
// Philox (seed, stream) or the flow points fu, ld ncall; the grid xmat of that pass) adds f[e]
// to the bin of each of the nh histograms (specs on the device; w, w2, cnt at offsets off[h];
// outside: 3 counters per histogram).
cudaError_t launch_hist_fill(const KArgs &a, const double *xmat, int bins, int dim, int64_t ncall,
                             uint64_t seed, uint32_t stream, const float *fu, const double *f,
                             const grn_hist_spec *specs, const int *off, int nh, double *w,
                             double *w2, unsigned long long *cnt, unsigned long long *outside,
                             cudaStream_t st);

// FP32 FMA throughput probe: returns flops executed by one launch.
double      fma_probe_flops(int blocks, int threads, int iters);
cudaError_t launch_fma_probe(int blocks, int threads, int iters, float *sink, cudaStream_t st);

}  // namespace grn
