// grn_api.cu — C ABI of the engine (include/graniitti_gb300.h): engine state,
// device buffers, parameter derivation, eikonal table management and the VEGAS
// driver (the host part of MGraniitti::SampleVegas / VEGAS).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "grn_flow.cuh"
#include "grn_internal.cuh"

using grn::KArgs;

namespace {

thread_local std::string g_last_error = "ok";

grn_status fail(grn_status st, const std::string &msg) {
  g_last_error = msg;
  return st;
}

#define GRN_CUDA(call)                                                                    \
  do {                                                                                    \
    const cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                                \
      return fail(GRN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

// Grow-only device buffer.
struct DevBuf {
  void  *p   = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p   = nullptr;
    cap = 0;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p   = nullptr;
    cap = 0;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

bool is_device_ptr(const void *ptr) {
  if (!ptr) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device memory of another GPU than `device` (unmanaged): the kernels would reach it
// through peer addressing that the engine never enables.
bool on_other_device(const void *ptr, int device) {
  if (!ptr) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice && a.device != device;
}

std::vector<double> simpson38_weights(int N) {
  std::vector<double> w(N + 1, 3.0);
  w[0] = w[N] = 1.0;
  for (int i = 3; i < N; i += 3) w[i] = 2.0;
  return w;
}

}  // namespace

struct grn_engine {
  int                device = 0;
  cudaStream_t       stream = nullptr;
  grn_process_params P{};
  grn::Consts        K{};
  int                dim = 8;

  // eikonal
  int                 n_bt = 0, n_kt2 = 0;
  bool                eik_ready = false;
  DevBuf              d_mbt, d_msa, d_eik_nodes, d_xs;
  std::vector<double> h_mbt, h_msa;
  double              xs[3] = {0, 0, 0};
  DevBuf              d_lc_kt, d_lc_phi;
  int                 n_kt_nodes = 0, n_phi_nodes = 0;
  double              loop_norm_im = 0.0;

  // staging for host arrays; screened work list of grn_event_weights
  DevBuf d_u, d_w, d_flags, d_aux, d_wlist, d_wrlist, d_wcount;
  int    loop_blocks = 0;
  int    loop_pair   = 0;  // record-mode loop: events per thread - 1 (set by grn_autotune)
  int    fp64_refine = 1;  // FP32 loops: redo badly conditioned events in FP64
  double refine_tol  = grn::kRefineTol;  // estimated relative error that sends them there
  int    born_blocks = 0;  // VEGAS stage-A grid (0: default), set by grn_autotune
  int    gen_blocks  = 0;  // FP32 generic loop grid (0: one resident wave), set by grn_autotune

  // VEGAS
  int         bins = 0;
  double      lambda = 1.5;
  int64_t     ncall = 0;
  uint64_t    seed = 1;
  int         nblocks = 0;
  DevBuf      d_xmat, d_xmat_prev, d_f2mat, d_f, d_acc, d_parts, d_sc;
  DevBuf      d_xmat_flat;  // uniform grid of FLAT passes (x = u, vw = 1)
  DevBuf      d_lidx, d_lx, d_lvw;  // screened work list of a VEGAS pass
  DevBuf      d_hpart;              // partial f^2 histograms of a pass (kHistBlocks x bins x dim)
  DevBuf      d_rlist;  // slots of that list refined in FP64
  // on-the-fly histograms: specs (host copy and device), bin offsets, sums
  std::vector<grn_hist_spec> hist;
  std::vector<int>           hist_off;
  DevBuf                     d_hspec, d_hoff, d_hw, d_hw2, d_hcnt, d_hout;
  DevBuf      d_recf, d_recd;                // loop records (record mode), shared by calls
  double     *h_sc = nullptr;  // pinned
  double      sumdata = 0, sumchi2 = 0, sweight = 0;
  double      maxf = 0, maxW = 0;
  double      evaluations = 0, amp_ok = 0, kin_ok = 0, fid_ok = 0, veto_ok = 0;
  int64_t     nan_total = 0;
  uint32_t    next_stream = 1;
  int         prec = GRN_PREC_FP64;
  int64_t     iters_since_clear = 0;
  uint32_t    last_stream = 0;
  int64_t     last_ncall = 0;
  bool        vegas_ready = false;
  bool        have_last = false;
  const float *last_fu = nullptr;  // flow points of the last pass (null: Philox points)
  // unweighting
  DevBuf      d_uw_counts, d_uw_misc, d_uw_idx;
  // flows created on this engine (detached when the engine is destroyed first)
  std::vector<grn_flow *> flows;
  int                     in_batches = 0;  // batches holding this engine
  // timing of the sampling kernel
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double      sample_ms = 0.0;
  int64_t     sample_launches = 0;

  KArgs args() const {
    KArgs a{};
    a.P            = P;
    a.K            = K;
    a.lc_kt        = d_lc_kt.as<double>();
    a.lc_phi       = d_lc_phi.as<double>();
    a.n_kt_nodes   = n_kt_nodes;
    a.n_phi_nodes  = n_phi_nodes;
    a.loop_norm_re = 0.0;
    a.loop_norm_im = loop_norm_im;
    a.loop_pair    = loop_pair;
    a.refine_tol   = fp64_refine ? refine_tol : 0.0;
    a.born_blocks  = born_blocks;
    a.gen_blocks   = gen_blocks;
    return a;
  }
};

// ---------------------------------------------------------------------------
// Flow proposal state (grn_flow.cu holds the kernels).
struct grn_flow {
  grn_engine *e      = nullptr;  // null once the engine has been destroyed
  int         device = 0;
  int         layers = 6;
  int         dim    = 8;      // hypercube dimension (the process's)
  int         hidden = 128;    // MLP width
  bool        wide   = false;  // (dim, hidden) != (8, 128): the kernels of grn_flow_wide.cu
  uint64_t    seed   = 1;
  int64_t     nparams = 0;
  int64_t     adam_t  = 0;
  double      mix     = 0.0;  // weight of the uniform component of the proposal
  DevBuf      d_theta, d_m, d_v, d_grad, d_w2p, d_w3p, d_w2c, d_w3c, d_loss, d_err;
  DevBuf      d_w2t, d_w2r, d_w3t, d_w3r;    // wide shapes: backward operand copies
  DevBuf      d_x, d_z, d_lq, d_coef, d_xs;  // batch scratch
  DevBuf      d_gpart, d_lpart;                // per-block gradient / loss slices
  DevBuf      d_tu, d_tlq, d_tcoef;          // training set
  DevBuf      d_fu, d_flq;                   // points of the last flow pass
  int         in_batches = 0;                // batches that draw a member's points from it
  int         first_wait_polls = -1;         // forward kernel: poll limit of the first wait
};

namespace {

grn_status derive_consts(const grn_process_params &P, grn::Consts &K) {
  using namespace grn;
  const bool rescon = P.process == GRN_PROC_TENSOR_RESCON;
  const bool rr = P.process == GRN_PROC_REGGE_RES || P.process == GRN_PROC_REGGE_RESCON;
  if ((P.process != GRN_PROC_REGGE_CON && P.process != GRN_PROC_TENSOR_CON &&
       P.process != GRN_PROC_TENSOR_RES && !rescon && !rr) ||
      (P.phase_space != GRN_PS_CONTINUUM && P.phase_space != GRN_PS_FACTORIZED))
    return fail(GRN_ERR_UNSUPPORTED, "only PP[CON|RES|RES+CON|CONTENSOR|RESTENSOR|RES+CONTENSOR]"
                                     "<C|F> 2-body processes are implemented");
  K.rr_n = 0;
  if (rr) {
    if (P.n_res < (P.process == GRN_PROC_REGGE_RES ? 1 : 0) || P.n_res > GRN_MAX_RESONANCES)
      return fail(GRN_ERR_INVALID, "PP[RES] needs 1 to 4 resonances (PP[RES+CON] 0 to 4)");
    if (P.spin_frame != GRN_FRAME_CM && P.spin_frame != GRN_FRAME_HX &&
        P.spin_frame != GRN_FRAME_CS)
      return fail(GRN_ERR_UNSUPPORTED, "spin frames CM, HX and CS are implemented");
    if (!std::isfinite(P.omega)) return fail(GRN_ERR_INVALID, "flux exponent omega");
    for (int r = 0; r < P.n_res; ++r) {
      const grn_resonance &R = P.res[r];
      if (!(R.M > 0) || !(R.W >= 0) || !std::isfinite(R.g_decay) || !(R.g_ff > 0))
        return fail(GRN_ERR_INVALID, "resonance mass, width, form factor or decay coupling");
      if (!((R.J == 0 || R.J == 2) && R.P == 1))
        return fail(GRN_ERR_UNSUPPORTED, "Regge resonances to two pseudoscalars: J^P = 0+, 2+");
      if (R.bw < 1 || R.bw > 4) return fail(GRN_ERR_INVALID, "Breit-Wigner form 1..4");
      if (R.J == 2) {
        double tr = 0.0;
        for (int i = 0; i < 5; ++i) {
          tr += R.rho[0][6 * i];
          if (!(R.rho[0][6 * i] >= 0) || R.rho[1][6 * i] != 0.0)
            return fail(GRN_ERR_INVALID, "spin density diagonal must be real and >= 0");
          for (int j = 0; j < 5; ++j)
            if (R.rho[0][5 * i + j] != R.rho[0][5 * j + i] ||
                R.rho[1][5 * i + j] != -R.rho[1][5 * j + i])
              return fail(GRN_ERR_INVALID, "spin density matrix must be Hermitian");
        }
        if (!(std::fabs(tr - 1.0) < 1e-6)) return fail(GRN_ERR_INVALID, "spin density trace 1");
      }
      K.rr_J[r]    = R.J;
      K.rr_bw[r]   = R.bw;
      K.rr_M[r]    = R.M;
      K.rr_W[r]    = R.W;
      K.rr_iff4[r] = 1.0 / (R.g_ff * R.g_ff * R.g_ff * R.g_ff);
      K.rr_g_re[r] = R.g_regge[0] * R.g_decay;
      K.rr_g_im[r] = R.g_regge[1] * R.g_decay;
    }
    K.rr_n = P.n_res;
  }
  if ((P.process == GRN_PROC_TENSOR_CON || rescon) &&
      !(P.tensor.ap_P > 0 && P.tensor.gPNN > 0 && P.tensor.gPps > 0))
    return fail(GRN_ERR_INVALID, "tensor-pomeron parameters are not set");
  K.n_res     = 0;
  K.res_smask = 0;
  if (P.process == GRN_PROC_TENSOR_RES || (rescon && P.n_res > 0)) {
    if (!(P.tensor.ap_P > 0 && P.tensor.gPNN > 0))
      return fail(GRN_ERR_INVALID, "tensor-pomeron parameters are not set");
    if (P.n_res < 1 || P.n_res > GRN_MAX_RESONANCES)
      return fail(GRN_ERR_INVALID, "RESTENSOR needs 1 to 4 resonances");
    if (std::fabs(P.m_central[0] - P.m_central[1]) > 1e-9)
      return fail(GRN_ERR_UNSUPPORTED, "RESTENSOR decays to an equal-mass pseudoscalar pair");
    const double g2 = P.tensor.gPNN * P.tensor.gPNN;
    for (int r = 0; r < P.n_res; ++r) {
      const grn_resonance &R = P.res[r];
      if (!(R.M > 0) || !(R.W >= 0) || !std::isfinite(R.g_decay))
        return fail(GRN_ERR_INVALID, "resonance mass, width or decay coupling invalid");
      if (R.J == 0)
        for (int i = 2; i < 7; ++i)
          if (std::fabs(R.g_tensor[i]) > 1e-6)
            return fail(GRN_ERR_UNSUPPORTED, "J = 0 resonances have two coupling structures");
      if (R.J == 2) {
        K.res_c0[r] = -4.5 * g2 * R.g_decay;
        K.res_c1[r] = 0.0;
        for (int i = 0; i < 7; ++i) {
          K.res_g[r][i] = R.g_tensor[i];
          // structures with |g| <= 1e-6 are skipped (iG_PPT_total, MTensorPomeron.cc:1659-1670;
          // #0 always enters)
          if (i == 0 || std::fabs(R.g_tensor[i]) > 1e-6) K.res_smask |= 1 << i;
          if (i > 0 && !(std::fabs(R.g_tensor[i]) > 1e-6)) K.res_g[r][i] = 0.0;
        }
      } else if (R.J == 0 && R.P == 1) {
        K.res_c0[r] = 18.0 * g2 * R.g_decay * R.g_tensor[0];
        K.res_c1[r] = 18.0 * g2 * R.g_decay * R.g_tensor[1];
      } else {
        return fail(GRN_ERR_UNSUPPORTED,
                    "RESTENSOR to two pseudoscalars is implemented for J = 0 (P = +1) and J = 2");
      }
      K.res_J[r]  = R.J;
      K.res_M2[r] = R.M * R.M;
      K.res_MW[r] = R.M * R.W;
    }
    K.n_res = P.n_res;
  }
  const bool nbody = P.n_central == 4 || P.n_central == 6;
  if (P.n_central != 2 && !nbody)
    return fail(GRN_ERR_UNSUPPORTED, "central states of 2, 4 or 6 particles");
  if (nbody) {
    // PP[CON]<F|C> -> a b c d (MRegge::ME6) or a b c d e f (MRegge::ME8)
    if (P.process != GRN_PROC_REGGE_CON)
      return fail(GRN_ERR_UNSUPPORTED,
                  "4- and 6-body central states: PP[CON]<F|C> (Regge ME6, ME8)");
    if (P.n_decay != 0 || P.central_spin != 0 || P.excitation != 0)
      return fail(GRN_ERR_UNSUPPORTED, "N-body central states of stable spin-0 particles");
    for (int k = 0; k < P.n_central; ++k)
      if (!(P.m_central[k] >= 0)) return fail(GRN_ERR_INVALID, "central masses");
  }
  if (P.n_decay != 0 && P.n_decay != 2)
    return fail(GRN_ERR_UNSUPPORTED, "central decays: none or two-body cascades of both");
  if (P.central_spin != 0 && P.central_spin != 1)
    return fail(GRN_ERR_UNSUPPORTED, "central particles of spin 0 or 1");
  if (rescon && (P.n_res < 0 || P.n_res > GRN_MAX_RESONANCES))
    return fail(GRN_ERR_INVALID, "RES+CONTENSOR takes 0 to 4 resonances");
  // OFFSHELL: widths of the cascades' Breit-Wigner mass draws (the reference default 5 unless
  // set by @OFFSHELL, MProcess::SetOFFSHELL); with 0 the central particles keep their pole
  // masses and the decay coordinates follow the 8 of the 2-body point directly
  K.offshell = P.offshell_user ? P.offshell : 5.0;
  K.dec0     = K.offshell > 0.0 ? 10 : 8;
  if (P.n_decay == 2) {
    if (!(K.offshell >= 0.0 && K.offshell <= 1e3))
      return fail(GRN_ERR_INVALID, "OFFSHELL must be in [0, 1000] widths");
    if (P.process == GRN_PROC_TENSOR_RES || rescon || rr)
      return fail(GRN_ERR_UNSUPPORTED, "RESTENSOR decays directly to two pseudoscalars");
    for (int k = 0; k < 4; ++k)
      if (!(P.m_daughter[k] >= 0))
        return fail(GRN_ERR_INVALID, "daughter masses must be non-negative");
    for (int k = 0; k < 2; ++k)
      if (!(P.width[k] >= 0) ||
          !(P.m_central[k] + K.offshell * P.width[k] >
            P.m_daughter[2 * k] + P.m_daughter[2 * k + 1]))
        return fail(GRN_ERR_INVALID, "central width, or decay kinematically closed");
  }
  if (P.process == GRN_PROC_TENSOR_CON && P.central_spin == 1) {
    if (!(P.tensor.gPvv[0] != 0 || P.tensor.gPvv[1] != 0))
      return fail(GRN_ERR_INVALID, "tensor-pomeron vector couplings gPvv are not set");
    // unstable vector mesons: the reference draws their masses (GetOffShellMass)
    if (P.n_decay != 2)
      return fail(GRN_ERR_UNSUPPORTED, "vector-meson pairs need their two-body decays");
  }
  if ((P.process == GRN_PROC_TENSOR_RES || rescon || rr) && P.central_spin != 0)
    return fail(GRN_ERR_UNSUPPORTED, "the resonances decay to pseudoscalars");
  // forward excitation (NSTARS): the Regge continuum of two stable central particles
  if (P.excitation < 0 || P.excitation > 2)
    return fail(GRN_ERR_INVALID, "excitation must be 0, 1 or 2");
  if (P.excitation) {
    if (P.process != GRN_PROC_REGGE_CON || P.n_central != 2 || P.n_decay != 0)
      return fail(GRN_ERR_UNSUPPORTED,
                  "forward excitation: the Regge continuum of two central particles");
    if (!(P.xi_max > 0.0 && P.xi_max <= 1.0))
      return fail(GRN_ERR_INVALID, "xi_max must be in (0, 1]");
    if (!(P.xi_max * P.sqrt_s * P.sqrt_s > 1.09 * 1.09))
      return fail(GRN_ERR_INVALID, "xi_max s below the inelastic threshold 1.09^2 GeV^2");
    if (!(P.soft.g3P > 0.0)) return fail(GRN_ERR_INVALID, "the triple-pomeron coupling g3P");
  }
  K.lnM2f_lo = std::log(1.09 * 1.09);  // neutron + pi+ threshold (MProcess.cc:1324)
  K.lnM2f_hi = P.excitation ? std::log(P.xi_max * P.sqrt_s * P.sqrt_s) : K.lnM2f_lo;
  K.gin      = std::sqrt(std::max(0.0, P.soft.g3P * P.soft.gN_P));
  if (!(P.sqrt_s > 2 * P.m_beam)) return fail(GRN_ERR_INVALID, "sqrt_s below threshold");
  if (!(P.gcuts.fpt_max > 0) || !(P.gcuts.kt_max > P.gcuts.kt_min) ||
      !(P.gcuts.rap_max > P.gcuts.rap_min))
    return fail(GRN_ERR_INVALID, "invalid generation cuts");
  if (!(P.s_factor >= 1.0)) return fail(GRN_ERR_INVALID, "s_factor must be >= 1");
  if (P.veto_active && (P.n_veto < 0 || P.n_veto > GRN_MAX_VETO))
    return fail(GRN_ERR_INVALID, "veto cuts: 0 to 8 domains");
  K.sqrt_s = P.sqrt_s;
  K.s      = P.sqrt_s * P.sqrt_s;
  const double E  = 0.5 * P.sqrt_s;
  const double pz = std::sqrt(std::max(0.0, E * E - P.m_beam * P.m_beam));
  K.L       = E + pz;
  K.invL    = 1.0 / K.L;
  K.invL2   = 1.0 / (K.L * K.L);
  K.ifc1    = 1.0 / P.soft.fc1;
  K.ifc2    = 1.0 / P.soft.fc2;
  K.eps     = P.m_beam * P.m_beam / K.L;
  K.mp2     = P.m_beam * P.m_beam;
  K.m3      = P.m_central[0];
  K.m4      = P.m_central[1];
  K.m3sq    = K.m3 * K.m3;
  K.m4sq    = K.m4 * K.m4;
  {
    // monotone images of the fiducial windows (fiducial_cuts): M^2, pT^2 (a lower edge <= 0
    // is no cut), exp(2 Y), sinh(eta)
    const grn_fidcuts &f = P.fcuts;
    const double ninf = -std::numeric_limits<double>::infinity();
    K.cut_m2lo    = f.M_min > 0 ? f.M_min * f.M_min : ninf;
    K.cut_m2hi    = f.M_max >= 0 ? f.M_max * f.M_max : ninf;
    K.cut_pt2lo   = f.Pt_min > 0 ? f.Pt_min * f.Pt_min : ninf;
    K.cut_pt2hi   = f.Pt_max >= 0 ? f.Pt_max * f.Pt_max : ninf;
    K.cut_e2ylo   = std::exp(2.0 * f.Y_min);
    K.cut_e2yhi   = std::exp(2.0 * f.Y_max);
    K.cut_sheta_lo = std::sinh(f.eta_min);
    K.cut_sheta_hi = std::sinh(f.eta_max);
  }
  K.lnpt_lo = std::log(P.gcuts.fpt_min + kZeroEps);
  K.lnpt_hi = std::log(P.gcuts.fpt_max);
  const int    Nf = 4;
  const double fwd_log = K.lnpt_hi - K.lnpt_lo;
  const double vol = (P.gcuts.kt_max - P.gcuts.kt_min) * (2.0 * kPi) *
                     std::pow(P.gcuts.rap_max - P.gcuts.rap_min, 2) * std::pow(2.0 * kPi, 2) *
                     fwd_log * fwd_log;
  K.w_const = (1.0 / P.s_factor) * (1.0 / std::pow(2.0, 2 * (Nf - 2))) *
              (1.0 / std::pow(2.0 * kPi, 3 * Nf - 4)) * vol * kGeV2barn / (2.0 * K.s);
  if (nbody && P.phase_space == GRN_PS_CONTINUUM) {
    // BNPhaseSpaceWeight x BNIntegralVolume for Nf = Kf + 2 (MContinuum.cc:619-656): kt, phi
    // and rapidity volumes of Kf - 1 difference momenta and Kf central particles
    const int    Kf = P.n_central, Nn = Kf + 2;
    const double vn = std::pow(P.gcuts.kt_max - P.gcuts.kt_min, Kf - 1) *
                      std::pow(2.0 * kPi, Kf - 1) * std::pow(P.gcuts.rap_max - P.gcuts.rap_min, Kf) *
                      std::pow(2.0 * kPi, 2) * fwd_log * fwd_log;
    K.w_const = (1.0 / P.s_factor) * (1.0 / std::pow(2.0, 2 * (Nn - 2))) *
                (1.0 / std::pow(2.0 * kPi, 3 * Nn - 4)) * vn * kGeV2barn / (2.0 * K.s);
  }
  if (P.phase_space == GRN_PS_FACTORIZED) {
    // mass window (B51RandomKin, MFactorized.cc:263-291): M_MIN = sum of daughter masses
    // + 1e-4 GeV, M_MAX = sqrt(s) - 2 m_beam, both clipped to the <F> generation cuts.
    double msum = K.m3 + K.m4;
    if (nbody) {  // summed in the decay-list order, as the reference does
      msum = 0.0;
      for (int k = 0; k < P.n_central; ++k) msum += P.m_central[k];
    }
    const double Mmin = std::max(msum + 1e-4, P.gcuts.M_min);
    const double Mmax = std::min(P.sqrt_s - 2.0 * P.m_beam, P.gcuts.M_max);
    if (!(Mmin < Mmax)) return fail(GRN_ERR_INVALID, "<F> mass window is empty (GENCUTS <F> M)");
    if (!(P.gcuts.Y_max > P.gcuts.Y_min)) return fail(GRN_ERR_INVALID, "<F> rapidity window");
    K.M2min = Mmin * Mmin;
    K.M2max = Mmax * Mmax;
    // dPhi2/(2 pi) = p*/(8 pi^2 M_X) with p*/M_X per event; B51PhaseSpaceWeight,
    // B51IntegralVolume (MFactorized.cc:418-450), ForwardVolume. The mass^2 window of the
    // volume is per event (it depends on the off-shell masses of a cascade) and sits in
    // the per-event Jacobian factor with p*/M_X.
    const double fwd = std::pow(2.0 * kPi, 2) * fwd_log * fwd_log;
    K.w_const = (1.0 / P.s_factor) * (1.0 / (8.0 * kPi * kPi)) * 0.5 *
                (1.0 / std::pow(2.0 * kPi, 5)) * (P.gcuts.Y_max - P.gcuts.Y_min) * fwd *
                kGeV2barn / (2.0 * K.s);
    // N-body: C_space = dPhi_N / (2 pi) comes per event (nbody_jacobian)
    if (nbody) K.w_const *= 8.0 * kPi * kPi;
  }
  K.M2prop  = K.m3sq;
  K.M2propB = nbody ? P.m_central[2] * P.m_central[2] : K.m3sq;
  K.g2     = std::pow(P.regge.c[0] / P.soft.gN_P, 2);
  K.gN2    = P.soft.gN_P * P.soft.gN_P;
  K.lns0   = std::log(P.regge.s0);
  K.n_active = 0;
  for (int k = 0; k < 3; ++k) {
    K.active[k] = P.regge.active[k] ? 1 : 0;
    K.n_active += K.active[k];
    // ReggeEta(alpha, sigma) = -(1 + sigma e^{-i pi alpha}) / sin(pi alpha) (MForm.cc:382)
    const std::complex<double> e =
        -(1.0 + P.regge.sgn[k] * std::exp(std::complex<double>(0, -kPi * P.regge.a0[k]))) /
        std::sin(kPi * P.regge.a0[k]);
    K.eta0_re[k] = e.real();
    K.eta0_im[k] = e.imag();
  }
  if (K.n_active == 0) return fail(GRN_ERR_INVALID, "no active Regge trajectory");
  if (P.regge.offshellFF < 0 || P.regge.offshellFF > 2)
    return fail(GRN_ERR_INVALID, "offshellFF must be 0, 1 or 2");
  return GRN_OK;
}

// Host linear interpolation of the screening table (IArray1D::Interpolate1D).
std::complex<double> msa_interp(const std::vector<double> &msa, int N, double a) {
  const double step = (grn::kMaxKT2 - grn::kMinKT2) / N;
  if (a < grn::kMinKT2) a = grn::kMinKT2;
  int i = static_cast<int>(std::floor((a - grn::kMinKT2) / step));
  i     = std::max(0, std::min(i, N - 1));
  const double *r0 = &msa[3 * i], *r1 = &msa[3 * (i + 1)];
  const std::complex<double> y0(r0[1], r0[2]), y1(r1[1], r1[2]);
  return y0 + (a - r0[0]) * ((y1 - y0) / (r1[0] - r0[0]));
}

// kt-loop node tables from the screening table and the loop numerics.
grn_status build_loop_nodes(grn_engine *e) {
  const grn_loop_numerics &L = e->P.loop;
  if (L.n_kt < 3 || L.n_phi < 3 || L.n_kt % 3 || L.n_phi % 3)
    return fail(GRN_ERR_INVALID, "loop interval counts must be multiples of 3 (Simpson 3/8)");
  if (L.n_kt + 1 > grn::kMaxLoopNodes || L.n_phi + 1 > grn::kMaxLoopNodes)
    return fail(GRN_ERR_INVALID, "too many loop nodes");
  if (!(L.kt_max > L.kt_min) || !(L.kt_max * L.kt_max <= grn::kMaxKT2 * (1 + 1e-5)))
    return fail(GRN_ERR_INVALID, "loop kt range outside the screening table");
  const double stepKT  = (L.kt_max - L.kt_min) / L.n_kt;
  const double stepPhi = 2.0 * grn::kPi / L.n_phi;
  const std::vector<double> U = simpson38_weights(L.n_phi), V = simpson38_weights(L.n_kt);
  std::vector<double> kt(3 * (L.n_kt + 1)), ph(3 * (L.n_phi + 1));
  for (int j = 0; j <= L.n_kt; ++j) {
    const double k = L.kt_min + j * stepKT;
    const std::complex<double> c = V[j] * k * msa_interp(e->h_msa, e->n_kt2, k * k);
    kt[3 * j]     = k;
    kt[3 * j + 1] = c.real();
    kt[3 * j + 2] = c.imag();
  }
  for (int i = 0; i <= L.n_phi; ++i) {
    const double phi = i * stepPhi;
    ph[3 * i]     = std::cos(phi);
    ph[3 * i + 1] = std::sin(phi);
    ph[3 * i + 2] = U[i];
  }
  GRN_CUDA(e->d_lc_kt.ensure(kt.size() * sizeof(double)));
  GRN_CUDA(e->d_lc_phi.ensure(ph.size() * sizeof(double)));
  GRN_CUDA(cudaMemcpyAsync(e->d_lc_kt.p, kt.data(), kt.size() * sizeof(double),
                           cudaMemcpyHostToDevice, e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->d_lc_phi.p, ph.data(), ph.size() * sizeof(double),
                           cudaMemcpyHostToDevice, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  e->n_kt_nodes   = L.n_kt + 1;
  e->n_phi_nodes  = L.n_phi + 1;
  // i / (8 pi^2 s) * 9 h_phi h_kt / 64 (MProcess.cc:254-261, MMath.h:470)
  e->loop_norm_im = (9.0 * stepPhi * stepKT / 64.0) / (8.0 * grn::kPi * grn::kPi * e->K.s);
  return GRN_OK;
}

grn_status require_screening_ready(grn_engine *e) {
  if (e->P.screening && !e->eik_ready)
    return fail(GRN_ERR_STATE, "screening is on: build or set the eikonal tables first");
  return GRN_OK;
}

}  // namespace

namespace grn {
// Used by the allocation-free entry point (grn_noalloc.cu): the engine's launch
// state without touching any of its buffers.
grn_status set_error(grn_status st, const char *msg) { return fail(st, msg); }

grn_status engine_noalloc_view(grn_engine *e, KArgs *args, int *device, cudaStream_t *stream,
                               int *loop_blocks, int *dim) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  const grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  if (e->loop_blocks == 0) e->loop_blocks = grn::loop_grid_blocks(e->device);
  *args        = e->args();
  *device      = e->device;
  *stream      = e->stream;
  *loop_blocks = e->loop_blocks;
  *dim         = e->dim;
  return GRN_OK;
}
}  // namespace grn

extern "C" {

void grn_default_params(grn_process_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->process     = GRN_PROC_REGGE_CON;
  p->phase_space = GRN_PS_CONTINUUM;
  p->n_central   = 2;
  p->screening   = 0;
  p->sqrt_s      = 13000.0;
  p->m_beam      = 9.38272081e-01;  // proton (modeldata/mass_width_2018.mcd)
  p->m_central[0] = p->m_central[1] = 1.3957061e-01;  // pi+-
  p->s_factor    = 1.0;
  p->gcuts = {-0.9, 0.9, 0.0, 5.0, 0.0, 2.5, -0.9, 0.9, 0.0, 5.0};
  p->fcuts.active = 1;
  p->fcuts.eta_min = -0.9;  p->fcuts.eta_max = 0.9;
  p->fcuts.rap_min = -10.0; p->fcuts.rap_max = 10.0;
  p->fcuts.pt_min = 0.1;    p->fcuts.pt_max = 1e5;
  p->fcuts.Et_min = 0.0;    p->fcuts.Et_max = 1e5;
  p->fcuts.M_min = 0.0;     p->fcuts.M_max = 1e5;
  p->fcuts.Y_min = -10.0;   p->fcuts.Y_max = 10.0;
  p->fcuts.Pt_min = 0.0;    p->fcuts.Pt_max = 1e5;
  p->fcuts.ft_min = 0.0;    p->fcuts.ft_max = 1e5;
  p->fcuts.fM_min = 0.0;    p->fcuts.fM_max = 1e5;
  // TUNE0 PARAM_SOFT (modeldata/TUNE0/GENERAL.json:9-29)
  p->soft = {0.098, 0.065, 8.20, 0.10, 0.15 * 8.20, 0.45, 0.34, 5.0, 10.0, 0, 0};
  // TUNE0 PARAM_REGGE + PARAM_PI (GENERAL.json:90-149)
  grn_regge_params &r = p->regge;
  const double a0[3] = {1.088, 0.55, 0.55}, ap[3] = {0.20, 0.93, 0.93}, sg[3] = {1, -1, 1};
  const double c[3] = {35.00184, 81.63672, 10.86264};
  for (int k = 0; k < 3; ++k) {
    r.a0[k] = a0[k]; r.ap[k] = ap[k]; r.sgn[k] = sg[k]; r.c[k] = c[k];
    r.active[k] = (k == 0);
  }
  r.s0 = 1.0;
  r.offshellFF = 2;
  r.b_EXP = 0.944; r.a_OREAR = 0.638; r.b_OREAR = 1.886; r.b_POW = 0.5;
  // Loop numerics: 15 x 12 intervals, kt in [1e-4, 1.75]; tables 10000 intervals
  p->loop = {15, 12, 1e-4, 1.75, 10000, 10000};
  // TUNE0 PARAM_TENSORPOM, pion coupling; Kelly proton form factors (GENERAL.json:178-219)
  p->tensor = {0.0808, 0.25, 1.87, 1.76, 1, 0, {0.70, 6.20}};
  p->excitation = 0;
  p->xi_max     = 1.0;  // GENCUT default (include/Graniitti/MKinematics.h:1575)
}

double grn_tensor_decay_coupling(int32_t J, double M, double W, double m_daughter, double BR) {
  // partial width = coupling^2 x phase space x |vertex|^2 (MTensorPomeron::GDecay)
  auto gdecay = [&](double Mr) {
    const double pw = W * BR;
    const double b  = std::sqrt(1.0 - 4.0 * (m_daughter / Mr) * (m_daughter / Mr));
    if (J == 0) return std::sqrt(pw / (1.0 / (16.0 * grn::kPi * Mr) * b));
    if (J == 1) return std::sqrt(pw / (Mr / (192.0 * grn::kPi) * b * b * b));
    if (J == 2) return std::sqrt(pw / (Mr / (480.0 * grn::kPi) * Mr * Mr * b * b * b * b * b));
    if (J == 4) return 1.0;
    return std::nan("");
  };
  // two-body phase space PDW2body with |A|^2 = 1: zero below threshold
  auto ps = [&](double Mr) {
    const double x = Mr * Mr, y = m_daughter * m_daughter;
    const double l = x * x + 2.0 * y * y - 2.0 * (2.0 * x * y + y * y);
    return std::sqrt(std::max(0.0, l)) / (16.0 * grn::kPi * x * Mr);
  };
  double g = gdecay(M);
  if (std::fabs(ps(M)) < 1e-12) {
    for (int i = 1; i <= 3; ++i) {
      g = gdecay(M + i * W);
      if (ps(M + i * W) > 1e-12) break;
    }
  }
  return g;
}

double grn_regge_decay_coupling(double M, double W, double m_daughter, double BR) {
  // |A_decay|^2 = BR Gamma / Gamma_PS with the two-body width Gamma_PS of |A|^2 = 1, the
  // mother mass raised by 1..3 widths while the decay is closed
  auto ps = [&](double Mr) {
    const double x = Mr * Mr, y = m_daughter * m_daughter;
    const double l = x * x + 2.0 * y * y - 2.0 * (2.0 * x * y + y * y);
    return std::sqrt(std::max(0.0, l)) / (16.0 * grn::kPi * x * Mr);
  };
  double p = ps(M);
  if (std::fabs(p) < 1e-12)
    for (int i = 1; i <= 3; ++i) {
      p = ps(M + i * W);
      if (p > 1e-12) break;
    }
  return std::sqrt(std::max(0.0, BR * W / p));
}

const char *grn_last_error(void) { return g_last_error.c_str(); }
const char *grn_version(void) { return "graniitti_gb300 0.1 (sm_103a)"; }

grn_status grn_create(const grn_process_params *p, int32_t device, grn_engine **out) {
  if (!p || !out) return fail(GRN_ERR_INVALID, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(GRN_ERR_NO_DEVICE, "no CUDA device visible");
  }
  if (device < 0 || device >= ndev) return fail(GRN_ERR_INVALID, "bad device index");
  grn::Consts K{};
  const grn_status st = derive_consts(*p, K);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(device));
  grn_engine *e = new grn_engine();
  e->device     = device;
  e->P          = *p;
  e->K          = K;
  // hypercube dimension: 8 for a 2-body point; cascades add the decay angles (4) and, unless
  // OFFSHELL = 0, the two masses (2); 4-body central states have 14
  e->dim = p->n_central >= 4 ? 3 * p->n_central + 2
                            : (p->n_decay == 2 ? K.dec0 + 4 : (p->excitation ? 10 : 8));
  cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaMallocHost(&e->h_sc, grn::VS_COUNT * sizeof(double));
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->ev0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->ev1);
  if (ce != cudaSuccess) {
    grn_destroy(e);
    return fail(GRN_ERR_CUDA, std::string("engine setup: ") + cudaGetErrorString(ce));
  }
  *out = e;
  return GRN_OK;
}

grn_status grn_destroy(grn_engine *e) {
  if (!e) return GRN_OK;
  if (e->in_batches > 0) return fail(GRN_ERR_STATE, "engine belongs to a batch: destroy it first");
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  DevBuf *bufs[] = {&e->d_mbt,   &e->d_msa,    &e->d_eik_nodes, &e->d_xs,        &e->d_lc_kt,
                    &e->d_lc_phi, &e->d_u,     &e->d_w,         &e->d_flags,     &e->d_aux,
                    &e->d_wlist, &e->d_wcount, &e->d_xmat,      &e->d_xmat_prev, &e->d_f2mat,
                    &e->d_f,     &e->d_acc,    &e->d_parts,     &e->d_sc,        &e->d_lidx,
                    &e->d_lx,    &e->d_lvw,    &e->d_hpart,     &e->d_uw_counts, &e->d_uw_misc,
                    &e->d_rlist, &e->d_wrlist, &e->d_hspec, &e->d_hoff,
                    &e->d_hw, &e->d_hw2, &e->d_hcnt, &e->d_hout,
                    &e->d_uw_idx, &e->d_recf,  &e->d_recd,      &e->d_xmat_flat};
  for (DevBuf *b : bufs) b->release();
  for (grn_flow *f : e->flows) f->e = nullptr;  // they stay valid for grn_flow_destroy
  if (e->h_sc) cudaFreeHost(e->h_sc);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return GRN_OK;
}

const grn_process_params *grn_engine_params(const grn_engine *e) { return e ? &e->P : nullptr; }

void   *grn_engine_stream(grn_engine *e) { return e ? static_cast<void *>(e->stream) : nullptr; }
int32_t grn_dim(const grn_engine *e) { return e ? e->dim : 0; }

// ---------------------------------------------------------------------------
// Eikonal tables

grn_status grn_eikonal_build(grn_engine *e, int32_t n_bt, int32_t n_kt2) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  if (n_bt <= 0) n_bt = e->P.loop.n_bt;
  if (n_kt2 <= 0) n_kt2 = e->P.loop.n_kt2;
  if (n_bt < 2 || n_kt2 < 2 || n_bt % 2 || n_kt2 % 2)
    return fail(GRN_ERR_INVALID, "table interval counts must be even and >= 2");
  GRN_CUDA(cudaSetDevice(e->device));
  GRN_CUDA(e->d_mbt.ensure(3 * (n_bt + 1) * sizeof(double)));
  GRN_CUDA(e->d_msa.ensure(3 * (n_kt2 + 1) * sizeof(double)));
  GRN_CUDA(e->d_eik_nodes.ensure((grn::kFBN + 1) * sizeof(double2)));
  GRN_CUDA(e->d_xs.ensure(3 * sizeof(double)));
  GRN_CUDA(grn::launch_eikonal_density(e->P.soft, e->K.s, n_bt, e->d_eik_nodes.as<double2>(),
                                       e->d_mbt.as<double>(), e->stream));
  GRN_CUDA(grn::launch_eikonal_screening(e->K.s, n_bt, e->d_mbt.as<double>(), n_kt2,
                                         e->d_eik_nodes.as<double2>(), e->d_msa.as<double>(),
                                         e->d_xs.as<double>(), e->stream));
  e->h_mbt.assign(3 * (n_bt + 1), 0.0);
  e->h_msa.assign(3 * (n_kt2 + 1), 0.0);
  GRN_CUDA(cudaMemcpyAsync(e->h_mbt.data(), e->d_mbt.p, e->h_mbt.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->h_msa.data(), e->d_msa.p, e->h_msa.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->xs, e->d_xs.p, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                           e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  e->n_bt  = n_bt;
  e->n_kt2 = n_kt2;
  const grn_status st = build_loop_nodes(e);
  if (st != GRN_OK) return st;
  e->eik_ready = true;
  return GRN_OK;
}

grn_status grn_eikonal_xs(grn_engine *e, double *tot, double *el, double *inel) {
  if (!e || !e->eik_ready) return fail(GRN_ERR_STATE, "eikonal tables not built");
  if (tot) *tot = e->xs[0];
  if (el) *el = e->xs[1];
  if (inel) *inel = e->xs[2];
  return GRN_OK;
}

grn_status grn_eikonal_get(grn_engine *e, double *mbt, double *msa) {
  if (!e || !e->eik_ready) return fail(GRN_ERR_STATE, "eikonal tables not built");
  if (mbt) std::memcpy(mbt, e->h_mbt.data(), e->h_mbt.size() * sizeof(double));
  if (msa) std::memcpy(msa, e->h_msa.data(), e->h_msa.size() * sizeof(double));
  return GRN_OK;
}

grn_status grn_eikonal_set(grn_engine *e, int32_t n_bt, const double *mbt, int32_t n_kt2,
                           const double *msa) {
  if (!e || !mbt || !msa || n_bt < 2 || n_kt2 < 2) return fail(GRN_ERR_INVALID, "bad tables");
  GRN_CUDA(cudaSetDevice(e->device));
  e->h_mbt.assign(mbt, mbt + 3 * (n_bt + 1));
  e->h_msa.assign(msa, msa + 3 * (n_kt2 + 1));
  GRN_CUDA(e->d_mbt.ensure(e->h_mbt.size() * sizeof(double)));
  GRN_CUDA(e->d_msa.ensure(e->h_msa.size() * sizeof(double)));
  GRN_CUDA(e->d_xs.ensure(3 * sizeof(double)));
  GRN_CUDA(cudaMemcpyAsync(e->d_mbt.p, e->h_mbt.data(), e->h_mbt.size() * sizeof(double),
                           cudaMemcpyHostToDevice, e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->d_msa.p, e->h_msa.data(), e->h_msa.size() * sizeof(double),
                           cudaMemcpyHostToDevice, e->stream));
  GRN_CUDA(e->d_eik_nodes.ensure((grn::kFBN + 1) * sizeof(double2)));
  // cross sections from the injected density (S3CalcXS)
  GRN_CUDA(grn::launch_eikonal_xs(e->d_mbt.as<double>(), n_bt, e->d_xs.as<double>(), e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->xs, e->d_xs.p, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                           e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  e->n_bt  = n_bt;
  e->n_kt2 = n_kt2;
  const grn_status st = build_loop_nodes(e);
  if (st != GRN_OK) return st;
  e->eik_ready = true;
  return GRN_OK;
}

// ---------------------------------------------------------------------------
// Event weights

grn_status grn_event_weights(grn_engine *e, const double *u, int64_t n, int32_t dim,
                             double *w_out, uint8_t *flags, int32_t prec) {
  if (!e || !u || !w_out || n < 0) return fail(GRN_ERR_INVALID, "null argument");
  if (dim != e->dim) return fail(GRN_ERR_INVALID, "dim must equal grn_dim()");
  if (prec != GRN_PREC_FP64 && prec != GRN_PREC_MIXED) return fail(GRN_ERR_INVALID, "bad prec");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  if (n == 0) return GRN_OK;
  GRN_CUDA(cudaSetDevice(e->device));
  if (on_other_device(u, e->device) || on_other_device(w_out, e->device) ||
      on_other_device(flags, e->device))
    return fail(GRN_ERR_INVALID, "device arrays must be on the engine's device");
  const bool dev_u = is_device_ptr(u), dev_w = is_device_ptr(w_out);
  const bool dev_f = flags ? is_device_ptr(flags) : true;
  const double *du = u;
  double       *dw = w_out;
  uint8_t      *df = flags;
  if (!dev_u) {
    GRN_CUDA(e->d_u.ensure(n * dim * sizeof(double)));
    GRN_CUDA(cudaMemcpyAsync(e->d_u.p, u, n * dim * sizeof(double), cudaMemcpyHostToDevice,
                             e->stream));
    du = e->d_u.as<double>();
  }
  if (!dev_w) {
    GRN_CUDA(e->d_w.ensure(n * sizeof(double)));
    dw = e->d_w.as<double>();
  }
  if (flags && !dev_f) {
    GRN_CUDA(e->d_flags.ensure(n));
    df = e->d_flags.as<uint8_t>();
  }
  GRN_CUDA(e->d_wlist.ensure(n * sizeof(int64_t)));
  GRN_CUDA(e->d_wrlist.ensure(n * sizeof(int64_t)));
  GRN_CUDA(e->d_wcount.ensure(2 * sizeof(unsigned long long)));
  if (e->loop_blocks == 0) e->loop_blocks = grn::loop_grid_blocks(e->device);
  const KArgs a = e->args();
  if (grn::record_mode(a, prec)) {
    GRN_CUDA(e->d_recf.ensure(static_cast<size_t>(n) * grn::kLoopEventFields * sizeof(float)));
    GRN_CUDA(e->d_recd.ensure(static_cast<size_t>(n) * grn::kRecordDoubles * sizeof(double)));
    GRN_CUDA(grn::launch_event_weights_rec(a, du, n, dim, dw, df, e->d_wlist.as<int64_t>(),
                                           e->d_recf.as<float>(), e->d_recd.as<double>(),
                                           e->d_wcount.as<unsigned long long>(), e->loop_blocks,
                                           e->stream, e->d_wrlist.as<int64_t>()));
  } else {
    GRN_CUDA(grn::launch_event_weights(a, prec, du, n, dim, dw, df, e->d_wlist.as<int64_t>(),
                                       e->d_wrlist.as<int64_t>(),
                                       e->d_wcount.as<unsigned long long>(), e->loop_blocks,
                                       e->stream));
  }
  if (!dev_w)
    GRN_CUDA(cudaMemcpyAsync(w_out, dw, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  if (flags && !dev_f)
    GRN_CUDA(cudaMemcpyAsync(flags, df, n, cudaMemcpyDeviceToHost, e->stream));
  if (!dev_u || !dev_w || (flags && !dev_f)) GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_event_kinematics(grn_engine *e, const double *u, int64_t n, int32_t dim,
                                double *p4_out, double *ts_out, uint8_t *flags) {
  if (!e || !u || n < 0) return fail(GRN_ERR_INVALID, "null argument");
  if (dim != e->dim) return fail(GRN_ERR_INVALID, "dim must equal grn_dim()");
  if (n == 0) return GRN_OK;
  GRN_CUDA(cudaSetDevice(e->device));
  // Host-staged path only (diagnostics / record building).
  GRN_CUDA(e->d_u.ensure(n * dim * sizeof(double)));
  GRN_CUDA(e->d_aux.ensure(n * 18 * sizeof(double)));
  GRN_CUDA(e->d_flags.ensure(n));
  double *dp4 = e->d_aux.as<double>(), *dts = dp4 + n * 16;
  GRN_CUDA(cudaMemcpyAsync(e->d_u.p, u, n * dim * sizeof(double),
                           is_device_ptr(u) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           e->stream));
  GRN_CUDA(grn::launch_event_kinematics(e->args(), e->d_u.as<double>(), n, dim, dp4, dts,
                                        e->d_flags.as<uint8_t>(), e->stream));
  if (p4_out)
    GRN_CUDA(cudaMemcpyAsync(p4_out, dp4, n * 16 * sizeof(double), cudaMemcpyDefault, e->stream));
  if (ts_out)
    GRN_CUDA(cudaMemcpyAsync(ts_out, dts, n * 2 * sizeof(double), cudaMemcpyDefault, e->stream));
  if (flags) GRN_CUDA(cudaMemcpyAsync(flags, e->d_flags.p, n, cudaMemcpyDefault, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_event_daughters(grn_engine *e, const double *u, int64_t n, int32_t dim,
                               double *pd_out) {
  if (!e || !u || !pd_out || n < 0) return fail(GRN_ERR_INVALID, "null argument");
  if (dim != e->dim) return fail(GRN_ERR_INVALID, "dim must equal grn_dim()");
  if (e->P.n_decay != 2 && e->P.n_central < 4)
    return fail(GRN_ERR_STATE, "the process has no decay cascades or N-body central states");
  if (n == 0) return GRN_OK;
  const int64_t per = e->P.n_central == 6 ? 24 : 16;  // doubles per point
  GRN_CUDA(cudaSetDevice(e->device));
  GRN_CUDA(e->d_u.ensure(n * dim * sizeof(double)));
  GRN_CUDA(e->d_aux.ensure(n * per * sizeof(double)));
  GRN_CUDA(cudaMemcpyAsync(e->d_u.p, u, n * dim * sizeof(double),
                           is_device_ptr(u) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           e->stream));
  GRN_CUDA(grn::launch_event_daughters(e->args(), e->d_u.as<double>(), n, dim,
                                       e->d_aux.as<double>(), e->stream));
  GRN_CUDA(cudaMemcpyAsync(pd_out, e->d_aux.p, n * per * sizeof(double), cudaMemcpyDefault,
                           e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_uniforms(grn_engine *e, uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                        int32_t dim, double *out) {
  if (!e || !out || n < 0 || dim < 1 || dim > grn::kMaxDim)
    return fail(GRN_ERR_INVALID, "bad argument");
  if (n == 0) return GRN_OK;
  GRN_CUDA(cudaSetDevice(e->device));
  const bool dev = is_device_ptr(out);
  double    *d   = out;
  if (!dev) {
    GRN_CUDA(e->d_aux.ensure(n * dim * sizeof(double)));
    d = e->d_aux.as<double>();
  }
  GRN_CUDA(grn::launch_uniforms(seed, stream, first, n, dim, d, e->stream));
  if (!dev) {
    GRN_CUDA(cudaMemcpyAsync(out, d, n * dim * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    GRN_CUDA(cudaStreamSynchronize(e->stream));
  }
  return GRN_OK;
}

// ---------------------------------------------------------------------------
// VEGAS

// Bin indices of dimensions 8..15 of the screened work list (null for 8 dimensions).

// Per-call buffers of a VEGAS pass: f values and the screened work list.
static grn_status vegas_alloc_calls(grn_engine *e, int64_t ncall) {
  const size_t n = static_cast<size_t>(std::max<int64_t>(ncall, 1));
  GRN_CUDA(e->d_f.ensure(n * sizeof(double)));
  GRN_CUDA(e->d_lidx.ensure(n * sizeof(int64_t)));
  GRN_CUDA(e->d_rlist.ensure(n * sizeof(int64_t)));
  GRN_CUDA(e->d_lx.ensure(static_cast<size_t>(e->dim) * n * sizeof(double)));
  GRN_CUDA(e->d_lvw.ensure(n * sizeof(double)));
  if (e->P.screening) {
    GRN_CUDA(e->d_recf.ensure(n * grn::kLoopEventFields * sizeof(float)));
    GRN_CUDA(e->d_recd.ensure(n * grn::kRecordDoubles * sizeof(double)));
  }
  return GRN_OK;
}

static grn_status vegas_alloc(grn_engine *e) {
  const int nh = e->bins * e->dim;
  GRN_CUDA(e->d_xmat.ensure(nh * sizeof(double)));
  GRN_CUDA(e->d_xmat_prev.ensure(nh * sizeof(double)));
  GRN_CUDA(e->d_f2mat.ensure(nh * sizeof(double)));
  GRN_CUDA(e->d_hpart.ensure(static_cast<size_t>(grn::kHistBlocks) * nh * sizeof(double)));
  GRN_CUDA(grn::vegas_hist_prepare());
  GRN_CUDA(e->d_sc.ensure(grn::VS_COUNT * sizeof(double)));
  GRN_CUDA(e->d_acc.ensure(grn::kAccSlots * sizeof(unsigned long long)));
  GRN_CUDA(e->d_parts.ensure(2 * grn::kVegasSumParts * sizeof(double)));
  if (e->nblocks == 0) e->nblocks = grn::vegas_grid_blocks(e->device);
  return vegas_alloc_calls(e, e->ncall);
}

static grn_status set_ncall(grn_engine *e, int64_t n) {
  if (n != e->ncall) {
    e->ncall = n;
    return vegas_alloc_calls(e, n);
  }
  return GRN_OK;
}

grn_status grn_vegas_init(grn_engine *e, const grn_vegas_params *vp) {
  if (!e || !vp) return fail(GRN_ERR_INVALID, "null argument");
  if (vp->bins < 2 || vp->bins % 2 || vp->bins > 256)
    return fail(GRN_ERR_INVALID, "VEGAS::BINS must be even and in [2, 256]");
  if (vp->ncall < 1) return fail(GRN_ERR_INVALID, "VEGAS::NCALL must be positive");
  if (!(vp->lambda >= 1.0 && vp->lambda <= 10.0))
    return fail(GRN_ERR_INVALID, "VEGAS::LAMBDA out of [1, 10]");
  GRN_CUDA(cudaSetDevice(e->device));
  e->bins   = vp->bins;
  e->lambda = vp->lambda;
  e->ncall  = vp->ncall;
  e->seed   = vp->seed;
  e->prec   = vp->prec;
  grn_status st = vegas_alloc(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(grn::launch_vegas_grid_init(e->d_xmat.as<double>(), e->bins, e->dim, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  e->sumdata = e->sumchi2 = e->sweight = 0.0;
  e->iters_since_clear = 0;
  e->vegas_ready = true;
  e->have_last   = false;
  return GRN_OK;
}

grn_status grn_vegas_clear(grn_engine *e) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  e->sumdata = e->sumchi2 = e->sweight = 0.0;
  e->iters_since_clear = 0;
  return GRN_OK;
}

grn_status grn_get_maxweight(grn_engine *e, double *maxf) {
  if (!e || !maxf) return fail(GRN_ERR_INVALID, "null argument");
  *maxf = e->maxf;
  return GRN_OK;
}

grn_status grn_set_maxweight(grn_engine *e, double maxf) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  if (!(maxf >= 0.0) || std::isinf(maxf)) return fail(GRN_ERR_INVALID, "maximum weight must be >= 0");
  e->maxf = maxf;
  e->maxW = 0.0;
  return GRN_OK;
}

// One sampling pass over e->ncall points with `prec` arithmetic: weights f into
// d_f, pass scalars into h_sc, optional grid refinement. With fu / flq the points
// come from the flow (dimension-major, leading dimension ncall) and carry 1/q.
static grn_status vegas_pass(grn_engine *e, int prec, int track_max, int refine,
                             uint32_t stream_id, const float *fu, const float *flq,
                             const double *grid = nullptr) {
  const int nh = e->bins * e->dim;
  const double *xmat = grid ? grid : e->d_xmat.as<double>();
  GRN_CUDA(cudaMemcpyAsync(e->d_xmat_prev.p, xmat, nh * sizeof(double),
                           cudaMemcpyDeviceToDevice, e->stream));
  const KArgs a   = e->args();
  const bool  rec = grn::record_mode(a, prec);
  float      *rf  = rec ? e->d_recf.as<float>() : nullptr;
  double     *rd  = rec ? e->d_recd.as<double>() : nullptr;
  // the mapped points of listed events: the generic loop's input; in record mode only the
  // input of the FP64 refinement
  double *lx = (rec && a.refine_tol <= 0.0) ? nullptr : e->d_lx.as<double>();
  GRN_CUDA(grn::launch_vegas_born(a, xmat, e->bins, e->dim, e->ncall, e->seed,
                                  stream_id, track_max, e->d_f.as<double>(),
                                  e->d_acc.as<unsigned long long>(), e->d_lidx.as<int64_t>(),
                                  lx, e->d_lvw.as<double>(), rf, rd, e->stream, fu, flq));
  // the timed kernel: the kt-loop stage when screening is on (in record mode the FP32 record
  // loop alone; its FP64 refinement follows)
  GRN_CUDA(cudaEventRecord(e->ev0, e->stream));
  GRN_CUDA(grn::launch_vegas_loop(a, prec, e->bins, e->dim, e->ncall, track_max,
                                  e->d_f.as<double>(), e->d_acc.as<unsigned long long>(),
                                  e->d_lidx.as<int64_t>(), lx, e->d_lvw.as<double>(), rf, rd,
                                  e->d_rlist.as<int64_t>(), e->nblocks, e->stream, !rec));
  GRN_CUDA(cudaEventRecord(e->ev1, e->stream));
  if (rec && lx)
    GRN_CUDA(grn::launch_vegas_loop_fp64(a, e->bins, e->dim, e->ncall, track_max,
                                         e->d_f.as<double>(), e->d_acc.as<unsigned long long>(),
                                         e->d_lidx.as<int64_t>(), lx, e->d_lvw.as<double>(),
                                         e->d_rlist.as<int64_t>(), e->stream));
  GRN_CUDA(grn::launch_vegas_reduce(e->d_f.as<double>(), e->ncall,
                                    e->d_acc.as<unsigned long long>(), e->d_parts.as<double>(),
                                    e->d_sc.as<double>(), e->stream));
  GRN_CUDA(cudaMemcpyAsync(e->h_sc, e->d_sc.p, grn::VS_COUNT * sizeof(double),
                           cudaMemcpyDeviceToHost, e->stream));
  if (refine) {
    GRN_CUDA(grn::launch_vegas_hist(e->bins, e->dim, e->ncall, e->seed, stream_id, fu,
                                    e->d_f.as<double>(), e->d_hpart.as<double>(),
                                    e->d_f2mat.as<double>(), e->stream));
    GRN_CUDA(grn::launch_vegas_refine(e->d_xmat.as<double>(), e->d_f2mat.as<double>(), e->bins,
                                      e->dim, e->lambda, e->stream));
  }
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  {
    float ms = 0.f;
    GRN_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    e->sample_ms += ms;
    e->sample_launches += 1;
  }
  e->last_stream = stream_id;
  e->last_ncall  = e->ncall;
  e->have_last   = true;
  e->last_fu     = fu;
  return GRN_OK;
}

// Global estimates after a pass, as the reference combines them after joining its
// threads (MGraniitti.cc:1222-1251).
static grn_status vegas_accumulate(grn_engine *e, int mode, int64_t iter_index,
                                   grn_vegas_result *out) {
  const double *sc    = e->h_sc;
  const double  calls = static_cast<double>(e->ncall);
  double fsum  = sc[grn::VS_FSUM] / calls;
  double f2sum = sc[grn::VS_F2SUM] * (1.0 / calls) * (1.0 / calls);
  const double I_this = fsum;
  f2sum = std::sqrt(f2sum * calls);
  f2sum = (f2sum - fsum) * (f2sum + fsum);
  if (f2sum <= 0.0) f2sum = 1.0e-30;
  const double I2_this = f2sum / calls;
  const double alpha   = 1.0 / I2_this;
  e->sumdata += alpha * I_this;
  e->sumchi2 += alpha * I_this * I_this;
  e->sweight += alpha;
  if (mode != 0) {
    e->maxf = std::max(e->maxf, sc[grn::VS_MAXF]);
    e->maxW = std::max(e->maxW, sc[grn::VS_MAXW]);
  }
  e->evaluations += sc[grn::VS_EVAL];
  e->amp_ok += sc[grn::VS_AMP_OK];
  e->kin_ok += sc[grn::VS_KIN_OK];
  e->fid_ok += sc[grn::VS_FID_OK];
  e->veto_ok += sc[grn::VS_VETO_OK];
  e->nan_total += static_cast<int64_t>(sc[grn::VS_NAN]);
  if (out) {
    out->sigma       = e->sumdata / e->sweight;
    out->sigma_err   = std::sqrt(1.0 / e->sweight);
    double chi2      = (e->sumchi2 - e->sumdata * e->sumdata / e->sweight) / (iter_index + 1e-5);
    out->chi2        = chi2 < 0 ? 0.0 : chi2;
    out->I_this      = I_this;
    out->I2_this     = I2_this;
    out->maxf        = e->maxf;
    out->maxW        = e->maxW;
    out->evaluations = e->evaluations;
    out->amplitude_ok  = e->amp_ok;
    out->kinematics_ok = e->kin_ok;
    out->fidcuts_ok    = e->fid_ok;
    out->vetocuts_ok   = e->veto_ok;
    out->iterations    = 1;
    out->nan_count     = e->nan_total;
    out->refined       = static_cast<int64_t>(sc[grn::VS_REFINED]);
  }
  if (e->nan_total > 50)
    return fail(GRN_ERR_NAN, "more than 50 NaN/Inf weights: check model parameters and cuts");
  return GRN_OK;
}

static grn_status vegas_iteration_impl(grn_engine *e, int prec, int mode, int refine,
                                       uint32_t stream_id, int64_t iter_index,
                                       grn_vegas_result *out) {
  const grn_status st = vegas_pass(e, prec, mode != 0, refine, stream_id, nullptr, nullptr);
  if (st != GRN_OK) return st;
  return vegas_accumulate(e, mode, iter_index, out);
}

grn_status grn_vegas_iteration(grn_engine *e, int32_t mode, int32_t refine, uint32_t iter_id,
                               grn_vegas_result *out) {
  if (!e || !e->vegas_ready) return fail(GRN_ERR_STATE, "grn_vegas_init first");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(e->device));
  grn_vegas_result r{};
  st = vegas_iteration_impl(e, e->prec, mode, refine, iter_id, e->iters_since_clear++, &r);
  if (out) *out = r;
  return st;
}

// The reference's VEGAS(init, calls, itermin) (MGraniitti.cc:1146-1338); returns the
// call multiplier (1 = done, 10 = chi2 restart) through *factor.
static grn_status vegas_run(grn_engine *e, const grn_vegas_params *vp, int init, int64_t calls,
                            int itermin, int *factor, grn_vegas_result *out) {
  *factor = 1;
  if (calls != e->ncall) {
    e->ncall = calls;
    const grn_status st = vegas_alloc_calls(e, calls);
    if (st != GRN_OK) return st;
  }
  if (init == 0) {
    GRN_CUDA(grn::launch_vegas_grid_init(e->d_xmat.as<double>(), e->bins, e->dim, e->stream));
    e->sumdata = e->sumchi2 = e->sweight = 0.0;
  } else if (init == 1) {
    e->sumdata = e->sumchi2 = e->sweight = 0.0;
  }
  for (int64_t iter = 0; iter < itermin; ++iter) {
    grn_vegas_result r{};
    grn_status st = vegas_iteration_impl(e, vp->prec, init, 1, e->next_stream++, iter, &r);
    if (st != GRN_OK) return st;
    if (out) {
      const int64_t its = out->iterations;
      *out              = r;
      out->iterations   = its + 1;
    }
    if (iter > 0) {
      if (std::isnan(r.sigma) || std::isinf(r.sigma))
        return fail(GRN_ERR_NAN, "VEGAS integral inf/nan: cuts or parameters need fixing");
      if (r.sigma < 1e-60)
        return fail(GRN_ERR_INVALID, "VEGAS integral < 1e-60: check cuts and decay mode");
      if (r.chi2 > 50) {
        *factor = 10;
        return GRN_OK;
      }
    }
    if (init > 0 && iter == itermin - 1 &&
        (r.chi2 > vp->chi2max || r.sigma_err / r.sigma > vp->precision))
      ++itermin;
  }
  return GRN_OK;
}

grn_status grn_vegas_integrate(grn_engine *e, const grn_vegas_params *vp, grn_vegas_result *out) {
  if (!e || !vp) return fail(GRN_ERR_INVALID, "null argument");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  st = grn_vegas_init(e, vp);
  if (st != GRN_OK) return st;
  grn_vegas_result r{};
  int     burnin = std::max(1, vp->burnin_iter);
  int64_t ncall  = vp->ncall;
  // SampleVegas, GMODE = 0 (MGraniitti.cc:1086-1126), without the wall-clock
  // based NCALL increase.
  while (true) {
    int factor = 1;
    while (true) {
      st = vegas_run(e, vp, 0, ncall, burnin, &factor, &r);
      if (st != GRN_OK) return st;
      ncall *= factor;
      if (factor == 1) break;
    }
    r.iterations = 0;
    st = vegas_run(e, vp, 1, ncall, vp->iter, &factor, &r);
    if (st != GRN_OK) return st;
    if (factor == 1) break;
    ncall *= factor;
    burnin *= 2;
  }
  if (out) *out = r;
  return GRN_OK;
}

// The reference's FLAT integrator (MGraniitti::SampleFlat, GMODE = 0,
// src/MGraniitti.cc:1446-1524; estimate Stats::CalculateCrossSection,
// include/Graniitti/MGraniitti.h:59-66): uniform points, sigma = sum W / N,
// sigma_err = sqrt((sum W^2 / N - sigma^2) / N), until sigma_err / sigma < precision
// and N > min_events. Passes of fp->ncall Philox points through a uniform grid.
grn_status grn_flat_integrate(grn_engine *e, const grn_flat_params *fp, grn_vegas_result *out) {
  if (!e || !fp) return fail(GRN_ERR_INVALID, "null argument");
  if (fp->ncall < 1 || !(fp->precision > 0) || fp->min_events < 0 ||
      (fp->prec != GRN_PREC_FP64 && fp->prec != GRN_PREC_MIXED))
    return fail(GRN_ERR_INVALID, "bad FLAT parameters");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(e->device));
  if (!e->vegas_ready) {
    e->bins   = 128;
    e->lambda = 1.5;
    e->ncall  = fp->ncall;
    st        = vegas_alloc(e);
    if (st != GRN_OK) return st;
    GRN_CUDA(grn::launch_vegas_grid_init(e->d_xmat.as<double>(), e->bins, e->dim, e->stream));
    e->vegas_ready = true;
  }
  st = set_ncall(e, fp->ncall);
  if (st != GRN_OK) return st;
  const int nh = e->bins * e->dim;
  GRN_CUDA(e->d_xmat_flat.ensure(nh * sizeof(double)));
  GRN_CUDA(grn::launch_vegas_grid_init(e->d_xmat_flat.as<double>(), e->bins, e->dim, e->stream));
  e->seed = fp->seed;
  e->prec = fp->prec;
  e->maxf = e->maxW = 0.0;
  double wsum = 0.0, w2sum = 0.0, nev = 0.0;
  grn_vegas_result r{};
  for (int64_t it = 0; it < 100000; ++it) {
    st = vegas_pass(e, fp->prec, 1, 0, e->next_stream++, nullptr, nullptr,
                    e->d_xmat_flat.as<double>());
    if (st != GRN_OK) return st;
    const double *sc = e->h_sc;
    wsum += sc[grn::VS_FSUM];
    w2sum += sc[grn::VS_F2SUM];
    nev += static_cast<double>(e->ncall);
    e->maxf = std::max(e->maxf, sc[grn::VS_MAXF]);
    e->maxW = std::max(e->maxW, sc[grn::VS_MAXW]);
    e->evaluations += sc[grn::VS_EVAL];
    e->amp_ok += sc[grn::VS_AMP_OK];
    e->kin_ok += sc[grn::VS_KIN_OK];
    e->fid_ok += sc[grn::VS_FID_OK];
    e->veto_ok += sc[grn::VS_VETO_OK];
    e->nan_total += static_cast<int64_t>(sc[grn::VS_NAN]);
    if (e->nan_total > 50)
      return fail(GRN_ERR_NAN, "more than 50 NaN/Inf weights: check model parameters and cuts");
    const double sigma = wsum / nev;
    const double var   = std::max(w2sum / nev - sigma * sigma, 0.0);
    r.sigma            = sigma;
    r.sigma_err        = std::sqrt(var / nev);
    r.I_this           = sc[grn::VS_FSUM] / static_cast<double>(e->ncall);
    r.I2_this          = var / static_cast<double>(e->ncall);
    r.maxf             = e->maxf;
    r.maxW             = e->maxW;
    r.evaluations      = e->evaluations;
    r.amplitude_ok     = e->amp_ok;
    r.kinematics_ok    = e->kin_ok;
    r.fidcuts_ok       = e->fid_ok;
    r.vetocuts_ok      = e->veto_ok;
    r.iterations       = it + 1;
    r.nan_count        = e->nan_total;
    r.refined          = static_cast<int64_t>(sc[grn::VS_REFINED]);
    if (sigma > 0 && r.sigma_err / sigma < fp->precision && nev > fp->min_events) break;
  }
  if (out) *out = r;
  return GRN_OK;
}

grn_status grn_vegas_get_grid(grn_engine *e, double *xmat) {
  if (!e || !e->vegas_ready || !xmat) return fail(GRN_ERR_STATE, "VEGAS not initialised");
  GRN_CUDA(cudaMemcpyAsync(xmat, e->d_xmat.p, e->bins * e->dim * sizeof(double),
                           cudaMemcpyDefault, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_vegas_set_grid(grn_engine *e, const double *xmat) {
  if (!e || !e->vegas_ready || !xmat) return fail(GRN_ERR_STATE, "VEGAS not initialised");
  GRN_CUDA(cudaMemcpyAsync(e->d_xmat.p, xmat, e->bins * e->dim * sizeof(double),
                           cudaMemcpyDefault, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

// ---------------------------------------------------------------------------
// Unweighting

grn_status grn_unweight(grn_engine *e, double fmax, uint64_t seed, int64_t *n_accepted,
                        int64_t *n_overflow, int64_t *idx_out, int64_t cap) {
  if (!e || !e->have_last) return fail(GRN_ERR_STATE, "no VEGAS iteration to unweight");
  if (!(fmax > 0)) return fail(GRN_ERR_INVALID, "fmax must be positive");
  GRN_CUDA(cudaSetDevice(e->device));
  const int64_t n   = e->last_ncall;
  const int     nb  = grn::unweight_blocks(n);
  const size_t  cnt = ((nb * sizeof(int) + 255) / 256) * 256 + nb * sizeof(int64_t);
  GRN_CUDA(e->d_uw_counts.ensure(cnt));
  GRN_CUDA(e->d_uw_misc.ensure(2 * sizeof(int64_t)));
  GRN_CUDA(cudaMemsetAsync(e->d_uw_misc.p, 0, 2 * sizeof(int64_t), e->stream));
  int64_t *didx     = nullptr;
  const bool dev_ix = idx_out && is_device_ptr(idx_out);
  if (idx_out && cap > 0) {
    if (dev_ix) {
      didx = idx_out;
    } else {
      GRN_CUDA(e->d_uw_idx.ensure(cap * sizeof(int64_t)));
      didx = e->d_uw_idx.as<int64_t>();
    }
  }
  int64_t *misc = e->d_uw_misc.as<int64_t>();
  GRN_CUDA(grn::launch_unweight(e->d_f.as<double>(), n, fmax, seed, 0x80000000u | e->last_stream,
                                e->d_uw_counts.as<int>(),
                                reinterpret_cast<unsigned long long *>(misc + 1), didx, cap, misc,
                                nb, e->stream));
  int64_t h[2] = {0, 0};
  GRN_CUDA(cudaMemcpyAsync(h, misc, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  if (n_accepted) *n_accepted = h[0];
  if (n_overflow) *n_overflow = h[1];
  if (didx && !dev_ix) {
    const int64_t m = std::min(h[0], cap);
    GRN_CUDA(cudaMemcpy(idx_out, didx, m * sizeof(int64_t), cudaMemcpyDeviceToHost));
  }
  return GRN_OK;
}

grn_status grn_vegas_points(grn_engine *e, const int64_t *idx, int64_t n, double *u_out) {
  if (!e || !e->have_last || !idx || !u_out) return fail(GRN_ERR_STATE, "no VEGAS iteration");
  if (n == 0) return GRN_OK;
  GRN_CUDA(cudaSetDevice(e->device));
  GRN_CUDA(e->d_uw_idx.ensure(n * sizeof(int64_t)));
  GRN_CUDA(e->d_aux.ensure(n * e->dim * sizeof(double)));
  GRN_CUDA(cudaMemcpyAsync(e->d_uw_idx.p, idx, n * sizeof(int64_t), cudaMemcpyDefault, e->stream));
  GRN_CUDA(grn::launch_vegas_points(e->d_xmat_prev.as<double>(), e->bins, e->dim, e->seed,
                                    e->last_stream, e->d_uw_idx.as<int64_t>(), n,
                                    e->d_aux.as<double>(), e->stream, e->last_fu, e->last_ncall));
  GRN_CUDA(cudaMemcpyAsync(u_out, e->d_aux.p, n * e->dim * sizeof(double), cudaMemcpyDefault,
                           e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_pass_weights(grn_engine *e, double *f_out, int64_t n) {
  if (!e || !f_out) return fail(GRN_ERR_INVALID, "null argument");
  if (!e->have_last) return fail(GRN_ERR_STATE, "no VEGAS iteration");
  if (n != e->last_ncall) return fail(GRN_ERR_INVALID, "n must be the last pass's ncall");
  GRN_CUDA(cudaSetDevice(e->device));
  GRN_CUDA(cudaMemcpyAsync(f_out, e->d_f.p, n * sizeof(double), cudaMemcpyDefault, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

// ---------------------------------------------------------------------------
// On-the-fly histograms

static int hist_bins(const grn_hist_spec &s) { return s.nbins * (s.nbins2 > 0 ? s.nbins2 : 1); }

grn_status grn_hist_define(grn_engine *e, const grn_hist_spec *specs, int32_t n) {
  if (!e || (n > 0 && !specs) || n < 0 || n > GRN_MAX_HIST)
    return fail(GRN_ERR_INVALID, "bad histogram list (at most GRN_MAX_HIST)");
  int total = 0;
  std::vector<int> off(n);
  for (int h = 0; h < n; ++h) {
    const grn_hist_spec &s = specs[h];
    const bool two = s.nbins2 > 0;
    if (s.obs < 0 || s.obs >= GRN_NUM_OBS || s.nbins < 1 || s.nbins > 100000 ||
        !(s.hi > s.lo) || (two && (s.obs2 < 0 || s.obs2 >= GRN_NUM_OBS || s.nbins2 > 100000 ||
                                   !(s.hi2 > s.lo2))))
      return fail(GRN_ERR_INVALID, "bad histogram spec");
    off[h] = total;
    total += hist_bins(s);
    if (total > (1 << 24)) return fail(GRN_ERR_INVALID, "too many histogram bins");
  }
  GRN_CUDA(cudaSetDevice(e->device));
  e->hist.assign(specs, specs + n);
  e->hist_off = off;
  const size_t nb = std::max(total, 1);
  GRN_CUDA(e->d_hspec.ensure(std::max(n, 1) * sizeof(grn_hist_spec)));
  GRN_CUDA(e->d_hoff.ensure(std::max(n, 1) * sizeof(int)));
  GRN_CUDA(e->d_hw.ensure(nb * sizeof(double)));
  GRN_CUDA(e->d_hw2.ensure(nb * sizeof(double)));
  GRN_CUDA(e->d_hcnt.ensure(nb * sizeof(unsigned long long)));
  GRN_CUDA(e->d_hout.ensure(3 * std::max(n, 1) * sizeof(unsigned long long)));
  if (n > 0) {
    GRN_CUDA(cudaMemcpyAsync(e->d_hspec.p, specs, n * sizeof(grn_hist_spec),
                             cudaMemcpyHostToDevice, e->stream));
    GRN_CUDA(cudaMemcpyAsync(e->d_hoff.p, off.data(), n * sizeof(int), cudaMemcpyHostToDevice,
                             e->stream));
  }
  return grn_hist_clear(e);
}

grn_status grn_hist_clear(grn_engine *e) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  GRN_CUDA(cudaSetDevice(e->device));
  const int n = static_cast<int>(e->hist.size());
  int total = 0;
  for (const grn_hist_spec &s : e->hist) total += hist_bins(s);
  if (total > 0) {
    GRN_CUDA(cudaMemsetAsync(e->d_hw.p, 0, total * sizeof(double), e->stream));
    GRN_CUDA(cudaMemsetAsync(e->d_hw2.p, 0, total * sizeof(double), e->stream));
    GRN_CUDA(cudaMemsetAsync(e->d_hcnt.p, 0, total * sizeof(unsigned long long), e->stream));
  }
  if (n > 0)
    GRN_CUDA(cudaMemsetAsync(e->d_hout.p, 0, 3 * n * sizeof(unsigned long long), e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_hist_fill(grn_engine *e) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  if (!e->have_last) return fail(GRN_ERR_STATE, "no VEGAS iteration");
  if (e->hist.empty()) return GRN_OK;
  GRN_CUDA(cudaSetDevice(e->device));
  GRN_CUDA(grn::launch_hist_fill(e->args(), e->d_xmat_prev.as<double>(), e->bins, e->dim,
                                 e->last_ncall, e->seed, e->last_stream, e->last_fu,
                                 e->d_f.as<double>(), e->d_hspec.as<grn_hist_spec>(),
                                 e->d_hoff.as<int>(), static_cast<int>(e->hist.size()),
                                 e->d_hw.as<double>(), e->d_hw2.as<double>(),
                                 e->d_hcnt.as<unsigned long long>(),
                                 e->d_hout.as<unsigned long long>(), e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

grn_status grn_hist_get(grn_engine *e, int32_t h, double *w, double *w2, int64_t *counts,
                        int64_t *outside) {
  if (!e || h < 0 || h >= static_cast<int32_t>(e->hist.size()))
    return fail(GRN_ERR_INVALID, "bad histogram index");
  GRN_CUDA(cudaSetDevice(e->device));
  const int off = e->hist_off[h], nb = hist_bins(e->hist[h]);
  if (w)
    GRN_CUDA(cudaMemcpyAsync(w, e->d_hw.as<double>() + off, nb * sizeof(double),
                             cudaMemcpyDefault, e->stream));
  if (w2)
    GRN_CUDA(cudaMemcpyAsync(w2, e->d_hw2.as<double>() + off, nb * sizeof(double),
                             cudaMemcpyDefault, e->stream));
  if (counts)
    GRN_CUDA(cudaMemcpyAsync(counts, e->d_hcnt.as<unsigned long long>() + off,
                             nb * sizeof(int64_t), cudaMemcpyDefault, e->stream));
  if (outside)
    GRN_CUDA(cudaMemcpyAsync(outside, e->d_hout.as<unsigned long long>() + 3 * h,
                             3 * sizeof(int64_t), cudaMemcpyDefault, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return GRN_OK;
}

// ---------------------------------------------------------------------------
// Several processes in one pass: one fused launch per stage, replayed as a CUDA graph.

}  // extern "C"

struct grn_batch {
  std::vector<grn_engine *> eng;
  int                       device = 0;
  cudaStream_t              stream = nullptr;
  DevBuf                    d_counter;        // work queues of the two stage-B kinds
  grn::BatchProc           *h_procs = nullptr;  // pinned: uploaded by the graph every pass
  int                       born_blocks = 0, loop_blocks = 0;
  int                       max_dim     = 8;  // largest hypercube dimension of the batch
  int                       max_nh      = 0;  // largest bins * dim of the batch
  bool                      has_kind[2] = {false, false};  // generic / record-mode processes
  // per member on the generic loop: its own branch of the captured graph (stage B and the
  // pass reductions), joined back into the main stream
  cudaStream_t              side[grn::kMaxBatch] = {};
  cudaEvent_t               join[grn::kMaxBatch] = {};
  cudaEvent_t               fork = nullptr;
  cudaGraphExec_t           exec[4] = {};  // by (refine, maximum tracking)
  cudaEvent_t               ev0 = nullptr, ev1 = nullptr;
  double                    last_ms = 0.0;
  bool                      registered = false;  // counted in the engines' in_batches
  std::vector<grn_flow *>   flows;               // per member: proposal of its points (or null)
};

extern "C" {
static grn_status flow_points(grn_flow *f, bool from_flow, uint32_t stream_id, int64_t n,
                              DevBuf &dst_u, DevBuf &dst_lq);
}
namespace {
grn_status flow_check_err(grn_flow *f);
}

namespace {

grn_status batch_capture(grn_batch *b, int refine, int track_max) {
  const int np = static_cast<int>(b->eng.size());
  GRN_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = grn::upload_batch_procs(b->h_procs, np, b->stream);
  for (int p = 0; p < np && ce == cudaSuccess; ++p) {
    grn_engine *e  = b->eng[p];
    const int   nh = e->bins * e->dim;
    ce = cudaMemcpyAsync(e->d_xmat_prev.p, e->d_xmat.p, nh * sizeof(double),
                         cudaMemcpyDeviceToDevice, b->stream);
    if (ce == cudaSuccess)
      ce = cudaMemsetAsync(e->d_acc.p, 0, grn::kAccSlots * sizeof(unsigned long long),
                           b->stream);
  }
  if (ce == cudaSuccess)
    ce = cudaMemsetAsync(b->d_counter.p, 0, sizeof(unsigned long long), b->stream);
  if (ce == cudaSuccess)
    ce = grn::launch_batch_born(np, b->born_blocks, b->max_dim, b->max_nh, b->stream);
  // stage B: the record-mode processes in one persistent launch on the main stream; each
  // process on the generic loop in its own branch of the graph (its FP32 loop, FP64
  // refinement and reductions overlap the other processes' work, notably the refinement
  // passes, which occupy few SMs)
  auto reduce = [&](int p, cudaStream_t s) {
    grn_engine *e  = b->eng[p];
    cudaError_t c = grn::launch_vegas_reduce(e->d_f.as<double>(), e->ncall,
                                             e->d_acc.as<unsigned long long>(),
                                             e->d_parts.as<double>(), e->d_sc.as<double>(), s);
    if (c == cudaSuccess)
      c = cudaMemcpyAsync(e->h_sc, e->d_sc.p, grn::VS_COUNT * sizeof(double),
                          cudaMemcpyDeviceToHost, s);
    if (c == cudaSuccess && refine)
      c = grn::launch_batch_hist(p, e->bins, e->dim, e->d_hpart.as<double>(),
                                 e->d_f2mat.as<double>(), s);
    if (c == cudaSuccess && refine)
      c = grn::launch_vegas_refine(e->d_xmat.as<double>(), e->d_f2mat.as<double>(), e->bins,
                                   e->dim, e->lambda, s);
    return c;
  };
  auto generic = [&](int p) { return b->eng[p]->P.screening && !b->h_procs[p].rf; };
  if (ce == cudaSuccess && b->has_kind[0]) ce = cudaEventRecord(b->fork, b->stream);
  for (int p = 0; p < np && ce == cudaSuccess; ++p) {
    if (!generic(p)) continue;
    grn_engine *e = b->eng[p];
    ce = cudaStreamWaitEvent(b->side[p], b->fork, 0);
    if (ce == cudaSuccess)
      ce = grn::launch_vegas_loop(b->h_procs[p].A, GRN_PREC_MIXED, e->bins, e->dim, e->ncall,
                                  track_max, e->d_f.as<double>(),
                                  e->d_acc.as<unsigned long long>(), e->d_lidx.as<int64_t>(),
                                  e->d_lx.as<double>(), e->d_lvw.as<double>(), nullptr, nullptr,
                                  e->d_rlist.as<int64_t>(), e->nblocks, b->side[p]);
    if (ce == cudaSuccess) ce = reduce(p, b->side[p]);
    if (ce == cudaSuccess) ce = cudaEventRecord(b->join[p], b->side[p]);
  }
  if (ce == cudaSuccess && b->has_kind[1])
    ce = grn::launch_batch_loop(np, b->d_counter.as<unsigned long long>(), b->loop_blocks,
                                b->max_nh, b->stream);
  for (int p = 0; p < np && ce == cudaSuccess; ++p) {
    if (generic(p)) continue;
    const grn::BatchProc &q = b->h_procs[p];
    grn_engine           *e = b->eng[p];
    if (q.r_list)  // the record loop's events for the FP64 loop
      ce = grn::launch_vegas_loop_fp64(q.A, e->bins, e->dim, e->ncall, track_max,
                                       e->d_f.as<double>(), e->d_acc.as<unsigned long long>(),
                                       e->d_lidx.as<int64_t>(), e->d_lx.as<double>(),
                                       e->d_lvw.as<double>(), q.r_list, b->stream);
    if (ce == cudaSuccess) ce = reduce(p, b->stream);
  }
  for (int p = 0; p < np && ce == cudaSuccess; ++p)
    if (generic(p)) ce = cudaStreamWaitEvent(b->stream, b->join[p], 0);
  cudaGraph_t       g  = nullptr;
  const cudaError_t ce2 = cudaStreamEndCapture(b->stream, &g);
  if (ce != cudaSuccess || ce2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return fail(GRN_ERR_CUDA, std::string("batch capture: ") +
                                  cudaGetErrorString(ce != cudaSuccess ? ce : ce2));
  }
  const cudaError_t ce3 = cudaGraphInstantiate(&b->exec[2 * refine + track_max], g, 0);
  cudaGraphDestroy(g);
  if (ce3 != cudaSuccess) return fail(GRN_ERR_CUDA, cudaGetErrorString(ce3));
  return GRN_OK;
}

}  // namespace

extern "C" {

grn_status grn_batch_create(grn_engine *const *engines, int32_t n, grn_batch **out) {
  if (!engines || !out || n < 1 || n > grn::kMaxBatch)
    return fail(GRN_ERR_INVALID, "a batch holds 1 to 8 engines");
  *out = nullptr;
  const int dev = engines[0] ? engines[0]->device : 0;
  for (int p = 0; p < n; ++p) {
    grn_engine *e = engines[p];
    if (!e) return fail(GRN_ERR_INVALID, "null engine");
    for (int q = 0; q < p; ++q)
      if (engines[q] == e) return fail(GRN_ERR_INVALID, "an engine appears twice");
    if (e->device != dev) return fail(GRN_ERR_INVALID, "engines of a batch share one device");
    if (!e->vegas_ready) return fail(GRN_ERR_STATE, "grn_vegas_init every engine first");
    const grn_status st = require_screening_ready(e);
    if (st != GRN_OK) return st;
    if (e->P.screening && e->prec != GRN_PREC_MIXED)
      return fail(GRN_ERR_UNSUPPORTED, "batched screened processes use GRN_PREC_MIXED");
  }
  GRN_CUDA(cudaSetDevice(dev));
  auto *b   = new grn_batch();
  b->device = dev;
  b->eng.assign(engines, engines + n);
  grn_status st = GRN_OK;
  bool sides_ok = true;
  for (int p = 0; p < n; ++p)
    sides_ok = sides_ok &&
               cudaStreamCreateWithFlags(&b->side[p], cudaStreamNonBlocking) == cudaSuccess &&
               cudaEventCreateWithFlags(&b->join[p], cudaEventDisableTiming) == cudaSuccess;
  if (!sides_ok || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void **>(&b->h_procs), n * sizeof(grn::BatchProc)) !=
          cudaSuccess ||
      b->d_counter.ensure(2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    st = fail(GRN_ERR_CUDA, "batch: allocation failed");
  }
  // stage-A blocks in proportion to the points of each process
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t total = 0;
  for (grn_engine *e : b->eng) total += e->ncall;
  const int nb = std::max(n, sms * 16);
  int       blk = 0;
  for (int p = 0; p < n && st == GRN_OK; ++p) {
    grn_engine *e = b->eng[p];
    st            = vegas_alloc_calls(e, e->ncall);
    if (st != GRN_OK) break;
    grn::BatchProc &q = b->h_procs[p];
    std::memset(&q, 0, sizeof(q));
    q.A         = e->args();
    const bool rec = grn::record_mode(q.A, GRN_PREC_MIXED);
    q.xmat      = e->d_xmat.as<double>();
    q.bins      = e->bins;
    q.dim       = e->dim;
    q.ncall     = e->ncall;
    q.seed      = e->seed;
    q.f_out     = e->d_f.as<double>();
    q.hpart     = e->d_hpart.as<double>();
    q.acc       = e->d_acc.as<unsigned long long>();
    q.l_idx     = e->d_lidx.as<int64_t>();
    q.l_x       = e->d_lx.as<double>();
    q.l_vw      = e->d_lvw.as<double>();
    b->max_dim  = std::max(b->max_dim, e->dim);
    b->max_nh   = std::max(b->max_nh, e->bins * e->dim);
    q.rf        = rec ? e->d_recf.as<float>() : nullptr;
    q.rd        = rec ? e->d_recd.as<double>() : nullptr;
    q.r_list    = (rec && q.A.refine_tol > 0.0) ? e->d_rlist.as<int64_t>() : nullptr;
    if (e->P.screening) b->has_kind[rec ? 1 : 0] = true;
    const int k = (p == n - 1) ? nb - blk
                               : std::max<int>(1, static_cast<int>(nb * (double(e->ncall) / total)));
    q.blk0 = blk;
    q.blk1 = std::min(nb - (n - 1 - p), blk + k);
    blk    = q.blk1;
  }
  b->born_blocks = nb;
  b->loop_blocks = grn::batch_loop_blocks(dev, b->max_nh);
  if (st != GRN_OK) {
    grn_batch_destroy(b);
    return st;
  }
  for (grn_engine *e : b->eng) e->in_batches += 1;
  b->registered = true;
  b->flows.assign(n, nullptr);
  *out = b;
  return GRN_OK;
}

grn_status grn_batch_set_flow(grn_batch *b, int32_t index, grn_flow *f) {
  if (!b || index < 0 || index >= static_cast<int32_t>(b->eng.size()))
    return fail(GRN_ERR_INVALID, "bad batch member");
  if (f && f->e != b->eng[index])
    return fail(GRN_ERR_INVALID, "the flow belongs to another engine");
  if (b->flows[index]) b->flows[index]->in_batches -= 1;
  b->flows[index] = f;
  if (f) f->in_batches += 1;
  b->h_procs[index].fu = b->h_procs[index].flq = nullptr;
  return GRN_OK;
}

grn_status grn_batch_destroy(grn_batch *b) {
  if (!b) return GRN_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaGraphExec_t &x : b->exec)
    if (x) cudaGraphExecDestroy(x);
  if (b->h_procs) cudaFreeHost(b->h_procs);
  b->d_counter.release();
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->fork) cudaEventDestroy(b->fork);
  for (int p = 0; p < grn::kMaxBatch; ++p) {
    if (b->join[p]) cudaEventDestroy(b->join[p]);
    if (b->side[p]) cudaStreamDestroy(b->side[p]);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->registered)
    for (grn_engine *e : b->eng) e->in_batches -= 1;
  for (grn_flow *f : b->flows)
    if (f) f->in_batches -= 1;
  delete b;
  return GRN_OK;
}

grn_status grn_batch_iteration(grn_batch *b, int32_t mode, int32_t refine, uint32_t iter_id,
                               grn_vegas_result *results, double *device_ms) {
  if (!b) return fail(GRN_ERR_INVALID, "null batch");
  GRN_CUDA(cudaSetDevice(b->device));
  const int np = static_cast<int>(b->eng.size());
  // members with a flow proposal: their points (as grn_flow_iteration draws them) on the
  // engines' streams, all before the pass
  for (int p = 0; p < np; ++p) {
    grn_flow *f = b->flows[p];
    if (!f) continue;
    if (!f->e) return fail(GRN_ERR_STATE, "a member's flow lost its engine");
    const grn_status st = flow_points(f, true, iter_id, b->eng[p]->ncall, f->d_fu, f->d_flq);
    if (st != GRN_OK) return st;
    b->h_procs[p].fu  = f->d_fu.as<float>();
    b->h_procs[p].flq = f->d_flq.as<float>();
  }
  for (int p = 0; p < np; ++p) {
    grn_engine *e = b->eng[p];
    if (e->ncall != b->h_procs[p].ncall || e->d_f.as<double>() != b->h_procs[p].f_out)
      return fail(GRN_ERR_STATE, "an engine's call buffers changed after grn_batch_create");
    GRN_CUDA(cudaStreamSynchronize(e->stream));  // the batch works on the engines' buffers
    b->h_procs[p].stream    = iter_id;
    b->h_procs[p].track_max = mode != 0;
  }
  for (int p = 0; p < np; ++p)
    if (b->flows[p]) {
      const grn_status st = flow_check_err(b->flows[p]);
      if (st != GRN_OK) return st;
    }
  const int r = refine ? 1 : 0, tm = mode != 0 ? 1 : 0;
  if (!b->exec[2 * r + tm]) {
    const grn_status st = batch_capture(b, r, tm);
    if (st != GRN_OK) return st;
  }
  GRN_CUDA(cudaEventRecord(b->ev0, b->stream));
  GRN_CUDA(cudaGraphLaunch(b->exec[2 * r + tm], b->stream));
  GRN_CUDA(cudaEventRecord(b->ev1, b->stream));
  GRN_CUDA(cudaStreamSynchronize(b->stream));
  float ms = 0.f;
  GRN_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->last_ms = ms;
  if (device_ms) *device_ms = ms;
  grn_status st = GRN_OK;
  for (int p = 0; p < np; ++p) {
    grn_engine *e  = b->eng[p];
    e->last_stream = iter_id;
    e->last_ncall  = e->ncall;
    e->have_last   = true;
    e->last_fu     = b->flows[p] ? b->flows[p]->d_fu.as<float>() : nullptr;
    grn_vegas_result res{};
    const grn_status s2 = vegas_accumulate(e, mode, e->iters_since_clear++, &res);
    if (results) results[p] = res;
    if (s2 != GRN_OK && st == GRN_OK) st = s2;
  }
  return st;
}

// ---------------------------------------------------------------------------
// Launch configuration of the kt-loop stage and its autotuner (no counterpart in the
// reference).

grn_status grn_get_tuning(grn_engine *e, grn_tuning *t) {
  if (!e || !t) return fail(GRN_ERR_INVALID, "null argument");
  if (e->loop_blocks == 0) e->loop_blocks = grn::loop_grid_blocks(e->device);
  if (e->nblocks == 0) e->nblocks = grn::vegas_grid_blocks(e->device);
  t->loop_pair     = e->loop_pair;
  t->vegas_blocks  = e->nblocks;
  t->weight_blocks = e->loop_blocks;
  t->fp64_refine   = e->fp64_refine;
  t->refine_tol    = e->refine_tol;
  t->born_blocks   = e->born_blocks;
  t->generic_blocks = e->gen_blocks;
  return GRN_OK;
}

grn_status grn_set_tuning(grn_engine *e, const grn_tuning *t) {
  if (!e || !t) return fail(GRN_ERR_INVALID, "null argument");
  if (t->loop_pair < 0 || t->loop_pair > 2 || t->vegas_blocks < 1 || t->weight_blocks < 1 ||
      t->vegas_blocks > (1 << 20) || t->weight_blocks > (1 << 20) ||
      (t->fp64_refine != 0 && t->fp64_refine != 1) ||
      !(t->refine_tol >= 1e-9 && t->refine_tol <= 1.0) || t->born_blocks < 0 ||
      t->born_blocks > (1 << 20) || t->generic_blocks < 0 || t->generic_blocks > (1 << 20))
    return fail(GRN_ERR_INVALID, "bad tuning");
  e->loop_pair   = t->loop_pair;
  e->fp64_refine = t->fp64_refine;
  e->refine_tol  = t->refine_tol;
  e->nblocks     = t->vegas_blocks;
  e->loop_blocks = t->weight_blocks;
  e->born_blocks = t->born_blocks;
  e->gen_blocks  = t->generic_blocks;
  return GRN_OK;
}

grn_status grn_autotune(grn_engine *e, int64_t sample, grn_tune_result *out) {
  if (!e || !out || sample < 1) return fail(GRN_ERR_INVALID, "bad argument");
  std::memset(out, 0, sizeof(*out));
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(e->device));
  st = grn_get_tuning(e, &out->best);
  if (st != GRN_OK) return st;
  KArgs a = e->args();
  const bool rec = grn::record_mode(a, GRN_PREC_MIXED);
  int sms = 0;
  GRN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device));
  // candidates: kernel variant x grid (multiples of the resident blocks)
  const int mults[3][3] = {{1, 4, 0}, {2, 4, 8}, {2, 4, 8}};
  if (e->vegas_ready) {
    const int64_t nc0 = e->ncall;
    int           nc  = 0;
    // time one launch sequence twice on the engine stream, keep the second
    auto timed = [&](auto &&launch, double &ms_out) -> grn_status {
      double tmin = 1e300;
      for (int rep = 0; rep < 2; ++rep) {
        GRN_CUDA(cudaEventRecord(e->ev0, e->stream));
        GRN_CUDA(launch());
        GRN_CUDA(cudaEventRecord(e->ev1, e->stream));
        GRN_CUDA(cudaEventSynchronize(e->ev1));
        float ms = 0.f;
        GRN_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        if (rep > 0) tmin = std::min(tmin, static_cast<double>(ms));
      }
      ms_out = tmin;
      return GRN_OK;
    };
    auto born = [&]() {
      return grn::launch_vegas_born(a, e->d_xmat.as<double>(), e->bins, e->dim, nc0, e->seed,
                                    0xA7A7A7u, 0, e->d_f.as<double>(),
                                    e->d_acc.as<unsigned long long>(), e->d_lidx.as<int64_t>(),
                                    e->d_lx.as<double>(), e->d_lvw.as<double>(),
                                    rec ? e->d_recf.as<float>() : nullptr,
                                    rec ? e->d_recd.as<double>() : nullptr, e->stream);
    };
    // 1. stage A: grids of 1, 2, 4, 8 times its resident blocks (the same points each time)
    {
      const int per  = grn::vegas_born_blocks_per_sm(e->dim, e->bins);
      double    best = 1e300;
      for (int m : {1, 2, 4, 8}) {
        a.born_blocks = sms * per * m;
        double ms = 0.0;
        st        = timed(born, ms);
        if (st != GRN_OK) return st;
        grn_tuning c = out->best;
        c.born_blocks = a.born_blocks;
        out->cand[nc] = c;
        out->ms[nc]   = ms;
        out->stage[nc] = 0;
        if (ms < best) {
          best                  = ms;
          out->best.born_blocks = a.born_blocks;
        }
        ++nc;
      }
      a.born_blocks = out->best.born_blocks;
    }
    // 2. the loop stage on one stage-A output (its outputs are rewritten by the next pass)
    if (e->P.screening) {
      GRN_CUDA(born());
      double best = 1e300;
      if (rec) {
        for (int pair = 0; pair < 3; ++pair)
          for (int m = 0; m < 3 && mults[pair][m]; ++m) {
            a.loop_pair      = pair;
            const int blocks = sms * grn::loop_rec_blocks_per_sm(pair) * mults[pair][m];
            double    ms     = 0.0;
            // no refinement list: every candidate reads the same stage-A output
            st = timed([&]() {
              return grn::launch_vegas_loop(a, GRN_PREC_MIXED, e->bins, e->dim, nc0, 0,
                                            e->d_f.as<double>(), e->d_acc.as<unsigned long long>(),
                                            e->d_lidx.as<int64_t>(), e->d_lx.as<double>(),
                                            e->d_lvw.as<double>(), e->d_recf.as<float>(),
                                            e->d_recd.as<double>(), nullptr, blocks, e->stream);
            }, ms);
            if (st != GRN_OK) return st;
            grn_tuning c   = out->best;
            c.loop_pair    = pair;
            c.vegas_blocks = blocks;
            c.weight_blocks = blocks;
            out->cand[nc]  = c;
            out->ms[nc]    = ms;
            out->stage[nc] = 1;
            if (ms < best) {
              best                   = ms;
              out->best.loop_pair    = pair;
              out->best.vegas_blocks = blocks;
              out->best.weight_blocks = blocks;
            }
            ++nc;
          }
      } else {
        const int per = grn::generic_loop_blocks_per_sm(e->dim);
        for (int m : {1, 2, 4}) {
          a.gen_blocks = sms * per * m;
          double ms    = 0.0;
          st = timed([&]() {
            return grn::launch_vegas_loop(a, GRN_PREC_MIXED, e->bins, e->dim, nc0, 0,
                                          e->d_f.as<double>(), e->d_acc.as<unsigned long long>(),
                                          e->d_lidx.as<int64_t>(), e->d_lx.as<double>(),
                                          e->d_lvw.as<double>(), nullptr, nullptr, nullptr,
                                          e->nblocks, e->stream);
          }, ms);
          if (st != GRN_OK) return st;
          grn_tuning c     = out->best;
          c.generic_blocks = a.gen_blocks;
          out->cand[nc]    = c;
          out->ms[nc]      = ms;
          out->stage[nc]   = 2;
          if (ms < best) {
            best                     = ms;
            out->best.generic_blocks = a.gen_blocks;
          }
          ++nc;
        }
      }
      unsigned long long listed = 0;
      GRN_CUDA(cudaMemcpy(&listed, e->d_acc.as<unsigned long long>() + grn::VS_COUNT,
                          sizeof(listed), cudaMemcpyDeviceToHost));
      out->sample_events = static_cast<int64_t>(listed);
    }
    out->n_candidates = nc;
    e->have_last = false;  // the tuning passes are not integration passes
    return grn_set_tuning(e, &out->best);
  }
  if (!rec) return GRN_OK;  // without VEGAS only the record loop has candidates
  const int64_t n = sample;
  GRN_CUDA(e->d_u.ensure(static_cast<size_t>(n) * e->dim * sizeof(double)));
  GRN_CUDA(e->d_w.ensure(static_cast<size_t>(n) * sizeof(double)));
  GRN_CUDA(e->d_flags.ensure(static_cast<size_t>(n)));
  GRN_CUDA(e->d_wlist.ensure(static_cast<size_t>(n) * sizeof(int64_t)));
  GRN_CUDA(e->d_wcount.ensure(2 * sizeof(unsigned long long)));
  GRN_CUDA(e->d_recf.ensure(static_cast<size_t>(n) * grn::kLoopEventFields * sizeof(float)));
  GRN_CUDA(e->d_recd.ensure(static_cast<size_t>(n) * grn::kRecordDoubles * sizeof(double)));
  GRN_CUDA(grn::launch_uniforms(0x7E57ull, 0, 0, n, e->dim, e->d_u.as<double>(), e->stream));
  GRN_CUDA(grn::launch_weights_born_rec(a, e->d_u.as<double>(), n, e->dim, e->d_w.as<double>(),
                                        e->d_flags.as<uint8_t>(), e->d_wlist.as<int64_t>(),
                                        e->d_recf.as<float>(), e->d_recd.as<double>(),
                                        e->d_wcount.as<unsigned long long>(), e->stream));
  double best = 1e300;
  int    nc   = 0;
  for (int pair = 0; pair < 3; ++pair) {
    for (int m = 0; m < 3 && mults[pair][m]; ++m) {
      a.loop_pair      = pair;
      const int blocks = sms * grn::loop_rec_blocks_per_sm(pair) * mults[pair][m];
      double    tmin   = 1e300;
      for (int rep = 0; rep < 3; ++rep) {
        GRN_CUDA(cudaEventRecord(e->ev0, e->stream));
        GRN_CUDA(grn::launch_weights_loop_rec(a, n, e->d_w.as<double>(), e->d_flags.as<uint8_t>(),
                                              e->d_wlist.as<int64_t>(), e->d_recf.as<float>(),
                                              e->d_recd.as<double>(),
                                              e->d_wcount.as<unsigned long long>(), blocks,
                                              e->stream));
        GRN_CUDA(cudaEventRecord(e->ev1, e->stream));
        GRN_CUDA(cudaEventSynchronize(e->ev1));
        float ms = 0.f;
        GRN_CUDA(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        if (rep > 0) tmin = std::min(tmin, static_cast<double>(ms));  // first launch warms up
      }
      grn_tuning c    = out->best;
      c.loop_pair     = pair;
      c.vegas_blocks  = blocks;
      c.weight_blocks = blocks;
      out->cand[nc]   = c;
      out->ms[nc]     = tmin;
      out->stage[nc]  = 1;
      if (tmin < best) {
        best = tmin;
        out->best.loop_pair     = pair;
        out->best.vegas_blocks  = blocks;
        out->best.weight_blocks = blocks;
      }
      ++nc;
    }
  }
  out->n_candidates = nc;
  unsigned long long listed = 0;
  GRN_CUDA(cudaMemcpy(&listed, e->d_wcount.p, sizeof(listed), cudaMemcpyDeviceToHost));
  out->sample_events = static_cast<int64_t>(listed);
  return grn_set_tuning(e, &out->best);
}

grn_status grn_kernel_timing(grn_engine *e, int32_t reset, double *total_ms, int64_t *launches) {
  if (!e) return fail(GRN_ERR_INVALID, "null engine");
  if (total_ms) *total_ms = e->sample_ms;
  if (launches) *launches = e->sample_launches;
  if (reset) {
    e->sample_ms       = 0.0;
    e->sample_launches = 0;
  }
  return GRN_OK;
}

grn_status grn_fp32_peak(int32_t device, double *tflops) {
  if (!tflops) return fail(GRN_ERR_INVALID, "null argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return fail(GRN_ERR_NO_DEVICE, "no such CUDA device");
  }
  GRN_CUDA(cudaSetDevice(device));
  int sms = 0;
  GRN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  float    *sink = nullptr;
  GRN_CUDA(cudaMalloc(&sink, sizeof(float)));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, nullptr);
    grn::launch_fma_probe(blocks, threads, iters, sink, nullptr);
    cudaEventRecord(b, nullptr);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && ms > 0) best = std::max(best, grn::fma_probe_flops(blocks, threads, iters) /
                                                   (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(GRN_ERR_CUDA, cudaGetErrorString(ce));
  *tflops = best;
  return GRN_OK;
}


// ---------------------------------------------------------------------------
// Flow proposal (INTEGRATOR "NEURO": MGraniitti::SampleNeuro, src/MGraniitti.cc:1527-1620)

}  // extern "C"

namespace {

// Host pointer -> device staging (device pointers pass through).
template <typename T>
grn_status stage_in(DevBuf &buf, const T *p, size_t count, cudaStream_t st, const T **out) {
  if (is_device_ptr(p)) {
    *out = p;
    return GRN_OK;
  }
  GRN_CUDA(buf.ensure(count * sizeof(T)));
  GRN_CUDA(cudaMemcpyAsync(buf.p, p, count * sizeof(T), cudaMemcpyHostToDevice, st));
  *out = buf.as<T>();
  return GRN_OK;
}

// SplitMix64 (Steele, Lea, Flood 2014): initial weights only.
double splitmix_uniform(uint64_t &state) {
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return static_cast<double>(z >> 11) * 0x1.0p-53;
}

grn::FlowWideBufs wide_bufs(grn_flow *f) {
  return {f->d_w2c.p, f->d_w3c.p, f->d_w2t.p, f->d_w2r.p, f->d_w3t.p, f->d_w3r.p};
}

grn_status flow_pack(grn_flow *f) {
  if (f->wide)
    GRN_CUDA(grn::launch_wflow_pack(f->dim, f->hidden, f->d_theta.as<float>(), f->layers,
                                    wide_bufs(f), f->e->stream));
  else
    GRN_CUDA(grn::launch_flow_pack(f->d_theta.as<float>(), f->layers, f->d_w2p.p, f->d_w3p.p,
                                   f->d_w2c.p, f->d_w3c.p, f->e->stream));
  return GRN_OK;
}

// Forward pass of the flow's shape (see launch_flow_forward).
cudaError_t flow_forward(grn_flow *f, int mode, const float *xin, int64_t ld_in, int64_t n,
                         uint64_t seed, uint32_t stream, int64_t first, float *xout,
                         int64_t ld_out, float *lq, float *xs_store) {
  if (f->wide)
    return grn::launch_wflow_forward(f->dim, f->hidden, mode, f->d_theta.as<float>(),
                                     wide_bufs(f), f->layers, xin, ld_in, n, seed, stream, first,
                                     xout, ld_out, lq, xs_store, f->d_err.as<int>(), f->e->stream);
  return grn::launch_flow_forward(mode, f->d_theta.as<float>(), f->d_w2c.p, f->d_w3c.p,
                                  f->layers, xin, ld_in, n, seed, stream, first, xout, ld_out, lq,
                                  xs_store, f->d_err.as<int>(), f->e->stream, f->first_wait_polls);
}

// Bounded waits inside the forward kernel report through d_err (read after a sync).
grn_status flow_check_err(grn_flow *f) {
  int h = 0;
  GRN_CUDA(cudaMemcpy(&h, f->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    cudaMemset(f->d_err.p, 0, sizeof(int));
    return fail(GRN_ERR_CUDA, "flow kernel: a bounded wait gave up (tensor-core or copy stall)");
  }
  return GRN_OK;
}

// Forward pass of the training step (layer inputs kept) + backward into d_grad.
grn_status flow_loss_grad(grn_flow *f, const float *x, int64_t ld, const float *coef, int64_t n,
                          int kind, double *loss_slot) {
  grn_engine *e = f->e;
  GRN_CUDA(f->d_xs.ensure(static_cast<size_t>(f->layers) * f->dim * n * sizeof(float)));
  GRN_CUDA(f->d_lq.ensure(n * sizeof(float)));
  GRN_CUDA(flow_forward(f, 0, x, ld, n, 0, 0, 0, nullptr, 0, f->d_lq.as<float>(),
                        f->d_xs.as<float>()));
  const int slices = grn::flow_backward_slices();
  GRN_CUDA(f->d_gpart.ensure(static_cast<size_t>(slices) * f->nparams * sizeof(float)));
  GRN_CUDA(f->d_lpart.ensure(static_cast<size_t>(slices) * sizeof(double)));
  if (f->wide)
    GRN_CUDA(grn::launch_wflow_backward(f->dim, f->hidden, f->d_theta.as<float>(), wide_bufs(f),
                                        f->layers, f->d_xs.as<float>(), f->d_lq.as<float>(), coef,
                                        n, kind, f->d_gpart.as<float>(), f->d_lpart.as<double>(),
                                        f->d_grad.as<float>(), loss_slot, e->stream));
  else
    GRN_CUDA(grn::launch_flow_backward(f->d_theta.as<float>(), f->d_w2p.p, f->d_w3p.p, f->layers,
                                       f->d_xs.as<float>(), f->d_lq.as<float>(), coef, n, kind,
                                       f->d_gpart.as<float>(), f->d_lpart.as<double>(),
                                       f->d_grad.as<float>(), loss_slot, e->stream));
  return GRN_OK;
}

grn_status flow_adam(grn_flow *f, double lr) {
  const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
  f->adam_t += 1;
  const double c1 = 1.0 - std::pow(b1, static_cast<double>(f->adam_t));
  const double c2 = 1.0 - std::pow(b2, static_cast<double>(f->adam_t));
  GRN_CUDA(grn::launch_flow_adam(f->d_theta.as<float>(), f->d_m.as<float>(), f->d_v.as<float>(),
                                 f->d_grad.as<float>(), f->nparams,
                                 static_cast<float>(lr * std::sqrt(c2) / c1), static_cast<float>(b1),
                                 static_cast<float>(b2), static_cast<float>(eps * std::sqrt(c2)),
                                 f->e->stream));
  return flow_pack(f);
}

grn_status check_flow(grn_flow *f) {
  if (!f) return fail(GRN_ERR_INVALID, "null flow");
  if (!f->e) return fail(GRN_ERR_STATE, "the flow's engine has been destroyed");
  GRN_CUDA(cudaSetDevice(f->e->device));
  return GRN_OK;
}

}  // namespace

extern "C" {

void grn_flow_default_params(grn_flow_params *p) {
  if (!p) return;
  p->dim    = 8;
  p->layers = 6;
  p->hidden = grn::flow::kHid;
  p->bins   = grn::flow::kBins;
  p->seed   = 1;
  p->mix_uniform = 0.0;
}

grn_status grn_flow_create(grn_engine *e, const grn_flow_params *p, grn_flow **out) {
  if (!e || !p || !out) return fail(GRN_ERR_INVALID, "null argument");
  *out = nullptr;
  if (p->dim != e->dim)
    return fail(GRN_ERR_UNSUPPORTED, "flow dimension must be the process dimension");
  const bool base = p->dim == grn::flow::kDim && p->hidden == grn::flow::kHid;
  if (p->bins != grn::flow::kBins || !(base || grn::flow_wide_supported(p->dim, p->hidden)))
    return fail(GRN_ERR_UNSUPPORTED,
                "flow kernels are built for bins = 16 and (dim, hidden) = (8, 128), (8, 256), "
                "(12, 128), (12, 256), (14, 128), (14, 256)");
  if (p->layers < 1 || p->layers > grn::flow::kMaxLayers)
    return fail(GRN_ERR_INVALID, "flow layers must be in [1, 12]");
  if (!(p->mix_uniform >= 0.0 && p->mix_uniform < 1.0))
    return fail(GRN_ERR_INVALID, "flow mix_uniform must be in [0, 1)");
  GRN_CUDA(cudaSetDevice(e->device));
  auto *f    = new grn_flow();
  f->e       = e;
  f->device  = e->device;
  e->flows.push_back(f);
  f->layers  = p->layers;
  f->dim     = p->dim;
  f->hidden  = p->hidden;
  f->wide    = !base;
  f->seed    = p->seed;
  f->mix     = p->mix_uniform;
  const int64_t lp = grn::flow_layer_params(f->dim, f->hidden);
  f->nparams = static_cast<int64_t>(p->layers) * lp;
  std::vector<float> th(f->nparams, 0.0f);
  uint64_t           state = p->seed;
  using grn::flow::kBins;
  using grn::flow::kRaw;
  const int   da = f->dim / 2, hid = f->hidden, nout = da * kRaw;
  const float b3d = static_cast<float>(std::log(std::expm1(1.0 - 1e-3)));
  for (int l = 0; l < p->layers; ++l) {
    float       *t  = th.data() + static_cast<size_t>(l) * lp;
    const double l1 = std::sqrt(6.0 / da), l2 = std::sqrt(6.0 / hid);
    for (int i = 0; i < da * hid; ++i) t[i] = static_cast<float>((2 * splitmix_uniform(state) - 1) * l1);
    float *w2 = t + da * hid + hid;
    for (int i = 0; i < hid * hid; ++i) w2[i] = static_cast<float>((2 * splitmix_uniform(state) - 1) * l2);
    float *b3 = t + lp - nout;
    for (int j = 0; j < da; ++j)
      for (int r = 2 * kBins; r < kRaw; ++r) b3[j * kRaw + r] = b3d;
  }
  const size_t pb = f->nparams * sizeof(float);
  grn_status   st = GRN_OK;
  bool         ok_w = true;
  if (f->wide) {
    const grn::FlowWideSizes z = grn::flow_wide_sizes(f->dim, f->hidden, f->layers);
    ok_w = f->d_w2c.ensure(z.w2c * 2) == cudaSuccess && f->d_w3c.ensure(z.w3c * 2) == cudaSuccess &&
           f->d_w2t.ensure(z.w2t * 2) == cudaSuccess && f->d_w2r.ensure(z.w2r * 2) == cudaSuccess &&
           f->d_w3t.ensure(z.w3t * 2) == cudaSuccess && f->d_w3r.ensure(z.w3r * 2) == cudaSuccess;
  } else {
    ok_w = f->d_w2p.ensure(grn::flow_w2p_elems(f->layers) * 2) == cudaSuccess &&
           f->d_w3p.ensure(grn::flow_w3p_elems(f->layers) * 2) == cudaSuccess &&
           f->d_w2c.ensure(grn::flow_w2c_elems(f->layers) * 2) == cudaSuccess &&
           f->d_w3c.ensure(grn::flow_w3c_elems(f->layers) * 2) == cudaSuccess;
  }
  if (!ok_w || f->d_theta.ensure(pb) != cudaSuccess || f->d_m.ensure(pb) != cudaSuccess ||
      f->d_v.ensure(pb) != cudaSuccess || f->d_grad.ensure(pb) != cudaSuccess ||
      f->d_loss.ensure(sizeof(double)) != cudaSuccess ||
      f->d_err.ensure(sizeof(int)) != cudaSuccess) {
    st = fail(GRN_ERR_CUDA, "flow: device allocation failed");
  } else if (cudaMemcpy(f->d_theta.p, th.data(), pb, cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemset(f->d_m.p, 0, pb) != cudaSuccess ||
             cudaMemset(f->d_v.p, 0, pb) != cudaSuccess ||
             cudaMemset(f->d_err.p, 0, sizeof(int)) != cudaSuccess) {
    st = fail(GRN_ERR_CUDA, "flow: upload failed");
  } else {
    st = flow_pack(f);
    if (st == GRN_OK && cudaStreamSynchronize(e->stream) != cudaSuccess)
      st = fail(GRN_ERR_CUDA, "flow: pack failed");
  }
  if (st != GRN_OK) {
    grn_flow_destroy(f);
    return st;
  }
  *out = f;
  return GRN_OK;
}

grn_status grn_flow_destroy(grn_flow *f) {
  if (!f) return GRN_OK;
  if (f->in_batches > 0) return fail(GRN_ERR_STATE, "the flow serves a batch: destroy it first");
  cudaSetDevice(f->device);
  if (f->e) {
    auto &v = f->e->flows;
    v.erase(std::remove(v.begin(), v.end(), f), v.end());
    cudaStreamSynchronize(f->e->stream);
  }
  for (DevBuf *b : {&f->d_theta, &f->d_m, &f->d_v, &f->d_grad, &f->d_w2p, &f->d_w3p, &f->d_w2c,
                    &f->d_w3c, &f->d_w2t, &f->d_w2r, &f->d_w3t, &f->d_w3r, &f->d_err, &f->d_loss,
                    &f->d_x, &f->d_z, &f->d_lq, &f->d_coef, &f->d_xs, &f->d_gpart,
                    &f->d_lpart, &f->d_tu, &f->d_tlq,
                    &f->d_tcoef, &f->d_fu, &f->d_flq})
    b->release();
  if (f->e && f->e->last_fu) {
    f->e->last_fu   = nullptr;
    f->e->have_last = false;
  }
  delete f;
  return GRN_OK;
}

grn_status grn_flow_set_wait_polls(grn_flow *f, int32_t polls) {
  if (!f) return fail(GRN_ERR_INVALID, "null flow");
  f->first_wait_polls = polls < 0 ? -1 : polls;
  return GRN_OK;
}

int64_t grn_flow_num_params(const grn_flow *f) { return f ? f->nparams : 0; }

grn_status grn_flow_get_params(grn_flow *f, float *theta) {
  grn_status st = check_flow(f);
  if (st != GRN_OK) return st;
  if (!theta) return fail(GRN_ERR_INVALID, "null argument");
  GRN_CUDA(cudaMemcpyAsync(theta, f->d_theta.p, f->nparams * sizeof(float), cudaMemcpyDefault,
                           f->e->stream));
  GRN_CUDA(cudaStreamSynchronize(f->e->stream));
  return GRN_OK;
}

grn_status grn_flow_set_params(grn_flow *f, const float *theta) {
  grn_status st = check_flow(f);
  if (st != GRN_OK) return st;
  if (!theta) return fail(GRN_ERR_INVALID, "null argument");
  const size_t pb = f->nparams * sizeof(float);
  GRN_CUDA(cudaMemcpyAsync(f->d_theta.p, theta, pb, cudaMemcpyDefault, f->e->stream));
  GRN_CUDA(cudaMemsetAsync(f->d_m.p, 0, pb, f->e->stream));
  GRN_CUDA(cudaMemsetAsync(f->d_v.p, 0, pb, f->e->stream));
  f->adam_t = 0;
  st        = flow_pack(f);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaStreamSynchronize(f->e->stream));
  return GRN_OK;
}

// Shared body of density / inverse / sample.
static grn_status flow_map(grn_flow *f, int mode, const float *xin, uint64_t seed,
                           uint32_t stream, int64_t first, int64_t n, float *xout, float *logq) {
  grn_status st = check_flow(f);
  if (st != GRN_OK) return st;
  if (n < 0 || !logq) return fail(GRN_ERR_INVALID, "bad argument");
  if (n == 0) return GRN_OK;
  grn_engine  *e  = f->e;
  const size_t nx = static_cast<size_t>(n) * f->dim;
  const float *dx = nullptr;
  if (xin) {
    st = stage_in(f->d_x, xin, nx, e->stream, &dx);
    if (st != GRN_OK) return st;
  }
  const bool dev_out = !xout || is_device_ptr(xout), dev_lq = is_device_ptr(logq);
  float     *dz = xout, *dl = logq;
  if (xout && !dev_out) {
    GRN_CUDA(f->d_z.ensure(nx * sizeof(float)));
    dz = f->d_z.as<float>();
  }
  if (!dev_lq) {
    GRN_CUDA(f->d_lq.ensure(n * sizeof(float)));
    dl = f->d_lq.as<float>();
  }
  GRN_CUDA(flow_forward(f, mode, dx, n, n, seed, stream, first, dz, n, dl, nullptr));
  if (xout && !dev_out)
    GRN_CUDA(cudaMemcpyAsync(xout, dz, nx * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
  if (!dev_lq)
    GRN_CUDA(cudaMemcpyAsync(logq, dl, n * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  return flow_check_err(f);
}

grn_status grn_flow_density(grn_flow *f, const float *x, int64_t n, float *z_out, float *logq) {
  if (!x) return fail(GRN_ERR_INVALID, "null argument");
  return flow_map(f, 0, x, 0, 0, 0, n, z_out, logq);
}

grn_status grn_flow_inverse(grn_flow *f, const float *z, int64_t n, float *x_out, float *logq) {
  if (!z || !x_out) return fail(GRN_ERR_INVALID, "null argument");
  return flow_map(f, 1, z, 0, 0, 0, n, x_out, logq);
}

grn_status grn_flow_sample(grn_flow *f, uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                           float *x_out, float *logq) {
  if (!x_out) return fail(GRN_ERR_INVALID, "null argument");
  return flow_map(f, 1, nullptr, seed, stream, first, n, x_out, logq);
}

grn_status grn_flow_loss_grad(grn_flow *f, const float *x, const float *coef, int64_t n,
                              int32_t kind, double *loss, float *grad) {
  grn_status st = check_flow(f);
  if (st != GRN_OK) return st;
  if (!x || !coef || n < 1 || (kind != 0 && kind != 1)) return fail(GRN_ERR_INVALID, "bad argument");
  grn_engine  *e  = f->e;
  const float *dx = nullptr, *dc = nullptr;
  st = stage_in(f->d_x, x, static_cast<size_t>(n) * f->dim, e->stream, &dx);
  if (st != GRN_OK) return st;
  st = stage_in(f->d_coef, coef, static_cast<size_t>(n), e->stream, &dc);
  if (st != GRN_OK) return st;
  st = flow_loss_grad(f, dx, n, dc, n, kind, f->d_loss.as<double>());
  if (st != GRN_OK) return st;
  double l = 0.0;
  GRN_CUDA(cudaMemcpyAsync(&l, f->d_loss.p, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  if (grad)
    GRN_CUDA(cudaMemcpyAsync(grad, f->d_grad.p, f->nparams * sizeof(float), cudaMemcpyDefault,
                             e->stream));
  GRN_CUDA(cudaStreamSynchronize(e->stream));
  if (loss) *loss = l / static_cast<double>(n);
  return flow_check_err(f);
}

grn_status grn_flow_train_step(grn_flow *f, const float *x, const float *coef, int64_t n,
                               int32_t kind, double lr, double *loss) {
  grn_status st = grn_flow_loss_grad(f, x, coef, n, kind, loss, nullptr);
  if (st != GRN_OK) return st;
  st = flow_adam(f, lr);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaStreamSynchronize(f->e->stream));
  return GRN_OK;
}

// Points of a pass (dimension-major, leading dimension n) and their log density:
// Philox uniforms (q = 1), or the proposal alpha * uniform + (1 - alpha) * flow whose first
// floor(alpha n) points are the uniform component (flow density from the density
// direction) and the rest flow samples.
static grn_status flow_points(grn_flow *f, bool from_flow, uint32_t stream_id, int64_t n,
                              DevBuf &dst_u, DevBuf &dst_lq) {
  grn_engine *e = f->e;
  GRN_CUDA(dst_u.ensure(static_cast<size_t>(n) * f->dim * sizeof(float)));
  GRN_CUDA(dst_lq.ensure(static_cast<size_t>(n) * sizeof(float)));
  float         *u = dst_u.as<float>(), *lq = dst_lq.as<float>();
  const uint64_t key = e->seed ^ 0xF10Bull;
  if (!from_flow) {
    GRN_CUDA(grn::launch_flow_uniform_dim(f->dim, key, stream_id, 0, n, n, u, lq, e->stream));
    return GRN_OK;
  }
  const int64_t nu = static_cast<int64_t>(f->mix * static_cast<double>(n));
  if (nu > 0) {
    GRN_CUDA(grn::launch_flow_uniform_dim(f->dim, key, stream_id, 0, nu, n, u, nullptr,
                                          e->stream));
    GRN_CUDA(flow_forward(f, 0, u, n, nu, 0, 0, 0, nullptr, 0, lq, nullptr));
  }
  GRN_CUDA(flow_forward(f, 1, nullptr, n, n - nu, key, stream_id, nu, u + nu, n, lq + nu,
                        nullptr));
  if (f->mix > 0.0) GRN_CUDA(grn::launch_flow_mix(lq, n, f->mix, e->stream));
  return GRN_OK;
}

grn_status grn_flow_train(grn_engine *e, grn_flow *f, const grn_flow_train_params *tp,
                          grn_flow_train_result *out) {
  if (!e || !f || !tp || f->e != e) return fail(GRN_ERR_INVALID, "bad argument");
  if (!e->vegas_ready) return fail(GRN_ERR_STATE, "grn_vegas_init (and adapt the grid) first");
  if (tp->n_train < 1 || tp->batch < 1 || tp->n_train % tp->batch || tp->epochs < 1 ||
      tp->rounds < 1 || (tp->loss != 0 && tp->loss != 1) || !(tp->lr > 0))
    return fail(GRN_ERR_INVALID, "bad training parameters (n_train must be a multiple of batch)");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(e->device));
  const int64_t ncall0 = e->ncall, n = tp->n_train, B = tp->batch;
  const int64_t steps_per_round = (n / B) * tp->epochs;
  const int64_t nsteps          = steps_per_round * tp->rounds;
  DevBuf        d_losses;
  GRN_CUDA(d_losses.ensure(nsteps * sizeof(double)));
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  GRN_CUDA(cudaEventRecord(t0, e->stream));
  grn_flow_train_result r{};
  int64_t step = 0;
  for (int round = 0; round < tp->rounds && st == GRN_OK; ++round) {
    st = set_ncall(e, n);
    if (st != GRN_OK) break;
    const uint32_t sid = 0x20000000u | static_cast<uint32_t>(tp->seed_stream + round);
    st = flow_points(f, round > 0, sid, n, f->d_tu, f->d_tlq);
    if (st != GRN_OK) break;
    st = vegas_pass(e, tp->prec, 0, 0, sid, f->d_tu.as<float>(), f->d_tlq.as<float>());
    if (st != GRN_OK) break;
    const double m1 = e->h_sc[grn::VS_FSUM] / n, m2 = e->h_sc[grn::VS_F2SUM] / n;
    if (round == 0) r.rel_var_start = m2 / (m1 * m1) - 1.0;
    if (!(m2 > 0)) {
      st = fail(GRN_ERR_INVALID, "flow training: all weights are zero");
      break;
    }
    GRN_CUDA(f->d_tcoef.ensure(n * sizeof(float)));
    GRN_CUDA(grn::launch_flow_coef(e->d_f.as<double>(), round > 0 ? f->d_tlq.as<float>() : nullptr,
                                   n, tp->loss, tp->loss == 1 ? m2 : m1, f->d_tcoef.as<float>(),
                                   e->stream));
    for (int ep = 0; ep < tp->epochs && st == GRN_OK; ++ep) {
      for (int64_t b = 0; b < n / B && st == GRN_OK; ++b) {
        st = flow_loss_grad(f, f->d_tu.as<float>() + b * B, n, f->d_tcoef.as<float>() + b * B, B,
                            tp->loss, d_losses.as<double>() + step);
        if (st == GRN_OK) st = flow_adam(f, tp->lr);
        ++step;
      }
    }
  }
  if (st == GRN_OK) {
    GRN_CUDA(cudaEventRecord(t1, e->stream));
    std::vector<double> losses(nsteps);
    GRN_CUDA(cudaMemcpyAsync(losses.data(), d_losses.p, nsteps * sizeof(double),
                             cudaMemcpyDeviceToHost, e->stream));
    GRN_CUDA(cudaStreamSynchronize(e->stream));
    st = flow_check_err(f);
    if (st != GRN_OK) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    r.train_ms   = ms;
    r.steps      = nsteps;
    r.loss_first = losses.front() / B;
    r.loss_last  = losses.back() / B;
    // evaluation pass through the trained flow: relative variance of the weights
    const uint32_t sid = 0x20000000u | static_cast<uint32_t>(tp->seed_stream + tp->rounds);
    st = flow_points(f, true, sid, n, f->d_tu, f->d_tlq);
    if (st == GRN_OK)
      st = vegas_pass(e, tp->prec, 0, 0, sid, f->d_tu.as<float>(), f->d_tlq.as<float>());
    if (st == GRN_OK) {
      const double m1 = e->h_sc[grn::VS_FSUM] / n, m2 = e->h_sc[grn::VS_F2SUM] / n;
      r.rel_var_flow = m2 / (m1 * m1) - 1.0;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  d_losses.release();
  e->have_last = false;  // the training passes are not integration passes
  e->last_fu   = nullptr;
  const grn_status st2 = set_ncall(e, ncall0);
  if (st == GRN_OK) st = st2;
  if (out) *out = r;
  return st;
}

grn_status grn_flow_iteration(grn_engine *e, grn_flow *f, int32_t mode, uint32_t iter_id,
                              grn_vegas_result *out) {
  if (!e || !f || f->e != e) return fail(GRN_ERR_INVALID, "bad argument");
  if (!e->vegas_ready) return fail(GRN_ERR_STATE, "grn_vegas_init first");
  grn_status st = require_screening_ready(e);
  if (st != GRN_OK) return st;
  GRN_CUDA(cudaSetDevice(e->device));
  st = flow_points(f, true, iter_id, e->ncall, f->d_fu, f->d_flq);
  if (st != GRN_OK) return st;
  st = vegas_pass(e, e->prec, mode != 0, 0, iter_id, f->d_fu.as<float>(), f->d_flq.as<float>());
  if (st != GRN_OK) return st;
  st = flow_check_err(f);
  if (st != GRN_OK) return st;
  grn_vegas_result r{};
  st = vegas_accumulate(e, mode, e->iters_since_clear++, &r);
  if (out) *out = r;
  return st;
}

grn_status grn_flow_integrate(grn_engine *e, grn_flow *f, const grn_vegas_params *vp,
                              grn_vegas_result *out) {
  if (!e || !f || !vp || f->e != e) return fail(GRN_ERR_INVALID, "bad argument");
  if (!e->vegas_ready) return fail(GRN_ERR_STATE, "grn_vegas_init first");
  if (vp->ncall < 1 || !(vp->precision > 0)) return fail(GRN_ERR_INVALID, "bad VEGAS parameters");
  grn_status st = set_ncall(e, vp->ncall);
  if (st != GRN_OK) return st;
  e->prec = vp->prec;
  grn_vegas_clear(e);
  e->maxf = e->maxW = 0.0;
  grn_vegas_result r{};
  int64_t its = 0;
  const int64_t itmin = std::max<int32_t>(2, vp->iter), itmax = 10000;
  for (; its < itmax; ++its) {
    st = grn_flow_iteration(e, f, 1, e->next_stream++, &r);
    if (st != GRN_OK) return st;
    if (its + 1 >= itmin && r.sigma > 0 && r.sigma_err / r.sigma <= vp->precision) {
      ++its;
      break;
    }
  }
  r.iterations = its;
  if (out) *out = r;
  return GRN_OK;
}

}  // extern "C"
