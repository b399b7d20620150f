/*
 * graniitti_gb300.h — C ABI of the GB300 event-weight engine.
 *
 * The engine replaces one data-parallel path of the GRANIITTI generator:
 *   unit-hypercube point u  ->  phase-space map  ->  |M|^2  ->  (eikonal kt-loop
 *   screening)  ->  event weight  ->  VEGAS accumulate / refine  ->  unweighting.
 * Every entry point below names the reference interface it stands in for
 * (paths relative to the GRANIITTI source tree).
 *
 * Conventions
 *   - Plain C types only; no exceptions cross this boundary. Every call returns a
 *     grn_status; grn_last_error() gives a message for the calling thread.
 *   - Array arguments may be host or device pointers unless stated otherwise;
 *     host arrays are staged through engine-owned device buffers (the copies are
 *     part of the call). Device arrays are used in place.
 *   - All work is ordered on the engine's CUDA stream (grn_engine_stream).
 *   - One engine per host thread. An engine is not re-entrant.
 *   - Units: GeV, GeV^2, weights in barn (the reference's convention).
 */
#ifndef GRANIITTI_GB300_H
#define GRANIITTI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                               */
/* ------------------------------------------------------------------------ */
typedef int32_t grn_status;
enum {
  GRN_OK              = 0,
  GRN_ERR_INVALID     = 1, /* bad argument or configuration                 */
  GRN_ERR_CUDA        = 2, /* CUDA runtime error (message has the detail)    */
  GRN_ERR_UNSUPPORTED = 3, /* process / option not implemented by the engine */
  GRN_ERR_NAN         = 4, /* more than 50 NaN/Inf weights (MProcess.h:317) */
  GRN_ERR_STATE       = 5, /* call order violated (e.g. tables not built)   */
  GRN_ERR_NO_DEVICE   = 6  /* no CUDA device visible                         */
};

/* Per-point flag bits: the four AuxIntData booleans (MProcess.h:37-52). */
enum {
  GRN_FLAG_KINEMATICS_OK = 1,
  GRN_FLAG_FIDCUTS_OK    = 2,
  GRN_FLAG_VETOCUTS_OK   = 4,
  GRN_FLAG_AMPLITUDE_OK  = 8
};

/* Process kinds: the PROC_k wrappers of MSubProc.h the engine implements. */
enum {
  GRN_PROC_REGGE_CON  = 1, /* "PP[CON]<C|F> -> a b", 2-body, MRegge::ME4 (MSubProc.h:361-380) */
  GRN_PROC_TENSOR_CON = 2, /* "PP[CONTENSOR]<C|F> -> a b", 2 pseudoscalars, tensor-pomeron
                              MTensorPomeron::ME4 "2xS" (MSubProc.h:288-300) */
  GRN_PROC_TENSOR_RES = 3, /* "PP[RESTENSOR]<F|C> -> a b", 2 pseudoscalars: coherent sum of
                              tensor-pomeron resonances, MTensorPomeron::ME3 (MSubProc.h:
                              278-285; src/MTensorPomeron.cc:164-565), J = 0 (P = +1) and
                              J = 2 with the pseudoscalar-pair decay */
  GRN_PROC_TENSOR_RESCON = 4, /* "PP[RES+CONTENSOR]<F|C> -> a b", 2 pseudoscalars: the 2xS
                              continuum and the resonances (0..4) summed coherently
                              (MSubProc.h:319-351) */
  GRN_PROC_REGGE_RES = 5,  /* "PP[RES]<F|C> -> a b", 2 pseudoscalars: Regge resonances
                              (MRegge::ME3 with spin::ProdAmp / DecayAmp), J^P = 0+ and 2+ */
  GRN_PROC_REGGE_RESCON = 6 /* "PP[RES+CON]<F|C> -> a b": the Regge continuum (MRegge::ME4)
                              and the Regge resonances summed coherently (MSubProc.h:398-433) */
};

/* Phase-space classes (MProcess subclasses). */
enum {
  GRN_PS_CONTINUUM  = 1, /* <C>: MContinuum (src/MContinuum.cc), 3 Nf - 4 = 8 dimensions */
  GRN_PS_FACTORIZED = 2  /* <F>: MFactorized (src/MFactorized.cc), 5 + 1 dimensions plus the
                            2-body decay angles (cos theta, phi) lifted into u[6], u[7] */
};

/* Arithmetic of the kt-loop (the tree-level kinematics is always FP64). */
enum {
  GRN_PREC_FP64  = 0, /* everything FP64: parity path against the reference */
  GRN_PREC_MIXED = 1  /* FP64 kinematics, FP32 loop amplitudes with compensated sums */
};

/* ------------------------------------------------------------------------ */
/* Configuration: what MGraniitti::ReadInput + MProcess::post_Constructor     */
/* derive from a steering card (src/MGraniitti.cc:318-963).                   */
/* ------------------------------------------------------------------------ */
typedef struct grn_soft_params { /* PARAM_SOFT, src/MForm.cc:71-151 */
  double delta_P, alpha_P, gN_P, gN_O, g3P, gamma, fc1, fc2, fc3;
  int32_t odderon_on;
  int32_t _pad;
} grn_soft_params;

typedef struct grn_regge_params { /* PARAM_REGGE, src/MRegge.cc:950-1039 */
  double  a0[3], ap[3], sgn[3];
  double  s0;
  int32_t active[3]; /* trajectory on/off ("n") for the final state */
  int32_t offshellFF; /* 0 exponential, 1 Orear, 2 power law */
  double  c[3];       /* final-state couplings ("c") */
  double  b_EXP, a_OREAR, b_OREAR, b_POW;
} grn_regge_params;

typedef struct grn_tensor_params { /* MTensorPomeronParam, include/Graniitti/MTensorPomeron.h:29-99 */
  double  delta_P, ap_P; /* pomeron trajectory: alpha(t) = 1 + delta_P + ap_P t */
  double  gPNN;          /* pomeron-proton-proton coupling */
  double  gPps;          /* pomeron-pseudoscalar coupling (gPpipi or gPKK) */
  int32_t em_kelly;      /* proton Dirac form factor F1: 1 = Kelly, 0 = dipole (PARAM_STRUCTURE EM) */
  int32_t _pad;
  double  gPvv[2];       /* pomeron-vector-vector couplings (gPrhorho or gPphiphi) [GeV^-3, GeV^-1] */
} grn_tensor_params;

/* One resonance of PP[RESTENSOR]: PARAM_RES (src/MForm.cc:250-340) and the decay
 * coupling of its pseudoscalar-pair mode (HELMatrix::g_decay_tensor[0]). */
#define GRN_MAX_RESONANCES 4
typedef struct grn_resonance {
  int32_t J;           /* spin: 0 or 2 */
  int32_t P;           /* parity: +1 (J = 0 with P = -1 decays to photon or vector pairs) */
  double  M, W;        /* peak mass and full width [GeV] (the BW propagators use W fixed) */
  double  g_tensor[7]; /* production couplings g_Tensor: [0], [1] for J = 0 (structures
                          iG_PPS_0, iG_PPS_1); [0] for J = 2 (iG_PPT_00; [1..6] must be 0) */
  double  g_decay;     /* decay coupling, grn_tensor_decay_coupling() unless the model gives it */
  /* Regge model (PP[RES], PP[RES+CON]; PARAM_RES of modeldata RES_*.json): */
  double  g_regge[2];  /* production coupling g_A exp(i g_phi): (re, im) */
  double  g_ff;        /* resonance form factor scale S0 [GeV]: exp(-(m^2 - M^2)^2 / S0^4) */
  int32_t bw;          /* Breit-Wigner form: 1 fixed width, 2 running width, 3 spin barrier,
                          4 spin dependent (MForm.cc:743-830) */
  int32_t _pad_bw;
  double  rho[2][25];  /* spin density matrix of J = 2 (re, im), rows M = -2..2 (J = 0: unused) */
} grn_resonance;

/* Spin polarization frame of the Regge resonances' density matrices (MSpin.cc:544-600). */
enum { GRN_FRAME_CM = 0, GRN_FRAME_HX = 1, GRN_FRAME_CS = 2 };

typedef struct grn_gencuts { /* GENCUT, include/Graniitti/MKinematics.h:1554-1576 */
  double rap_min, rap_max;       /* <C> final-state rapidity window */
  double kt_min, kt_max;         /* <C> intermediate kt (post_Constructor default 10/Kf) */
  double fpt_min, fpt_max;       /* forward-leg pT (SetTechnicalBoundaries default 0, 2.5) */
  double Y_min, Y_max;           /* <F> central-system rapidity window */
  double M_min, M_max;           /* <F> central-system mass window */
} grn_gencuts;

typedef struct grn_fidcuts { /* FIDCUT, include/Graniitti/MKinematics.h:1579-1611 */
  int32_t active;
  int32_t _pad;
  double  eta_min, eta_max, rap_min, rap_max, pt_min, pt_max, Et_min, Et_max;
  double  M_min, M_max, Y_min, Y_max, Pt_min, Pt_max;
  double  ft_min, ft_max, fM_min, fM_max;
} grn_fidcuts;

typedef struct grn_loop_numerics { /* MEikonalNumerics, include/Graniitti/MEikonal.h:26-95 */
  int32_t n_kt;      /* NumberLoopKT: kt intervals (multiple of 3) */
  int32_t n_phi;     /* NumberLoopPHI: phi intervals (multiple of 3) */
  double  kt_min;    /* MinLoopKT */
  double  kt_max;    /* MaxLoopKT */
  int32_t n_bt;      /* NumberBT: density-table intervals (even) */
  int32_t n_kt2;     /* NumberKT2: screening-table intervals (even) */
} grn_loop_numerics;

#define GRN_MAX_VETO 8 /* veto domains */

typedef struct grn_process_params {
  int32_t process;        /* GRN_PROC_* */
  int32_t phase_space;    /* GRN_PS_* */
  int32_t n_central;      /* first-level central final states (2 supported) */
  int32_t screening;      /* POMLOOP */
  double  sqrt_s;         /* from the beam energies (symmetric beams) */
  double  m_beam;         /* beam (and elastic forward) mass */
  double  m_central[8];   /* central final-state masses */
  double  s_factor;       /* identical-particle symmetry factor (MProcess.cc:449) */
  grn_gencuts       gcuts;
  grn_fidcuts       fcuts;
  grn_soft_params   soft;
  grn_regge_params  regge;   /* also the off-shell meson form factor of the tensor model */
  grn_loop_numerics loop;
  grn_tensor_params tensor;
  int32_t           n_res;   /* GRN_PROC_TENSOR_RES: resonances in the coherent sum (1..4) */
  int32_t           _pad_res;
  grn_resonance     res[GRN_MAX_RESONANCES];
  /* Decay cascade of the two central particles, "a > {c d} b > {e f}" (MDecayBranch legs,
   * include/Graniitti/MParticle.h:60-90), in the <C> and <F> classes: each central particle
   * has an off-shell mass drawn from a relativistic Breit-Wigner within +-OFFSHELL widths
   * (MProcess::GetOffShellMass, src/MProcess.cc:753-812) and decays isotropically to two
   * daughters (ConstructDecayKinematics, :1231-1283). The draws are extra hypercube
   * coordinates after the 8 of the 2-body point: u[8], u[9] the two masses, u[10..11] and
   * u[12..13] the two decays (cos theta, phi), 14 dimensions; with OFFSHELL = 0 (process
   * command @OFFSHELL:0) the masses are the pole masses and the decays take u[8..11], 12
   * dimensions. */
  int32_t           n_decay;      /* 0: stable central particles; 2: two-body cascades */
  int32_t           central_spin; /* spin of the central particles (0 or 1: "2xS" / "2xV") */
  double            width[2];     /* widths of the central particles [GeV] */
  double            m_daughter[4];/* daughter masses: central 1 -> [0], [1]; 2 -> [2], [3] */
  /* Regge resonances: spin correlations of production (SPINGEN) and decay (SPINDEC), the
   * frame of the density matrices (GRN_FRAME_*), the flux exponent (PARAM_REGGE omega) */
  int32_t           spin_gen, spin_dec, spin_frame;
  /* OFFSHELL, the number of widths of the Breit-Wigner mass draws of cascades
   * (include/Graniitti/MProcess.h:363): offshell when offshell_user is set (process command
   * @OFFSHELL:x, MProcess::SetOFFSHELL), else the reference default 5 */
  int32_t           offshell_user;
  double            omega;
  double            offshell;
  /* Veto cuts (VETOCUTS, MProcess::VetoCuts / FindVetoCuts, src/MProcess.cc:1069-1175): an
   * event is rejected when any final-state particle of the central system (the leaves of the
   * decay tree) has pt_min[k] <= pT <= pt_max[k] and eta_min[k] <= eta <= eta_max[k] for some
   * domain k < n_veto. Elastic forward protons are not tested (the reference tests only the
   * fragments of excited forward systems). */
  int32_t           veto_active, n_veto;
  double            veto_eta_min[GRN_MAX_VETO], veto_eta_max[GRN_MAX_VETO];
  double            veto_pt_min[GRN_MAX_VETO], veto_pt_max[GRN_MAX_VETO];
  /* Forward excitation (NSTARS, MProcess::SampleForwardMasses, src/MProcess.cc:1317-1365):
   * 0 elastic forward protons, 1 one of them excited (the side drawn 50-50), 2 both. The
   * excited masses^2 are drawn log-uniformly in [1.09^2, xi_max s] (GENCUTS "Xi"); the
   * excited leg's vertex is sqrt(g3P gN_P) S3FINEL(t, M^2) (MRegge::PomPomProtonVertex). The
   * hypercube gains the mass coordinates and, for 1, the side choice (2-body states: 10
   * dimensions). Implemented for the Regge continuum of two central particles. */
  int32_t           excitation;
  int32_t           _pad_x;
  double            xi_max;
} grn_process_params;

/* Fill every field with the reference defaults for "PP[CON]<C> -> pi+ pi-" at
 * sqrt(s) = 13 TeV, TUNE0 (modeldata/TUNE0/GENERAL.json), cuts as documented. */
void grn_default_params(grn_process_params *p);

/* Decay coupling of a spin-J resonance (mass M, full width W) to two pseudoscalars of mass
 * m_daughter with branching ratio BR: MTensorPomeron::GDecay (src/MTensorPomeron.cc:134-156)
 * with the threshold retry of MProcess::ProcessHelicityDecay (src/MProcess.cc:683-703): when
 * M is below 2 m_daughter the coupling is taken at M + i W, i = 1, 2, 3, the first one above
 * threshold. Returns NaN for J other than 0, 1, 2. */
double grn_tensor_decay_coupling(int32_t J, double M, double W, double m_daughter, double BR);
/* Decay coupling of the Regge resonances (PP[RES], PP[RES+CON]) to two particles of mass
 * m_daughter: sqrt(BR W / Gamma_PS), Gamma_PS the two-body width with |A|^2 = 1
 * (MProcess::ProcessHelicityDecay, src/MProcess.cc:670-713), with the same threshold retry. */
double grn_regge_decay_coupling(double M, double W, double m_daughter, double BR);

/* ------------------------------------------------------------------------ */
/* Engine lifetime                                                            */
/* ------------------------------------------------------------------------ */
typedef struct grn_engine grn_engine;

/* Replaces process construction + MProcess::post_Constructor
 * (src/MGraniitti.cc:245-276, src/MContinuum.cc:64-89). */
grn_status grn_create(const grn_process_params *p, int32_t device, grn_engine **out);
grn_status grn_destroy(grn_engine *e);
/* CUDA stream (cudaStream_t) of the engine, as an opaque pointer. */
void *grn_engine_stream(grn_engine *e);
/* Phase-space dimension (MProcess::GetdLIPSDim, include/Graniitti/MProcess.h:160). */
int32_t grn_dim(const grn_engine *e);
/* The parameters the engine was created with (owned by the engine). */
const grn_process_params *grn_engine_params(const grn_engine *e);
/* Message of the last failing call on this thread (never NULL). */
const char *grn_last_error(void);
/* Library version string. */
const char *grn_version(void);

/* ------------------------------------------------------------------------ */
/* Eikonal tables                                                             */
/* ------------------------------------------------------------------------ */
/* Builds the impact-parameter density table (MBT) and the kt^2 screening
 * amplitude table (MSA) on the device and the eikonal cross sections.
 * Replaces MEikonal::S3Constructor (src/MEikonal.cc:46-132) including
 * S3Density (177-216), S3Screening (222-245) and S3CalcXS (254-376, single
 * channel). n_bt / n_kt2 <= 0 take the values in the process parameters. */
grn_status grn_eikonal_build(grn_engine *e, int32_t n_bt, int32_t n_kt2);
/* sigma_tot, sigma_el, sigma_inel in barn (MEikonal::GetTotXS, MEikonal.cc:39-43). */
grn_status grn_eikonal_xs(grn_engine *e, double *tot, double *el, double *inel);
/* Copy tables out: rows of (x, Re, Im); mbt has n_bt+1 rows, msa n_kt2+1 rows
 * (IArray1D::F, include/Graniitti/MEikonal.h:149). Host pointers. */
grn_status grn_eikonal_get(grn_engine *e, double *mbt, double *msa);
/* Inject precomputed tables (MGraniitti::Initialize(const MEikonal&),
 * src/MGraniitti.cc:1045-1054; IArray1D::ReadArray, MEikonal.cc:436-482). */
grn_status grn_eikonal_set(grn_engine *e, int32_t n_bt, const double *mbt, int32_t n_kt2,
                           const double *msa);

/* ------------------------------------------------------------------------ */
/* Event weights: the per-point boundary                                      */
/* ------------------------------------------------------------------------ */
/* Batch form of MProcess::EventWeight(randvec, aux)
 * (include/Graniitti/MProcess.h:84; src/MContinuum.cc:164-193).
 *   u      : n points x dim, point-major (randvec of each point contiguous)
 *   w_out  : n weights [barn], 0 when a cut or the kinematics fails
 *   flags  : n bytes of GRN_FLAG_* (may be NULL)
 *   prec   : GRN_PREC_FP64 or GRN_PREC_MIXED (loop arithmetic)
 * The call is synchronous with respect to the host when any pointer is a host
 * pointer; with device pointers it is stream-ordered. */
grn_status grn_event_weights(grn_engine *e, const double *u, int64_t n, int32_t dim,
                             double *w_out, uint8_t *flags, int32_t prec);

/* Allocation-free variant of grn_event_weights. It has no counterpart in the
 * reference. For callers that may not allocate device memory while running (an
 * application whose device memory belongs to its own pool allocator, a service that
 * sizes its memory once at start-up and must not meet an out-of-memory error or the
 * synchronisation of cudaFree mid-run), this call allocates nothing: its scratch
 * (the screened work list and its FP64 refinement list) is a fixed 16 MiB array inside
 * the library, held by every device that loads the library until the process exits.
 *   - u, w_out and flags must be device pointers; n <= GRN_NOALLOC_MAX_POINTS,
 *     larger batches are rejected with GRN_ERR_INVALID.
 *   - Stream-ordered on the engine's stream; returns without synchronising.
 *   - The first call on a device looks up the scratch address (one-time set-up);
 *     make that first call before any stream capture.
 *   - All calls on a device share the one scratch array: calls that overlap on the
 *     GPU (two engines on different streams, concurrently) race; serialise them.
 *   - The scratch address is kept for the life of the device's primary context: do
 *     not use the library across a cudaDeviceReset.
 *   - dim must equal grn_dim(e) (8 for 2-body states, 12 or 14 for cascades, 14 for
 *     4-body states).
 * Results: identical to grn_event_weights in FP64. In MIXED this call runs the generic
 * FP32 kt-loop with FP64 refinement for every process, while grn_event_weights takes
 * the record-mode loop for screened single-trajectory Regge processes: there the two
 * agree to the FP32-loop tolerance (1e-5 relative), elsewhere exactly. */
#define GRN_NOALLOC_MAX_POINTS 1048576
grn_status grn_event_weights_noalloc(grn_engine *e, const double *u, int64_t n, int32_t dim,
                                     double *w_out, uint8_t *flags, int32_t prec);

/* Kinematics of the same points without the amplitude, for record building and
 * tests: per point 16 doubles = (px,py,pz,E) of the two forward legs and the two
 * central particles (LORENTZSCALAR::pfinal[1..4]), plus t1, t2 into ts (2 per
 * point, may be NULL). Replaces BNRandomKin+BNBuildKin (MContinuum.cc:276-435). */
grn_status grn_event_kinematics(grn_engine *e, const double *u, int64_t n, int32_t dim,
                                double *p4_out, double *ts_out, uint8_t *flags);

/* Cascade processes (n_decay = 2): the four daughters of the two central particles, per
 * point 16 doubles (px, py, pz, E) in the order central 1 -> 2 daughters, central 2 -> 2
 * daughters (the leaves of lts.decaytree, ConstructDecayKinematics). N-body central states
 * (n_central = 4, 6): the central particles (LORENTZSCALAR::pfinal[3..]), 16 or 24 doubles
 * per point. GRN_ERR_STATE for other engines. */
grn_status grn_event_daughters(grn_engine *e, const double *u, int64_t n, int32_t dim,
                               double *pd_out);

/* ------------------------------------------------------------------------ */
/* Counter-based uniforms (Philox4x32-10, Salmon et al., SC'11)               */
/* ------------------------------------------------------------------------ */
/* out[i*dim + d] = uniform double in [0,1) of point (first + i), dimension d,
 * key = seed, stream = stream id. The reference draws from std::ranlux48
 * (include/Graniitti/MRandom.h:62); the engine's draws are counter-based so that
 * any point can be regenerated. */
grn_status grn_uniforms(grn_engine *e, uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                        int32_t dim, double *out);

/* ------------------------------------------------------------------------ */
/* VEGAS                                                                      */
/* ------------------------------------------------------------------------ */
typedef struct grn_vegas_params { /* VEGASPARAM, include/Graniitti/MVEGAS.h:18-32 */
  int32_t bins;       /* BINS (even) */
  int32_t iter;       /* ITER */
  int64_t ncall;      /* NCALL per iteration */
  double  lambda;     /* LAMBDA */
  double  chi2max;    /* CHI2MAX */
  double  precision;  /* PRECISION (relative) */
  int32_t burnin_iter;/* BURN-IN iterations (SampleVegas default 3) */
  int32_t prec;       /* GRN_PREC_* of the weights */
  uint64_t seed;      /* Philox key */
} grn_vegas_params;

typedef struct grn_vegas_result {
  double  sigma, sigma_err, chi2;  /* global estimates [barn] (MGraniitti.cc:1222-1251) */
  double  I_this, I2_this;         /* this iteration's integral and error^2 */
  double  maxf, maxW;              /* max VEGAS-weighted f and raw W (init > 0 only) */
  double  evaluations;             /* Stats::evaluations */
  double  amplitude_ok, kinematics_ok, fidcuts_ok, vetocuts_ok; /* pass counts */
  int64_t iterations;              /* iterations run in this call */
  int64_t nan_count;               /* NaN/Inf weights zeroed */
  int64_t refined;                 /* events of the last pass whose FP32 kt-loop was redone
                                      in FP64 (error estimate above tolerance, see grn_tuning) */
} grn_vegas_result;

/* VEGASData::Init (MVEGAS.h:38-56) with init = 0 (fresh uniform grid). */
grn_status grn_vegas_init(grn_engine *e, const grn_vegas_params *vp);
/* One VEGAS iteration: draw ncall points, map through the grid, weigh them and
 * accumulate f, f^2 histograms and the global estimates; then, if refine != 0,
 * VEGASData::OptimizeGrid (MVEGAS.h:107-142). mode: 0 = burn-in (init 0, maxf not
 * tracked), 1 = integration (init 1). Replaces one pass of the iteration loop of
 * MGraniitti::VEGAS + VEGASMultiThread (MGraniitti.cc:1146-1443).
 * The weighted values f of the last iteration stay on the device for
 * grn_unweight. */
grn_status grn_vegas_iteration(grn_engine *e, int32_t mode, int32_t refine, uint32_t iter_id,
                               grn_vegas_result *out);
/* Full integration as MGraniitti::SampleVegas with GMODE = 0
 * (src/MGraniitti.cc:1074-1126): burn-in iterations, then integration
 * iterations until PRECISION and CHI2MAX are met (chi2 > 50 restarts with 10x
 * calls). */
grn_status grn_vegas_integrate(grn_engine *e, const grn_vegas_params *vp, grn_vegas_result *out);
/* FLAT integrator (INTEGRATOR "FLAT": MGraniitti::SampleFlat, src/MGraniitti.cc:1446-1524):
 * uniform points, sigma = sum W / N, sigma_err = sqrt((sum W^2 / N - sigma^2) / N)
 * (Stats::CalculateCrossSection, include/Graniitti/MGraniitti.h:59-66), passes of ncall
 * points until sigma_err / sigma < precision and N > min_events (FLATPARAM). The maximum
 * weight (grn_get_maxweight) is max W. The last pass stays on the device for
 * grn_unweight / grn_vegas_points. */
typedef struct grn_flat_params {
  int64_t  ncall;      /* points per pass */
  double   precision;  /* FLAT::PRECISION */
  int64_t  min_events; /* FLAT::MIN_EVENTS */
  int32_t  prec;       /* GRN_PREC_* */
  int32_t  _pad;
  uint64_t seed;       /* Philox key */
} grn_flat_params;
grn_status grn_flat_integrate(grn_engine *e, const grn_flat_params *fp, grn_vegas_result *out);
/* Grid access: xmat as bins x dim doubles, bin-major (VEGASData::xmat). Host. */
grn_status grn_vegas_get_grid(grn_engine *e, double *xmat);
grn_status grn_vegas_set_grid(grn_engine *e, const double *xmat);
/* Clear the global (sumdata, sumchi2, sweight) estimates: VEGASData::ClearIntegral. */
grn_status grn_vegas_clear(grn_engine *e);
/* Maximum weight used for unweighting: max f = W * vw (divided by q for flow
 * passes) over the integration passes so far (MGraniitti::GetMaxweight /
 * SetMaxweight, src/MGraniitti.cc:966-985). Setting 0 starts a fresh maximum
 * (the reference requires > 0: one generator object runs one integration). */
grn_status grn_get_maxweight(grn_engine *e, double *maxf);
grn_status grn_set_maxweight(grn_engine *e, double maxf);

/* ------------------------------------------------------------------------ */
/* Unweighting                                                                */
/* ------------------------------------------------------------------------ */
/* Hit-or-miss over the last iteration's points: accept point i when
 * U_i < f_i / fmax, count f_i > fmax as overflow (rejected).
 * Replaces the acceptance test of MGraniitti::SaveEvent (MGraniitti.cc:1651-1664).
 * idx_out (capacity cap, host or device, may be NULL) receives the accepted
 * point indices in increasing order. */
grn_status grn_unweight(grn_engine *e, double fmax, uint64_t seed, int64_t *n_accepted,
                        int64_t *n_overflow, int64_t *idx_out, int64_t cap);
/* The u vectors of points of the last iteration (n x dim, host), for record
 * building (MProcess::EventRecord on the host). */
grn_status grn_vegas_points(grn_engine *e, const int64_t *idx, int64_t n, double *u_out);

/* The weights f = W vw (/ q for flow passes) of every point of the last iteration, in point
 * order (n = the pass's ncall; host or device). */
grn_status grn_pass_weights(grn_engine *e, double *f_out, int64_t n);

/* ------------------------------------------------------------------------ */
/* On-the-fly histograms (MUserHistograms, src/MUserHistograms.cc:23-125)     */
/* ------------------------------------------------------------------------ */
/* Observables of a point (the reference's level-1 and level-2 histograms): central system
 * mass, rapidity, pT; |delta phi| and pT of the forward legs; mass of the first central
 * particle (cascades); rapidities of the two central particles; cos(theta) and phi of the
 * first central particle in the Collins-Soper, helicity, anti-helicity, pseudo-Gottfried-Jackson
 * (beam 2) and non-rotated rest frames of the system (kinematics::LorentzFrame,
 * MKinematics.h:952-1011) and in the lab. */
enum {
  GRN_OBS_M = 0, GRN_OBS_Y, GRN_OBS_PT, GRN_OBS_DPHI_PP, GRN_OBS_PT1, GRN_OBS_M0,
  GRN_OBS_RAP3, GRN_OBS_RAP4,
  GRN_OBS_COSTH_CS, GRN_OBS_PHI_CS, GRN_OBS_COSTH_HX, GRN_OBS_PHI_HX,
  GRN_OBS_COSTH_AH, GRN_OBS_PHI_AH, GRN_OBS_COSTH_PG, GRN_OBS_PHI_PG,
  GRN_OBS_COSTH_CM, GRN_OBS_PHI_CM, GRN_OBS_COSTH_LA, GRN_OBS_PHI_LA,
  GRN_NUM_OBS
};
/* One histogram: nbins uniform bins of [lo, hi) of obs; 2D with nbins2 > 0 (bin index
 * ix * nbins2 + iy). */
typedef struct grn_hist_spec {
  int32_t obs, nbins;
  double  lo, hi;
  int32_t obs2, nbins2;
  double  lo2, hi2;
} grn_hist_spec;
#define GRN_MAX_HIST 32
/* Replace the engine's histograms by n specs (cleared). */
grn_status grn_hist_define(grn_engine *e, const grn_hist_spec *specs, int32_t n);
/* Add the points of the last iteration (VEGAS, flow or batched pass) with f > 0, each with
 * weight f (the reference's total weight W x VEGAS weight), on the device. */
grn_status grn_hist_fill(grn_engine *e);
/* Histogram h: sum of weights and of squared weights and the fill count per bin; outside[3]:
 * fills below, above (either coordinate) and NaN. Any pointer may be NULL. */
grn_status grn_hist_get(grn_engine *e, int32_t h, double *w, double *w2, int64_t *counts,
                        int64_t *outside);
grn_status grn_hist_clear(grn_engine *e);

/* ------------------------------------------------------------------------ */
/* Learned proposal: coupling-layer spline flow in front of the VEGAS map     */
/* ------------------------------------------------------------------------ */
/* Counterpart of the reference's neural-network integrator (INTEGRATOR
 * "NEURO": MGraniitti::SampleNeuro, src/MGraniitti.cc:1527-1620, network and
 * optimiser in include/Graniitti/MNeuroJacobian.h), which samples u through a
 * trained map and weighs each point by EventWeight(u) * |det du/dz| / p(z).
 * Here the map is a normalizing flow over the hypercube placed in front of the
 * VEGAS grid: z uniform -> u = T^{-1}(z) (flow) -> x = VEGAS map(u) -> W(x);
 * the exact weight of a point is f = W(x) * vw(u) / q(u), so the estimator is
 * unbiased whatever the training reached. Architecture: `layers` coupling
 * layers (the transformed half alternates through six fixed masks), each a
 * rational-quadratic spline with `bins` bins whose parameters come from an MLP
 * 4 -> hidden -> ReLU -> hidden -> ReLU -> 4 * (3 bins + 1); BF16 operands on the
 * tensor cores with FP32 accumulation, FP32 splines, FP32 master weights.
 * Points are dimension-major float arrays (dim x n). */
typedef struct grn_flow grn_flow;

typedef struct grn_flow_params {
  int32_t  dim;     /* must equal grn_dim(): 8 (2-body), 12 or 14 (two-body cascades) */
  int32_t  layers;  /* coupling layers, 1..12 (default 6) */
  int32_t  hidden;  /* MLP width: 128 (default) or 256 */
  int32_t  bins;    /* spline bins (16) */
  uint64_t seed;    /* initial weights */
  double   mix_uniform; /* alpha in [0, 1): passes sample alpha * uniform + (1 - alpha) * flow,
                           so every weight is at most (plain VEGAS weight) / alpha (default 0) */
} grn_flow_params;

#define GRN_FLOW_LOSS_KL       0 /* weighted maximum likelihood: -E[f log q] */
#define GRN_FLOW_LOSS_VARIANCE 1 /* variance of the weights: E[f^2 q0 / q] */

typedef struct grn_flow_train_params {
  int64_t  n_train;     /* points per training round (multiple of batch) */
  int64_t  batch;       /* points per Adam step */
  int32_t  epochs;      /* passes over a round's points */
  int32_t  rounds;      /* round 0 draws plain VEGAS points, later rounds the flow's */
  double   lr;          /* Adam step size */
  int32_t  loss;        /* GRN_FLOW_LOSS_* */
  int32_t  prec;        /* GRN_PREC_* of the training weights */
  uint32_t seed_stream; /* first Philox stream id of the training passes */
  uint32_t _pad;
} grn_flow_train_params;

typedef struct grn_flow_train_result {
  int64_t steps;          /* Adam steps taken */
  double  loss_first;     /* batch loss of the first and the last step */
  double  loss_last;
  double  rel_var_start;  /* <f^2>/<f>^2 - 1 of the first training pass (plain VEGAS points) */
  double  rel_var_flow;   /* the same over a fresh pass drawn from the trained flow */
  double  train_ms;       /* device time of the training (passes + steps) */
} grn_flow_train_result;

void       grn_flow_default_params(grn_flow_params *p);
/* The flow lives on the engine's device and stream. */
grn_status grn_flow_create(grn_engine *e, const grn_flow_params *p, grn_flow **out);
grn_status grn_flow_destroy(grn_flow *f);
/* Diagnostic control of the flow's tensor-core forward kernel (no counterpart in the
 * reference): every wait of the kernel on a copy or a product is bounded, and a wait that
 * gives up makes the call return GRN_ERR_CUDA (outputs invalid) after the kernel has let
 * its copies and products in flight complete and released its tensor memory. polls >= 0
 * sets the poll limit of each CTA's first wait (its first weight copy; 0 gives up at once,
 * the way to exercise that path); polls < 0 restores the default (2^22 polls). Applies to
 * the (8, 128) shape. The flow stays usable after such an error. */
grn_status grn_flow_set_wait_polls(grn_flow *f, int32_t polls);
int64_t    grn_flow_num_params(const grn_flow *f);
/* FP32 master weights, layer after layer: W1[4][H], b1[H], W2[H][H], b2[H],
 * W3[H][4(3K+1)], b3[4(3K+1)] (row-major [in][out]). Host or device pointer.
 * Setting them resets the optimiser state. */
grn_status grn_flow_get_params(grn_flow *f, float *theta);
grn_status grn_flow_set_params(grn_flow *f, const float *theta);
/* Density direction: z = T(x) (z_out may be NULL) and log q(x). */
grn_status grn_flow_density(grn_flow *f, const float *x, int64_t n, float *z_out, float *logq);
/* Sampling direction from given z: x = T^{-1}(z) and log q(x). */
grn_status grn_flow_inverse(grn_flow *f, const float *z, int64_t n, float *x_out, float *logq);
/* Sampling with z = Philox uniforms of points first..first+n-1 (key seed, stream id). */
grn_status grn_flow_sample(grn_flow *f, uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                           float *x_out, float *logq);
/* Batch loss (mean over n points) and its gradient with respect to the master
 * weights (grad: grn_flow_num_params floats, may be NULL). loss kind as
 * GRN_FLOW_LOSS_*: variance: mean coef exp(-log q); KL: -mean coef log q. */
grn_status grn_flow_loss_grad(grn_flow *f, const float *x, const float *coef, int64_t n,
                              int32_t kind, double *loss, float *grad);
/* grn_flow_loss_grad followed by one Adam step (beta1 0.9, beta2 0.999, eps 1e-8). */
grn_status grn_flow_train_step(grn_flow *f, const float *x, const float *coef, int64_t n,
                               int32_t kind, double lr, double *loss);
/* Train on weights the engine generates with its current VEGAS grid (which the
 * flow then sits in front of; keep the grid fixed afterwards). */
grn_status grn_flow_train(grn_engine *e, grn_flow *f, const grn_flow_train_params *tp,
                          grn_flow_train_result *out);
/* One integration pass of e's ncall points drawn from the flow; no grid
 * refinement; updates the global estimates like grn_vegas_iteration and leaves
 * f on the device for grn_unweight / grn_vegas_points. */
grn_status grn_flow_iteration(grn_engine *e, grn_flow *f, int32_t mode, uint32_t iter_id,
                              grn_vegas_result *out);
/* Clear the estimates and the maximum weight, then flow passes of vp->ncall points until
 * sigma_err / sigma <= vp->precision (at least max(2, vp->iter) passes). */
grn_status grn_flow_integrate(grn_engine *e, grn_flow *f, const grn_vegas_params *vp,
                              grn_vegas_result *out);

/* ------------------------------------------------------------------------ */
/* Event records: the output path of MGraniitti::SaveEvent                   */
/* ------------------------------------------------------------------------ */
/* Writes unweighted (or weighted) events in the generator's output formats
 * (FORMAT "hepmc3", "hepmc2", "hepevt"; src/MGraniitti.cc:180-211, 1665-1715) with the
 * event-record layout of MProcess::CommonRecord (src/MProcess.cc:1588-1680): beams
 * (status 4), forward protons (1), two generic propagators (PDG 99, status 81), the
 * central system (PDG 90, status 81) and its two daughters (1); four vertices; the
 * cross section in pb with every event (GenCrossSection) and the event weight.
 * The text is produced by the library itself (HepMC3's ASCII v3 / HepMC2 IO_GenEvent /
 * HEPEVT layouts), so no HepMC installation is needed. */
typedef struct grn_writer grn_writer;
enum { GRN_FORMAT_HEPMC3 = 0, GRN_FORMAT_HEPMC2 = 1, GRN_FORMAT_HEPEVT = 2 };
/* tool / card: the generator name and the steering-card path recorded in the run
 * information (may be NULL). */
grn_status grn_writer_open(const char *path, int32_t format, const char *tool, const char *card,
                           grn_writer **out);
grn_status grn_writer_close(grn_writer *w);
/* Events from hypercube points u (n x dim, host, point-major: e.g. from
 * grn_vegas_points): kinematics by grn_event_kinematics (and grn_event_daughters), PDG codes
 * in pdg[n_pdg]: the beams and the two central particles (n_pdg = 3), followed for cascades
 * by the four daughters (n_pdg = 7; the central particles are then written with status 2 and
 * their decay vertices, WriteDecayKinematics, src/MProcess.cc:1289-1315, at the origin), or
 * for N-body central states the beams and the central particles (n_pdg = 1 + n_central),
 * weight written with every event (1 for unweighted events), cross section and error in pb.
 * Event numbers continue from the writer's count. Points whose kinematics fail are skipped
 * (*written says how many were written). */
grn_status grn_write_events(grn_writer *w, grn_engine *e, const double *u, int64_t n,
                            const int32_t *pdg, int32_t n_pdg, double weight, double sigma_pb,
                            double sigma_err_pb, int64_t *written);
/* The same from 4-vectors already at hand: p4 = n x 16 doubles, (px, py, pz, E) of the
 * two forward legs and the two central particles (the layout of grn_event_kinematics);
 * mass = beam and the two central masses; symmetric beams of total energy sqrt_s. */
grn_status grn_write_records(grn_writer *w, const double *p4, int64_t n, const int32_t pdg[3],
                             const double mass[3], double sqrt_s, double weight, double sigma_pb,
                             double sigma_err_pb);
/* Cascades from 4-vectors: p4 as for grn_write_records (the central particles with their
 * off-shell masses), pd = n x 16 doubles of the four daughters (grn_event_daughters);
 * pdg, mass: beam, the two central particles, the four daughters. */
grn_status grn_write_cascade_records(grn_writer *w, const double *p4, const double *pd, int64_t n,
                                     const int32_t pdg[7], const double mass[7], double sqrt_s,
                                     double weight, double sigma_pb, double sigma_err_pb);

/* ------------------------------------------------------------------------ */
/* Several processes in one pass (no counterpart in the reference)            */
/* ------------------------------------------------------------------------ */
/* A batch runs one integration pass of every engine it holds (1..8 processes on one
 * device, each with its own VEGAS grid, ncall, seed and buffers) as two fused launches:
 * stage A of all processes (blocks in proportion to their points), then one persistent
 * stage-B launch whose blocks take chunks of work from a queue over the screened events
 * of all processes (dynamic balance between processes of different cost). The pass is
 * captured once as a CUDA graph (one per refine setting) and replayed; per-pass values
 * reach the graph through a pinned table it uploads. Results, the f values of the pass
 * (grn_unweight / grn_vegas_points) and the estimates of each engine are as after
 * grn_vegas_iteration on that engine. Screened processes run the FP32 loop
 * (GRN_PREC_MIXED). Engines cannot be destroyed while a batch holds them. */
typedef struct grn_batch grn_batch;
grn_status grn_batch_create(grn_engine *const *engines, int32_t n, grn_batch **out);
grn_status grn_batch_destroy(grn_batch *b);
/* results: one grn_vegas_result per engine (may be NULL); device_ms: device time of the
 * whole pass (may be NULL). */
grn_status grn_batch_iteration(grn_batch *b, int32_t mode, int32_t refine, uint32_t iter_id,
                               grn_vegas_result *results, double *device_ms);
/* Member `index` draws its points from the flow f (created on that member's engine; NULL:
 * Philox points again): each grn_batch_iteration first samples them on the engine's stream
 * exactly as grn_flow_iteration with the same iter_id, then the member's weights are
 * f = W vw / q. A flow that serves a batch cannot be destroyed. */
grn_status grn_batch_set_flow(grn_batch *b, int32_t index, grn_flow *f);

/* ------------------------------------------------------------------------ */
/* Launch configuration and autotuner (no counterpart in the reference)       */
/* ------------------------------------------------------------------------ */
/* The kt-loop stage in record mode (screened, GRN_PREC_MIXED, one trajectory) has two
 * kernels: one event per thread, or two events per thread on the packed FP32x2
 * arithmetic (same results up to FP32 rounding), each with a grid size.
 * fp64_refine (default 1): with GRN_PREC_MIXED, the FP32 generic kt-loop (tensor pomeron,
 * resonances, vector pairs, several Regge trajectories) also sums |U_i c_j| |A_ij| over
 * its points; an event whose estimated relative weight error 16 2^-24 |norm| sum / |A| is
 * above 1e-5 is recomputed with the FP64 loop in a second pass of the same call (the phi
 * integrals of some tensor couplings cancel by up to 10^12). 0 keeps every FP32 weight. */
typedef struct grn_tuning {
  int32_t loop_pair;     /* 0 one event per thread, 1 two events per thread, 2 two events per
                            thread with 3 resident blocks per SM (168 registers) */
  int32_t vegas_blocks;  /* grid of the loop stage of VEGAS and flow passes */
  int32_t weight_blocks; /* grid of the loop stage of grn_event_weights */
  int32_t fp64_refine;   /* 1 recompute badly conditioned FP32-loop events in FP64, 0 never */
  double  refine_tol;    /* relative weight error above which an FP32-loop event's estimated
                            rounding sends it to FP64 (default 1e-5; in [1e-9, 1]) */
  int32_t born_blocks;   /* grid of the VEGAS stage A (kinematics, cuts, records); 0 default */
  int32_t generic_blocks;/* grid of the FP32 generic loop stage of VEGAS passes (processes
                            outside record mode); 0 one resident wave */
} grn_tuning;
grn_status grn_get_tuning(grn_engine *e, grn_tuning *t);
grn_status grn_set_tuning(grn_engine *e, const grn_tuning *t);

#define GRN_TUNE_MAX 16
typedef struct grn_tune_result {
  grn_tuning best;           /* the configuration kept */
  int32_t    n_candidates;
  int32_t    _pad;
  double     ms[GRN_TUNE_MAX];   /* stage time of each candidate (best of 2 after a warm-up) */
  grn_tuning cand[GRN_TUNE_MAX];
  int32_t    stage[GRN_TUNE_MAX];/* what candidate k varies: 0 the stage-A grid, 1 the record
                                    loop's variant and grid, 2 the generic FP32 loop's grid */
  int64_t    sample_events;  /* listed (screened) events the loop candidates were timed on */
} grn_tune_result;
/* Times the candidates with CUDA events on the engine stream and keeps the fastest of each
 * stage. Once grn_vegas_init has run, on a full VEGAS pass of the engine (ncall points, its
 * grid; sample is then unused): the stage-A grid (1, 2, 4, 8 times its resident blocks), then
 * on one stage-A output the loop stage: in record mode the kernel variant x grid (1 to 8 times
 * the resident blocks), otherwise the FP32 generic loop's grid (1, 2, 4 resident waves; MIXED
 * passes). Without VEGAS, the record loop on the loop records of `sample` Philox points
 * through grn_event_weights' kernels. Needs the eikonal tables of screened processes. */
grn_status grn_autotune(grn_engine *e, int64_t sample, grn_tune_result *out);

/* ------------------------------------------------------------------------ */
/* Measurement helpers (no counterpart in the reference)                      */
/* ------------------------------------------------------------------------ */
/* Device time of the dominant kernel of a VEGAS pass (the kt-loop stage when
 * screening is on), accumulated from CUDA events recorded around each launch on
 * the engine stream since the last reset. */
grn_status grn_kernel_timing(grn_engine *e, int32_t reset, double *total_ms, int64_t *launches);
/* FP32 FMA throughput of the device in TFLOP/s (2 flops per FMA), measured with
 * a register-resident FMA-chain kernel over every SM. */
grn_status grn_fp32_peak(int32_t device, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* GRANIITTI_GB300_H */
