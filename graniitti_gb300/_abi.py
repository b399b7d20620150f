"""ctypes mirror of include/graniitti_gb300.h and the loader of the CUDA library.

The library is built in-tree (graniitti_gb300/_build/libgrn.so) by
graniitti_gb300.build.build_library(). Loading never falls back to anything:
a missing or unloadable library raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgrn.so")

c_double = ctypes.c_double
c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_uint32 = ctypes.c_uint32
c_uint64 = ctypes.c_uint64
c_void_p = ctypes.c_void_p

# Status codes
GRN_OK = 0
GRN_ERR_INVALID = 1
GRN_ERR_CUDA = 2
GRN_ERR_UNSUPPORTED = 3
GRN_ERR_NAN = 4
GRN_ERR_STATE = 5
GRN_ERR_NO_DEVICE = 6

GRN_FLAG_KINEMATICS_OK = 1
GRN_FLAG_FIDCUTS_OK = 2
GRN_FLAG_VETOCUTS_OK = 4
GRN_FLAG_AMPLITUDE_OK = 8

GRN_PROC_REGGE_CON = 1
GRN_PROC_TENSOR_CON = 2
GRN_PROC_TENSOR_RES = 3
GRN_PROC_TENSOR_RESCON = 4
GRN_PROC_REGGE_RES = 5
GRN_PROC_REGGE_RESCON = 6
GRN_FRAME_CM, GRN_FRAME_HX, GRN_FRAME_CS = 0, 1, 2
GRN_MAX_RESONANCES = 4
GRN_MAX_VETO = 8
GRN_PS_CONTINUUM = 1
GRN_PS_FACTORIZED = 2
GRN_PREC_FP64 = 0
GRN_PREC_MIXED = 1
GRN_NOALLOC_MAX_POINTS = 1048576


class SoftParams(ctypes.Structure):
    _fields_ = [(n, c_double) for n in
                ("delta_P", "alpha_P", "gN_P", "gN_O", "g3P", "gamma", "fc1", "fc2", "fc3")] + \
               [("odderon_on", c_int32), ("_pad", c_int32)]


class ReggeParams(ctypes.Structure):
    _fields_ = [("a0", c_double * 3), ("ap", c_double * 3), ("sgn", c_double * 3),
                ("s0", c_double), ("active", c_int32 * 3), ("offshellFF", c_int32),
                ("c", c_double * 3), ("b_EXP", c_double), ("a_OREAR", c_double),
                ("b_OREAR", c_double), ("b_POW", c_double)]


class TensorParams(ctypes.Structure):
    _fields_ = [("delta_P", c_double), ("ap_P", c_double), ("gPNN", c_double), ("gPps", c_double),
                ("em_kelly", c_int32), ("_pad", c_int32), ("gPvv", c_double * 2)]


class GenCuts(ctypes.Structure):
    _fields_ = [(n, c_double) for n in
                ("rap_min", "rap_max", "kt_min", "kt_max", "fpt_min", "fpt_max",
                 "Y_min", "Y_max", "M_min", "M_max")]


class FidCuts(ctypes.Structure):
    _fields_ = [("active", c_int32), ("_pad", c_int32)] + [(n, c_double) for n in (
        "eta_min", "eta_max", "rap_min", "rap_max", "pt_min", "pt_max", "Et_min", "Et_max",
        "M_min", "M_max", "Y_min", "Y_max", "Pt_min", "Pt_max",
        "ft_min", "ft_max", "fM_min", "fM_max")]


class LoopNumerics(ctypes.Structure):
    _fields_ = [("n_kt", c_int32), ("n_phi", c_int32), ("kt_min", c_double), ("kt_max", c_double),
                ("n_bt", c_int32), ("n_kt2", c_int32)]


class Resonance(ctypes.Structure):
    _fields_ = [("J", c_int32), ("P", c_int32), ("M", c_double), ("W", c_double),
                ("g_tensor", c_double * 7), ("g_decay", c_double),
                ("g_regge", c_double * 2), ("g_ff", c_double), ("bw", c_int32),
                ("_pad_bw", c_int32), ("rho", (c_double * 25) * 2)]


class ProcessParams(ctypes.Structure):
    _fields_ = [("process", c_int32), ("phase_space", c_int32), ("n_central", c_int32),
                ("screening", c_int32), ("sqrt_s", c_double), ("m_beam", c_double),
                ("m_central", c_double * 8), ("s_factor", c_double),
                ("gcuts", GenCuts), ("fcuts", FidCuts), ("soft", SoftParams),
                ("regge", ReggeParams), ("loop", LoopNumerics), ("tensor", TensorParams),
                ("n_res", c_int32), ("_pad_res", c_int32),
                ("res", Resonance * GRN_MAX_RESONANCES),
                ("n_decay", c_int32), ("central_spin", c_int32), ("width", c_double * 2),
                ("m_daughter", c_double * 4),
                ("spin_gen", c_int32), ("spin_dec", c_int32), ("spin_frame", c_int32),
                ("offshell_user", c_int32), ("omega", c_double), ("offshell", c_double),
                ("veto_active", c_int32), ("n_veto", c_int32),
                ("veto_eta_min", c_double * GRN_MAX_VETO), ("veto_eta_max", c_double * GRN_MAX_VETO),
                ("veto_pt_min", c_double * GRN_MAX_VETO), ("veto_pt_max", c_double * GRN_MAX_VETO),
                ("excitation", c_int32), ("_pad_x", c_int32), ("xi_max", c_double)]


class VegasParams(ctypes.Structure):
    _fields_ = [("bins", c_int32), ("iter", c_int32), ("ncall", c_int64), ("lambda_", c_double),
                ("chi2max", c_double), ("precision", c_double), ("burnin_iter", c_int32),
                ("prec", c_int32), ("seed", c_uint64)]


class VegasResult(ctypes.Structure):
    _fields_ = [(n, c_double) for n in (
        "sigma", "sigma_err", "chi2", "I_this", "I2_this", "maxf", "maxW", "evaluations",
        "amplitude_ok", "kinematics_ok", "fidcuts_ok", "vetocuts_ok")] + \
               [("iterations", c_int64), ("nan_count", c_int64), ("refined", c_int64)]


class FlatParams(ctypes.Structure):
    _fields_ = [("ncall", c_int64), ("precision", c_double), ("min_events", c_int64),
                ("prec", c_int32), ("_pad", c_int32), ("seed", c_uint64)]


OBS = ["M", "Y", "PT", "DPHI_PP", "PT1", "M0", "RAP3", "RAP4",
       "COSTH_CS", "PHI_CS", "COSTH_HX", "PHI_HX", "COSTH_AH", "PHI_AH", "COSTH_PG", "PHI_PG",
       "COSTH_CM", "PHI_CM", "COSTH_LA", "PHI_LA"]
GRN_NUM_OBS = len(OBS)
GRN_MAX_HIST = 32


class HistSpec(ctypes.Structure):
    _fields_ = [("obs", c_int32), ("nbins", c_int32), ("lo", c_double), ("hi", c_double),
                ("obs2", c_int32), ("nbins2", c_int32), ("lo2", c_double), ("hi2", c_double)]


class Tuning(ctypes.Structure):
    _fields_ = [("loop_pair", c_int32), ("vegas_blocks", c_int32), ("weight_blocks", c_int32),
                ("fp64_refine", c_int32), ("refine_tol", c_double), ("born_blocks", c_int32),
                ("generic_blocks", c_int32)]


GRN_TUNE_MAX = 16


class TuneResult(ctypes.Structure):
    _fields_ = [("best", Tuning), ("n_candidates", c_int32), ("_pad", c_int32),
                ("ms", c_double * GRN_TUNE_MAX), ("cand", Tuning * GRN_TUNE_MAX),
                ("stage", c_int32 * GRN_TUNE_MAX), ("sample_events", c_int64)]


GRN_FORMAT_HEPMC3 = 0
GRN_FORMAT_HEPMC2 = 1
GRN_FORMAT_HEPEVT = 2
FORMATS = {"hepmc3": GRN_FORMAT_HEPMC3, "hepmc2": GRN_FORMAT_HEPMC2, "hepevt": GRN_FORMAT_HEPEVT}

GRN_FLOW_LOSS_KL = 0
GRN_FLOW_LOSS_VARIANCE = 1


class FlowParams(ctypes.Structure):
    _fields_ = [("dim", c_int32), ("layers", c_int32), ("hidden", c_int32), ("bins", c_int32),
                ("seed", c_uint64), ("mix_uniform", c_double)]


class FlowTrainParams(ctypes.Structure):
    _fields_ = [("n_train", c_int64), ("batch", c_int64), ("epochs", c_int32),
                ("rounds", c_int32), ("lr", c_double), ("loss", c_int32), ("prec", c_int32),
                ("seed_stream", c_uint32), ("_pad", c_uint32)]


class FlowTrainResult(ctypes.Structure):
    _fields_ = [("steps", c_int64)] + [(n, c_double) for n in (
        "loss_first", "loss_last", "rel_var_start", "rel_var_flow", "train_ms")]


# Every exported entry point with its ctypes signature (restype, argtypes).
SIGNATURES = {
    "grn_default_params": (None, [c_void_p]),
    "grn_tensor_decay_coupling": (c_double, [c_int32, c_double, c_double, c_double, c_double]),
    "grn_regge_decay_coupling": (c_double, [c_double, c_double, c_double, c_double]),
    "grn_create": (c_int32, [c_void_p, c_int32, c_void_p]),
    "grn_destroy": (c_int32, [c_void_p]),
    "grn_engine_stream": (c_void_p, [c_void_p]),
    "grn_dim": (c_int32, [c_void_p]),
    "grn_last_error": (ctypes.c_char_p, []),
    "grn_version": (ctypes.c_char_p, []),
    "grn_eikonal_build": (c_int32, [c_void_p, c_int32, c_int32]),
    "grn_eikonal_xs": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "grn_eikonal_get": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "grn_eikonal_set": (c_int32, [c_void_p, c_int32, c_void_p, c_int32, c_void_p]),
    "grn_event_weights": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p,
                                    c_int32]),
    "grn_event_weights_noalloc": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p,
                                            c_void_p, c_int32]),
    "grn_event_kinematics": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p,
                                       c_void_p]),
    "grn_uniforms": (c_int32, [c_void_p, c_uint64, c_uint32, c_int64, c_int64, c_int32,
                               c_void_p]),
    "grn_vegas_init": (c_int32, [c_void_p, c_void_p]),
    "grn_vegas_iteration": (c_int32, [c_void_p, c_int32, c_int32, c_uint32, c_void_p]),
    "grn_vegas_integrate": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "grn_flat_integrate": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "grn_engine_params": (c_void_p, [c_void_p]),
    "grn_batch_create": (c_int32, [c_void_p, c_int32, c_void_p]),
    "grn_batch_destroy": (c_int32, [c_void_p]),
    "grn_batch_iteration": (c_int32, [c_void_p, c_int32, c_int32, c_uint32, c_void_p, c_void_p]),
    "grn_batch_set_flow": (c_int32, [c_void_p, c_int32, c_void_p]),
    "grn_get_tuning": (c_int32, [c_void_p, c_void_p]),
    "grn_set_tuning": (c_int32, [c_void_p, c_void_p]),
    "grn_autotune": (c_int32, [c_void_p, c_int64, c_void_p]),
    "grn_writer_open": (c_int32, [ctypes.c_char_p, c_int32, ctypes.c_char_p, ctypes.c_char_p,
                                  c_void_p]),
    "grn_writer_close": (c_int32, [c_void_p]),
    "grn_write_events": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_int32,
                                   c_double, c_double, c_double, c_void_p]),
    "grn_write_cascade_records": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                            c_void_p, c_double, c_double, c_double, c_double]),
    "grn_event_daughters": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p]),
    "grn_write_records": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_double,
                                    c_double, c_double, c_double]),
    "grn_vegas_get_grid": (c_int32, [c_void_p, c_void_p]),
    "grn_vegas_set_grid": (c_int32, [c_void_p, c_void_p]),
    "grn_vegas_clear": (c_int32, [c_void_p]),
    "grn_get_maxweight": (c_int32, [c_void_p, c_void_p]),
    "grn_set_maxweight": (c_int32, [c_void_p, c_double]),
    "grn_unweight": (c_int32, [c_void_p, c_double, c_uint64, c_void_p, c_void_p, c_void_p,
                               c_int64]),
    "grn_vegas_points": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p]),
    "grn_pass_weights": (c_int32, [c_void_p, c_void_p, c_int64]),
    "grn_hist_define": (c_int32, [c_void_p, c_void_p, c_int32]),
    "grn_hist_fill": (c_int32, [c_void_p]),
    "grn_hist_get": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p]),
    "grn_hist_clear": (c_int32, [c_void_p]),
    "grn_kernel_timing": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p]),
    "grn_fp32_peak": (c_int32, [c_int32, c_void_p]),
    "grn_flow_default_params": (None, [c_void_p]),
    "grn_flow_create": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "grn_flow_destroy": (c_int32, [c_void_p]),
    "grn_flow_set_wait_polls": (c_int32, [c_void_p, c_int32]),
    "grn_flow_num_params": (c_int64, [c_void_p]),
    "grn_flow_get_params": (c_int32, [c_void_p, c_void_p]),
    "grn_flow_set_params": (c_int32, [c_void_p, c_void_p]),
    "grn_flow_density": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "grn_flow_inverse": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "grn_flow_sample": (c_int32, [c_void_p, c_uint64, c_uint32, c_int64, c_int64, c_void_p,
                                  c_void_p]),
    "grn_flow_loss_grad": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_void_p,
                                     c_void_p]),
    "grn_flow_train_step": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_double,
                                      c_void_p]),
    "grn_flow_train": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "grn_flow_iteration": (c_int32, [c_void_p, c_void_p, c_int32, c_uint32, c_void_p]),
    "grn_flow_integrate": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load_library(path=LIB_PATH):
    """Load libgrn.so and attach the signatures. Raises when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "graniitti_gb300: CUDA library %s is missing; build it with "
            "graniitti_gb300.build.build_library()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GrnError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("grn status %d: %s" % (status, msg))
        self.status = status


def check(status):
    if status != GRN_OK:
        msg = _lib.grn_last_error().decode() if _lib is not None else "?"
        raise GrnError(status, msg)
