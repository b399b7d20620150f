"""Model and particle data the engine needs, bundled with the package.

Values are those of the generator's TUNE0 parameter set
(modeldata/TUNE0/GENERAL.json: PARAM_SOFT 9-29, PARAM_REGGE 90-129, PARAM_PI 146-149,
PARAM_TENSORPOM 178-201, PARAM_STRUCTURE 207-219; RES_*.json and BRANCHING.json for the
resonances)
and of its PDG 2018 mass/width table (modeldata/mass_width_2018.mcd). Only the
entries the engine's processes use are carried; the layout is this package's own.
"""

TUNES = {
    "TUNE0": {
        "PARAM_SOFT": {
            "DELTA_P": 0.098, "ALPHA_P": 0.065, "gN_P": 8.20, "gN_O": 0.10, "g3P": 0.15,
            "gamma": 0.45, "fc1": 0.34, "fc2": 5.0, "fc3": 10.0, "ODDERON_ON": False,
        },
        "PARAM_REGGE": {
            "a0": [1.088, 0.55, 0.55], "ap": [0.20, 0.93, 0.93], "sgn": [1, -1, 1], "s0": 1.0,
            "offshellFF": 2, "b_EXP": 0.944, "a_OREAR": 0.638, "b_OREAR": 1.886, "b_POW": 0.500,
            "omega": 0.5,
        },
        # Spin correlations of the Regge resonances (GENERAL.json PARAM_SPIN).
        "PARAM_SPIN": {"SPINGEN": True, "SPINDEC": True, "FRAME": "CS"},
        "PARAM_TENSORPOM": {
            "delta_P": 0.0808, "ap_P": 0.25, "gPNN": 1.87, "gPpipi": 1.76, "gPKK": 1.54,
            "gPrhorho": [0.70, 6.20], "gPphiphi": [0.49, 4.27],
        },
        "PARAM_STRUCTURE": {"EM": "KELLY"},
        # Final-state Reggeon couplings c and on/off flags n, by coupling class.
        "COUPLINGS": {
            "PARAM_PI": {"c": [35.00184, 81.63672, 10.86264], "n": [True, False, False]},
            "PARAM_K": {"c": [30.35376, 44.31084, 23.38164], "n": [True, False, False]},
            "PARAM_P": {"c": [27.0, 0.0, 0.0], "n": [True, False, False]},
            "PARAM_RHO": {"c": [25.0, 0.0, 0.0], "n": [True, False, False]},
            "PARAM_PHI": {"c": [18.0, 0.0, 0.0], "n": [True, False, False]},
            "PARAM_X": {"c": [15.0, 0.0, 0.0], "n": [True, False, False]},
        },
    }
}

# Resonances that decay to pseudoscalar pairs, TUNE0 (modeldata/TUNE0/RES_*.json: PARAM_RES
# M, W, J, P, g_Tensor for the tensor pomeron; BW, g_A, g_phi, g_FF and the diagonal of the
# spin density matrix, M = -J..J, for the Regge model), by the generator's names.
RESONANCES = {
    "TUNE0": {
        "f0_500": dict(pdg=9000221, M=0.5, W=0.4, J=0, P=1, g_Tensor=[0.1, 0.0],
                       BW=2, g_A=0.05, g_phi=-3.14159, g_FF=1.0),
        "f0_980": dict(pdg=9010221, M=0.980, W=0.08, J=0, P=1, g_Tensor=[0.4, 2.0],
                       BW=2, g_A=0.065, g_phi=-3.14159, g_FF=1.0),
        "f0_1500": dict(pdg=9030221, M=1.506, W=0.112, J=0, P=1, g_Tensor=[0.1, 0.0],
                        BW=2, g_A=0.03, g_phi=-3.14159, g_FF=1.0),
        "f0_1710": dict(pdg=10331, M=1.704, W=0.123, J=0, P=1, g_Tensor=[0.45, 2.6],
                        BW=2, g_A=0.03, g_phi=-3.14159, g_FF=1.0),
        "f2_1270": dict(pdg=225, M=1.2755, W=0.1867, J=2, P=1,
                        g_Tensor=[2.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0],
                        BW=2, g_A=0.7, g_phi=-1.57, g_FF=1.0, rho=[0.5, 0, 0, 0, 0.5]),
        "f2_1525": dict(pdg=335, M=1.525, W=0.073, J=2, P=1,
                        g_Tensor=[0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0],
                        BW=2, g_A=0.19, g_phi=-1.57, g_FF=1.0, rho=[0.5, 0, 0, 0, 0.5]),
        "f2_1950": dict(pdg=9050225, M=1.936, W=0.464, J=2, P=1,
                        g_Tensor=[1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0],
                        BW=2, g_A=0.1, g_phi=-1.57, g_FF=1.0, rho=[0.5, 0, 0, 0, 0.5]),
    }
}

# Branching ratios of the pseudoscalar-pair decay modes (modeldata/TUNE0/BRANCHING.json),
# by resonance PDG code and unordered daughter pair.
BRANCHING = {
    225: {("pi+", "pi-"): 0.562, ("K+", "K-"): 0.0227},
    335: {("K+", "K-"): 0.4435, ("pi+", "pi-"): 0.00546},
    9050225: {("pi+", "pi-"): 1.0},
    9010221: {("pi+", "pi-"): 0.5, ("K+", "K-"): 0.345},
    9030221: {("pi+", "pi-"): 0.2299, ("K+", "K-"): 0.0425},
    10331: {("K+", "K-"): 0.18, ("pi+", "pi-"): 0.0552},
    9000221: {("pi+", "pi-"): 1.0, ("K+", "K-"): 0.01},
}

# name -> (pdg, mass GeV, width GeV, coupling class)
PARTICLES = {
    "p+": (2212, 9.38272081e-01, 0.0, "PARAM_P"),
    "p-": (-2212, 9.38272081e-01, 0.0, "PARAM_P"),
    "pi+": (211, 1.3957061e-01, 2.5284e-17, "PARAM_PI"),
    "pi-": (-211, 1.3957061e-01, 2.5284e-17, "PARAM_PI"),
    "pi0": (111, 1.349770e-01, 7.73e-09, "PARAM_PI"),
    "K+": (321, 4.93677e-01, 5.317e-17, "PARAM_K"),
    "rho(770)0": (113, 7.7526e-01, 1.491e-01, "PARAM_RHO"),
    "phi(1020)0": (333, 1.019461e+00, 4.249e-03, "PARAM_PHI"),
    "K-": (-321, 4.93677e-01, 5.317e-17, "PARAM_K"),
}

# Spin of the central particles that are not spin 0 (PDG table, J).
SPIN = {"rho(770)0": 1, "phi(1020)0": 1}

# Tensor-pomeron vector-vector coupling pair of each vector meson (PARAM_TENSORPOM key).
VECTOR_COUPLING = {"rho(770)0": "gPrhorho", "phi(1020)0": "gPphiphi"}
