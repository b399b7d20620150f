"""Parameters of the weight fixtures: card, process, off-shell form factor, loop grid and
screening table of each tests/golden/*_weights.npz (shared by make_golden.py and the tests)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PROC = "PP[CON]<C> -> pi+ pi-"

# Card, process and off-shell form factor of the weight fixtures that do not store them.
BASE_META = {
    "c1_tune0_weights.npz": ("pp_con_pipi.json", PROC, 2),
    "c1_edge_weights.npz": ("pp_con_pipi.json", PROC, 2),
    "c1_expff_weights.npz": ("pp_con_pipi.json", PROC, 0),
    "c1_orearff_weights.npz": ("pp_con_pipi.json", PROC, 1),
    "c2_screened_63x33_weights.npz": ("pp_con_pipi_screened.json", PROC, None),
    "c2_screened_15x12_weights.npz": ("pp_con_pipi_screened.json", PROC, None),
    "f_tree_weights.npz": ("pp_con_pipi.json", "PP[CON]<F> -> pi+ pi-", None),
    "f_screened_15x12_weights.npz": ("pp_con_pipi_screened.json", "PP[CON]<F> -> pi+ pi-", None),
    "t_tree_weights.npz": ("pp_con_pipi.json", "PP[CONTENSOR]<C> -> pi+ pi-", None),
    "tf_tree_weights.npz": ("pp_con_pipi.json", "PP[CONTENSOR]<F> -> pi+ pi-", None),
    "t_screened_15x12_weights.npz": ("pp_con_pipi_screened.json", "PP[CONTENSOR]<C> -> pi+ pi-",
                                     None),
}


def weight_fixtures():
    return sorted(f for f in os.listdir(HERE) if f.endswith("_weights.npz"))


def fixture_params(name, g):
    """(params, msa): engine/oracle parameters of weight fixture `name` (loaded npz g) and its
    screening table (the reference's 1024 x 10000 tables, or None when unscreened)."""
    from graniitti_gb300 import card
    if "card" in g:
        cname, proc, ff = str(g["card"]), str(g["proc"]), None
    else:
        cname, proc, ff = BASE_META[name]
    P = card.build_params(card.read_card(os.path.join(HERE, "cards", cname)), proc)
    if ff is not None:
        P.regge.offshellFF = ff
    if "loop_kt" in g:
        P.loop.n_kt, P.loop.n_phi = int(g["loop_kt"]), int(g["loop_phi"])
        P.loop.kt_max = float(g["loop_ktmax"])
    msa = None
    if P.screening:
        msa = np.load(os.path.join(HERE, "eikonal_nbt1024_nkt10000.npz"))["msa"]
    return P, msa
