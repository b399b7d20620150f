"""The C-ABI library loads without a GPU and exports every declared entry point."""
import ctypes
import os
import re
import subprocess

from conftest import REPO

HEADER = os.path.join(REPO, "include", "graniitti_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(grn_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ("grn_create", "grn_event_weights", "grn_eikonal_build", "grn_vegas_iteration",
              "grn_vegas_integrate", "grn_unweight", "grn_last_error"):
        assert s in syms


def test_library_exports_all_symbols(lib_built):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_built], capture_output=True,
                         text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_and_signatures(lib_built):
    from graniitti_gb300 import _abi
    lib = _abi.load_library(lib_built)
    for name in _abi.SIGNATURES:
        assert hasattr(lib, name)
    assert b"sm_103a" in lib.grn_version()
    # struct layout agrees with the C compiler's
    from graniitti_gb300._abi import ProcessParams
    P = ProcessParams()
    lib.grn_default_params(ctypes.byref(P))
    assert P.sqrt_s == 13000.0 and P.regge.offshellFF == 2 and P.loop.n_kt == 15
    assert abs(P.fcuts.eta_max - 0.9) < 1e-15 and abs(P.soft.fc2 - 5.0) < 1e-15


def test_create_without_device_fails_cleanly(lib_built):
    """No GPU in this container: grn_create reports GRN_ERR_NO_DEVICE, no crash."""
    try:
        import torch
        if torch.cuda.is_available():
            import pytest
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    from graniitti_gb300 import _abi
    lib = _abi.load_library(lib_built)
    P = _abi.ProcessParams()
    lib.grn_default_params(ctypes.byref(P))
    h = ctypes.c_void_p()
    st = lib.grn_create(ctypes.byref(P), 0, ctypes.byref(h))
    assert st == _abi.GRN_ERR_NO_DEVICE and not h.value
