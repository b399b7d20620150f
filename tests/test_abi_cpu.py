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


STRUCTS = ["grn_soft_params", "grn_regge_params", "grn_tensor_params", "grn_resonance",
           "grn_gencuts",
           "grn_fidcuts", "grn_loop_numerics", "grn_process_params", "grn_vegas_params",
           "grn_vegas_result", "grn_flat_params", "grn_flow_params", "grn_flow_train_params",
           "grn_flow_train_result", "grn_tuning", "grn_tune_result"]
MIRROR = {"grn_soft_params": "SoftParams", "grn_regge_params": "ReggeParams",
          "grn_tensor_params": "TensorParams", "grn_resonance": "Resonance",
          "grn_gencuts": "GenCuts", "grn_fidcuts": "FidCuts",
          "grn_loop_numerics": "LoopNumerics", "grn_process_params": "ProcessParams",
          "grn_vegas_params": "VegasParams", "grn_vegas_result": "VegasResult",
          "grn_flat_params": "FlatParams", "grn_flow_params": "FlowParams",
          "grn_flow_train_params": "FlowTrainParams", "grn_flow_train_result": "FlowTrainResult",
          "grn_tuning": "Tuning", "grn_tune_result": "TuneResult"}


def test_ctypes_struct_sizes_match_the_c_compiler(tmp_path):
    """Every struct of the header has the same size in C and in the ctypes mirror."""
    from graniitti_gb300 import _abi
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "graniitti_gb300.h"\nint main(void) {\n' +
                   "".join('  printf("%%s %%zu\\n", "%s", sizeof(%s));\n' % (n, n) for n in STRUCTS) +
                   "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        name, size = line.split()
        assert ctypes.sizeof(getattr(_abi, MIRROR[name])) == int(size), name
