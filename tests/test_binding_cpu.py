"""The reference-side binding in INTEGRATION.md (class MContinuumGPU, deriving from the
reference's gra::MContinuum and calling the C ABI) compiles against the reference's own headers
and this library's header: g++ -fsyntax-only, with the stand-in headers of oracle/refbuild/shim
for the libraries missing from the reference's tree. Skipped where the reference's sources are
absent."""
import os
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GRANIITTI_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))


def _binding_source():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    start = text.index("// MContinuumGPU.h")
    return text[start:text.index("```", start)]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "Graniitti")),
                    reason="reference sources not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_reference_binding_compiles():
    src = _binding_source()
    assert "class MContinuumGPU : public gra::MContinuum" in src
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "binding.cc")
        with open(f, "w") as fh:
            fh.write(src + "\nint main() { return 0; }\n")
        inc = ["-I" + os.path.join(REPO, "oracle", "refbuild", "shim"), "-I" + REF,
               "-I" + os.path.join(REF, "include"), "-I" + os.path.join(REF, "libs"),
               "-I" + os.path.join(REF, "libs", "FTensor"),
               "-I" + os.path.join(REF, "libs", "Eigen", "unsupported"),
               "-I" + os.path.join(REPO, "include")]
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only"] + inc + [f],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
