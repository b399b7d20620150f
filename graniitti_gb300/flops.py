"""Algorithmic FP32 work per kt-loop point, counted by instrumentation
(csrc/flopcount.cc instantiates the device loop arithmetic with a counting scalar)."""
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "flopcount.cc")
EXE = os.path.join(HERE, "_build", "flopcount")


def build():
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    deps = [SRC] + [os.path.join(HERE, "csrc", f) for f in ("grn_physics.cuh", "grn_loop3.cuh")]
    if os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in deps):
        return EXE
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(HERE, "..", "include"),
                           "-I", os.path.join(HERE, "csrc"), SRC, "-o", EXE])
    return EXE


def loop_point_counts():
    out = subprocess.run([build()], capture_output=True, text=True, check=True).stdout
    return json.loads(out)
