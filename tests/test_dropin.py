"""Drop-in check: a C application (C99, SpFFT's C interface) and a C++ application (C++17,
spfft::Transform / TransformFloat and the exception classes), written the way SpFFT applications
are, compile unchanged against include/spfft/ and link libspfft_gb300 (CPU). On the GPU they run,
and their outputs match the oracle."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import rel_l2

ROOT = Path(__file__).resolve().parents[1]
SRC = Path(__file__).resolve().parent / "dropin"


def _build(tmp_path: Path, lib) -> dict:
    libdir = str(sp.library_path().parent)
    out = {}
    for name, compiler, std in (("app_c.c", "gcc", "-std=c99"), ("app_cpp.cpp", "g++", "-std=c++17")):
        if shutil.which(compiler) is None:
            pytest.skip(f"{compiler} not available")
        exe = tmp_path / Path(name).stem
        subprocess.run([compiler, std, "-O2", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(SRC / name),
                        "-L", libdir, "-lspfft_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       check=True, capture_output=True, text=True)
        out[name] = exe
    return out


def test_applications_compile_and_link(lib, tmp_path):
    exes = _build(tmp_path, lib)
    assert all(e.exists() for e in exes.values())


def _load(prefix: Path, ttype: int, n: int, single: bool):
    idx = np.fromfile(f"{prefix}_indices.bin", dtype=np.int32).reshape(-1, 3)
    v = np.fromfile(f"{prefix}_values.bin", dtype=np.float64)
    s = np.fromfile(f"{prefix}_space.bin", dtype=np.float64)
    f = np.fromfile(f"{prefix}_forward.bin", dtype=np.float64)
    values = v[0::2] + 1j * v[1::2]
    space = (s[0::2] + 1j * s[1::2]) if ttype == 0 else s
    return idx, values, space.reshape(n, n, n), f[0::2] + 1j * f[1::2]


@pytest.mark.gpu
@pytest.mark.parametrize("app,ttype,n,radius,precision", [
    ("app_c.c", 0, 16, 5, 64), ("app_c.c", 1, 24, 7, 64),
    ("app_cpp.cpp", 0, 32, 8, 64), ("app_cpp.cpp", 1, 48, 12, 64), ("app_cpp.cpp", 1, 48, 12, 32)])
def test_applications_run_against_the_oracle(lib, tmp_path, app, ttype, n, radius, precision):
    exe = _build(tmp_path, lib)[app]
    prefix = tmp_path / "out"
    args = [str(exe), str(ttype), str(n), str(radius)]
    if app == "app_cpp.cpp":
        args.append(str(precision))
    res = subprocess.run(args + [str(prefix)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    idx, values, space, forward = _load(prefix, ttype, n, precision == 32)
    oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
    tol = 1e-12 if precision == 64 else 1e-5
    assert rel_l2(space, oracle.backward(values)) <= tol
    assert rel_l2(forward, oracle.forward(space)) <= tol
