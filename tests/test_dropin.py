"""Drop-in check: a C application (C99, SpFFT's C interface) and a C++ application (C++17,
spfft::Transform / TransformFloat and the exception classes), written the way SpFFT applications
are, compile unchanged against include/spfft/ and link libspfft_gb300 (CPU). On the GPU they run,
and their outputs match the oracle.

The reference's own example programs (examples/example.c and example.cpp of the reference, read
from the reference tree at test time: $SPFFT_REFERENCE_SRC or the staged copy baseline/_ref)
compile unchanged against include/spfft/ and link libspfft_gb300. Unchanged they create
SPFFT_PU_HOST transforms, which this GPU-only library refuses with SPFFT_INVALID_PARAMETER_ERROR
(their exit status); with the processing unit of their grid and transform creation set to
SPFFT_PU_GPU (their data locations stay SPFFT_PU_HOST, host buffers, as a GPU transform accepts)
they run on the GPU and print the oracle's results."""
from __future__ import annotations

import os
import re
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


def _reference_examples() -> Path:
    for cand in (os.environ.get("SPFFT_REFERENCE_SRC"), str(ROOT / "baseline" / "_ref")):
        if cand and (Path(cand) / "examples" / "example.c").exists():
            return Path(cand) / "examples"
    pytest.skip("the reference's examples are not available (SPFFT_REFERENCE_SRC or baseline/_ref)")


def _build_example(src: Path, tmp_path: Path, gpu: bool) -> Path:
    c = src.suffix == ".c"
    compiler = "gcc" if c else "g++"
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    if gpu:
        text = src.read_text()
        # the processing unit of the grid and of the transform (the creation calls only)
        if c:
            text, n1 = re.subn(r"(spfft_grid_create\([^;]*?)SPFFT_PU_HOST", r"\1SPFFT_PU_GPU", text, flags=re.S)
            text, n2 = re.subn(r"(spfft_transform_create\([^;]*?)SPFFT_PU_HOST", r"\1SPFFT_PU_GPU", text, flags=re.S)
        else:
            text, n1 = re.subn(r"(spfft::Grid grid\([^;]*?)SPFFT_PU_HOST", r"\1SPFFT_PU_GPU", text, flags=re.S)
            text, n2 = re.subn(r"(create_transform\(\s*)SPFFT_PU_HOST", r"\1SPFFT_PU_GPU", text, flags=re.S)
        assert n1 == 1 and n2 == 1
        src = tmp_path / ("gpu_" + src.name)
        src.write_text(text)
    libdir = str(sp.library_path().parent)
    exe = tmp_path / (src.stem + ("_c" if c else "_cpp"))
    std = "-std=c99" if c else "-std=c++17"
    res = subprocess.run([compiler, std, "-O2", "-I", str(ROOT / "include"), str(src), "-L", libdir,
                          "-lspfft_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe


def test_reference_examples_compile_unchanged(lib, tmp_path):
    ex = _reference_examples()
    for name in ("example.c", "example.cpp"):
        assert _build_example(ex / name, tmp_path, gpu=False).exists()


def _printed_blocks(stdout: str) -> dict:
    """The numbers the examples print, by section: 'Input', 'After backward transform',
    'After forward transform (without normalization)'."""
    out, key = {}, None
    for line in stdout.splitlines():
        line = line.strip()
        if line.endswith(":") and not line.startswith("Dimensions"):
            key = line[:-1]
            out[key] = []
        elif key and "," in line:
            re_, im_ = line.split(",")
            out[key].append(complex(float(re_), float(im_)))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["example.c", "example.cpp"])
def test_reference_examples_run_on_the_gpu(lib, tmp_path, name):
    ex = _reference_examples()
    unchanged = subprocess.run([str(_build_example(ex / name, tmp_path, gpu=False))], capture_output=True,
                               text=True, timeout=120)
    if name == "example.c":  # the C example exits with the failing call's status
        assert unchanged.returncode == int(sp.ErrorCode.SPFFT_INVALID_PARAMETER_ERROR)
    else:  # the C++ example ends in the uncaught exception
        assert unchanged.returncode != 0
    res = subprocess.run([str(_build_example(ex / name, tmp_path, gpu=True))], capture_output=True, text=True,
                         timeout=120)
    assert res.returncode == 0, res.stderr
    blocks = _printed_blocks(res.stdout)
    # the examples' input: values (i, -i) at every (x, y, z) of a 2^3 grid, x slowest
    idx = np.array([(x, y, z) for x in range(2) for y in range(2) for z in range(2)], dtype=np.int32)
    vals = np.array([complex(i, -i) for i in range(8)])
    assert np.allclose(blocks["Input"], vals)
    oracle = pipeline.HostPipeline(0, 2, 2, 2, idx)
    space = oracle.backward(vals).reshape(-1)
    assert np.allclose(blocks["After backward transform"], space, atol=1e-5)
    fwd = oracle.forward(space.reshape(2, 2, 2))
    assert np.allclose(blocks["After forward transform (without normalization)"], fwd, atol=1e-4)
