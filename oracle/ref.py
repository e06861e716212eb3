"""Runs the reference's own code built by oracle/Makefile: ``_ref/ref_indices`` (its index planner
and test-input generator) and ``_ref/libref_pipeline.so`` (its host transform path, with FFTW
replaced by the project's FFTW-API shim). Test infrastructure only; available only where the
reference sources were present at build time."""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
EXE = HERE / "_ref" / "ref_indices"
LIB = HERE / "_ref" / "libref_pipeline.so"
_lib = None


def available() -> bool:
    return EXE.exists()


def plan(transform_type: int, dx: int, dy: int, dz: int, triplets) -> dict:
    t = np.asarray(triplets, dtype=np.int64).reshape(-1)
    n = t.size // 3
    res = subprocess.run([str(EXE), "plan", str(transform_type), str(dx), str(dy), str(dz), str(n)],
                         input=" ".join(map(str, t.tolist())), capture_output=True, text=True, check=True)
    out = {}
    for line in res.stdout.splitlines():
        tag, *vals = line.split()
        out[tag] = [int(v) for v in vals]
    if "error" in out:
        return {"error": out["error"][0]}
    return {"value_indices": np.array(out.get("values", []), dtype=np.int64),
            "stick_keys": np.array(out.get("sticks", []), dtype=np.int64),
            "zero_zero_stick": out["zz"][0]}


def test_case(dx: int, dy: int, dz: int, r2c: bool, centered: bool) -> dict:
    """Index set and values of the reference's local transform test for these dims."""
    res = subprocess.run([str(EXE), "gen", str(dx), str(dy), str(dz), str(int(r2c)), str(int(centered))],
                         capture_output=True, text=True, check=True)
    out = {}
    for line in res.stdout.splitlines():
        tag, *vals = line.split()
        out[tag] = vals
    idx = np.array([int(v) for v in out.get("indices", [])], dtype=np.int64)
    re = np.array([float(v) for v in out.get("re", [])])
    im = np.array([float(v) for v in out.get("im", [])])
    return {"indices": idx, "values": re + 1j * im}


def pipeline_available() -> bool:
    return LIB.exists()


def pipeline_run(transform_type: int, dx: int, dy: int, dz: int, triplets, values=None, space=None,
                 precision: str = "float64", scaling: int = 0, threads: int = 1):
    """The reference's host transform path (spfft::Transform or TransformFloat on SPFFT_PU_HOST,
    external space buffer). Given `values`: backward, then forward of the result with `scaling`.
    Given `space` instead: forward with `scaling`, then backward of the result (the order of the
    reference's R2C tests). Returns (space [dz, dy, dx] complex or real, values) after both steps;
    raises RuntimeError with the reference's SpfftError code on failure."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(LIB))
        _lib.ref_pipeline_run.argtypes = ([ctypes.c_int] * 6 + [ctypes.c_void_p, ctypes.c_int] +
                                          [ctypes.c_void_p] * 4 + [ctypes.c_int] * 2)
        _lib.ref_pipeline_run.restype = ctypes.c_int
    idx = np.ascontiguousarray(np.asarray(triplets, dtype=np.int32).reshape(-1))
    n = idx.size // 3
    c2c = transform_type == 0
    ns = dz * dy * dx
    forward_first = space is not None
    vin = np.zeros(2 * max(n, 1))
    sin = np.zeros(ns * (2 if c2c else 1))
    if forward_first:
        s = np.asarray(space).reshape(-1)
        if c2c:
            sin = np.ascontiguousarray(np.stack([s.real, s.imag], axis=1).reshape(-1).astype(np.float64))
        else:
            sin = np.ascontiguousarray(s.astype(np.float64))
    elif n:
        v = np.asarray(values, dtype=np.complex128).reshape(-1)
        vin = np.ascontiguousarray(np.stack([v.real, v.imag], axis=1).reshape(-1))
    sout = np.zeros_like(sin)
    vout = np.zeros(2 * max(n, 1))
    rc = _lib.ref_pipeline_run(0 if precision == "float64" else 1, transform_type, dx, dy, dz, n,
                               idx.ctypes.data if n else None, int(forward_first), vin.ctypes.data,
                               sin.ctypes.data, vout.ctypes.data, sout.ctypes.data, scaling, threads)
    if rc != 0:
        raise RuntimeError(f"reference pipeline error {rc}")
    if c2c:
        sout = (sout[0::2] + 1j * sout[1::2]).reshape(dz, dy, dx)
    else:
        sout = sout.reshape(dz, dy, dx)
    return sout, (vout[0::2] + 1j * vout[1::2])[:n]
