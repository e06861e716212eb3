"""Runs ``_ref/ref_indices`` (the reference's own index code, built by oracle/Makefile).
Test infrastructure only; available only where the reference sources were present at build time."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
EXE = HERE / "_ref" / "ref_indices"


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
