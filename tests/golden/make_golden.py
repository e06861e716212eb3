"""Generates the committed golden fixtures of this directory from the reference's OWN code.

Requires oracle/_ref/ref_indices (built by `make -C oracle`, which compiles the reference's
src/parameters/parameters.cpp and its tests/test_util/generate_indices.hpp from the reference
sources). Run from the repository root:  python tests/golden/make_golden.py

ref_cases.npz   For every size combination of the reference's local test suite whose dims are all
                in {1, 2, 11, 12, 13} (tests/local_tests/test_local_transform.cpp:95-111), C2C and
                R2C, plain and centered: the index triplets the reference's generator produces
                (std::mt19937(42), create_value_indices / center_indices) and the reference
                planner's output for them (value indices, stick keys, zero-zero stick).
ref_edges.npz   Hand-made planner edge cases (bounds, centered switch, R2C x range, too many values,
                empty input) with the reference planner's output or error code.
dense_small.npz A few small transforms (inputs and unnormalised dense DFT outputs, numpy) used to
                pin the floating-point results independently of the oracle pipeline code.
ref_pipeline.npz The reference's OWN host transform path (oracle/_ref/libref_pipeline.so: its
                execution_host.cpp and everything it calls, with FFTW replaced by the project's
                FFTW-API shim) run on the inputs of its local test suite, FP64: C2C backward then
                forward of the generated values; R2C forward then backward of the real space
                domain the suite builds (a uniform(0,1) draw at each index position), as in
                tests/test_util/test_transform.hpp:153-276.
"""
from __future__ import annotations

import itertools
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import dense, ref  # noqa: E402

OUT = Path(__file__).resolve().parent


def ref_cases() -> None:
    arrays = {}
    keys = []
    small = (1, 2, 11, 12, 13)
    for r2c, centered in itertools.product((False, True), (False, True)):
        dims = (1, 2, 11) if centered else small
        for dx, dy, dz in itertools.product(dims, dims, dims):
            case = ref.test_case(dx, dy, dz, r2c, centered)
            idx = case["indices"]
            plan = ref.plan(int(r2c), dx, dy, dz, idx)
            key = f"{'r2c' if r2c else 'c2c'}_{'cen' if centered else 'pos'}_{dx}_{dy}_{dz}"
            keys.append(key)
            arrays[key + "/indices"] = idx.astype(np.int8)
            arrays[key + "/value_indices"] = plan["value_indices"].astype(np.int16)
            arrays[key + "/stick_keys"] = plan["stick_keys"].astype(np.int16)
            arrays[key + "/zz"] = np.array([plan["zero_zero_stick"]], dtype=np.int32)
    arrays["keys"] = np.array(keys)
    np.savez_compressed(OUT / "ref_cases.npz", **arrays)


EDGES = [
    # (name, type, dx, dy, dz, triplets)
    ("mixed_sign_probe", 0, 4, 4, 4, [0, 0, 0, 1, 0, -1, -1, 2, -1, 1, 0, 2]),
    ("plain_max", 0, 5, 4, 3, [4, 3, 2, 0, 0, 0]),
    ("plain_over", 0, 5, 4, 3, [5, 0, 0]),
    ("centered_bounds", 0, 5, 4, 3, [-2, -1, -1, 2, 2, 1]),
    ("centered_over", 0, 5, 4, 3, [-2, -1, -1, 3, 0, 0]),
    ("centered_under", 0, 5, 4, 3, [-3, 0, 0, 0, 0, -1]),
    ("r2c_x_max", 1, 6, 4, 4, [3, 3, 3, 0, 1, 2]),
    ("r2c_x_over", 1, 6, 4, 4, [4, 0, 0]),
    ("r2c_x_negative", 1, 6, 4, 4, [-1, 0, 0]),
    ("r2c_centered_yz", 1, 6, 4, 4, [0, -1, -1, 3, 2, 2, 1, -2, 0]),
    ("too_many", 0, 1, 1, 2, [0, 0, 0, 0, 0, 1, 0, 0, 0]),
    ("duplicates", 0, 3, 3, 3, [1, 1, 1, 1, 1, 1, 2, 2, 2]),
    ("empty", 0, 3, 3, 3, []),
    ("zz_absent", 1, 4, 4, 4, [1, 0, 0, 2, 3, 1]),
    ("zz_middle_keys", 0, 4, 4, 4, [-1, -1, 0, 0, 0, 1, 1, 1, 1]),
    ("dims_one", 0, 1, 1, 1, [0, 0, 0]),
]


def ref_edges() -> None:
    arrays = {}
    names = []
    for name, t, dx, dy, dz, trip in EDGES:
        trip = np.array(trip, dtype=np.int64)
        res = ref.plan(t, dx, dy, dz, trip)
        names.append(name)
        arrays[name + "/args"] = np.array([t, dx, dy, dz], dtype=np.int32)
        arrays[name + "/indices"] = trip.astype(np.int32)
        if "error" in res:
            arrays[name + "/error"] = np.array([res["error"]], dtype=np.int32)
        else:
            arrays[name + "/value_indices"] = res["value_indices"].astype(np.int32)
            arrays[name + "/stick_keys"] = res["stick_keys"].astype(np.int32)
            arrays[name + "/zz"] = np.array([res["zero_zero_stick"]], dtype=np.int32)
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT / "ref_edges.npz", **arrays)


def dense_small() -> None:
    rng = np.random.default_rng(20241203)
    arrays = {}
    names = []
    for name, t, (dx, dy, dz) in [("c2c_5_6_7", 0, (5, 6, 7)), ("c2c_12_11_13", 0, (12, 11, 13)),
                                 ("r2c_8_6_5", 1, (8, 6, 5)), ("r2c_11_12_13", 1, (11, 12, 13))]:
        case = ref.test_case(dx, dy, dz, t == 1, True)
        idx = case["indices"]
        if t == 0:
            vals = rng.uniform(-1, 1, idx.size // 3) + 1j * rng.uniform(-1, 1, idx.size // 3)
            space = dense.backward(t, dx, dy, dz, idx, vals)
        else:
            space = rng.uniform(-1, 1, (dz, dy, dx))
            vals = dense.forward(t, dx, dy, dz, idx, space)
            space = space * (dx * dy * dz)  # backward(forward(f)) = N f
        fwd_in = space if t == 0 else space / (dx * dy * dz)
        names.append(name)
        arrays[name + "/args"] = np.array([t, dx, dy, dz], dtype=np.int32)
        arrays[name + "/indices"] = idx.astype(np.int32)
        arrays[name + "/values"] = vals
        arrays[name + "/space"] = space  # backward(values)
        arrays[name + "/forward_in"] = fwd_in
        arrays[name + "/forward_out"] = dense.forward(t, dx, dy, dz, idx, fwd_in)
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT / "dense_small.npz", **arrays)


def r2c_space_of_test(dx: int, dy: int, dz: int, idx: np.ndarray, re: np.ndarray) -> np.ndarray:
    """The real space domain the reference's R2C test builds: the value drawn for triplet i sits at
    the triplet's own (storage) position (test_transform.hpp:232-237, 257-263)."""
    t = idx.reshape(-1, 3)
    space = np.zeros((dz, dy, dx))
    space[t[:, 2] % dz, t[:, 1] % dy, t[:, 0] % dx] = re
    return space


PIPELINE_CASES = [(11, 12, 13), (13, 11, 12), (12, 12, 12), (2, 11, 13), (13, 1, 12), (11, 2, 1),
                  (1, 1, 1), (12, 13, 2)]


def ref_pipeline() -> None:
    arrays = {}
    names = []
    for r2c, centered in itertools.product((False, True), (False, True)):
        for dx, dy, dz in PIPELINE_CASES:
            case = ref.test_case(dx, dy, dz, r2c, centered)
            idx = case["indices"].astype(np.int32)
            if idx.size == 0:
                continue
            name = f"{'r2c' if r2c else 'c2c'}_{'cen' if centered else 'pos'}_{dx}_{dy}_{dz}"
            arrays[name + "/args"] = np.array([int(r2c), dx, dy, dz], dtype=np.int32)
            arrays[name + "/indices"] = idx.astype(np.int8)
            if r2c:
                space_in = r2c_space_of_test(dx, dy, dz, idx, case["values"].real)
                space, values = ref.pipeline_run(1, dx, dy, dz, idx, space=space_in)
                arrays[name + "/space_in"] = space_in
            else:
                space, values = ref.pipeline_run(0, dx, dy, dz, idx, values=case["values"])
                arrays[name + "/values_in"] = case["values"]
            arrays[name + "/space_out"] = space
            arrays[name + "/values_out"] = values
            names.append(name)
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT / "ref_pipeline.npz", **arrays)


if __name__ == "__main__":
    if not ref.available():
        sys.exit("oracle/_ref/ref_indices missing: run `make -C oracle` where the reference exists")
    ref_cases()
    ref_edges()
    dense_small()
    if ref.pipeline_available():
        ref_pipeline()
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)
