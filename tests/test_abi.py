"""The C-ABI library loads and exports every function its public headers declare (CPU only)."""
import re
import subprocess
from pathlib import Path

import spfft_gb300 as sp

INCLUDE = Path(__file__).resolve().parents[1] / "include" / "spfft"


def declared_c_functions() -> set:
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"SPFFT_EXPORT\s+SpfftError\s+(\w+)\s*\(", text))
    return names


def exported_symbols() -> set:
    out = subprocess.run(["nm", "-D", "--defined-only", str(sp.library_path())], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_every_declared_function_is_exported(lib):
    declared = declared_c_functions()
    assert len(declared) >= 79
    missing = declared - exported_symbols()
    assert not missing, sorted(missing)


def test_reference_c_api_surface_is_complete(lib):
    # Every non-MPI C function of the reference interface (include/spfft/{grid,transform,
    # multi_transform}{,_float}.h) must be present.
    base = ["create", "destroy", "max_dim_x", "max_dim_y", "max_dim_z", "max_num_local_z_columns",
            "max_local_z_length", "processing_unit", "device_id", "num_threads"]
    tr = ["create", "create_independent", "destroy", "clone", "forward", "forward_ptr", "backward",
          "backward_ptr", "get_space_domain", "dim_x", "dim_y", "dim_z", "local_z_length",
          "local_slice_size", "local_z_offset", "global_size", "num_local_elements",
          "num_global_elements", "device_id", "num_threads", "execution_mode", "set_execution_mode"]
    multi = ["forward", "forward_ptr", "backward", "backward_ptr"]
    want = set()
    for p in ("spfft_", "spfft_float_"):
        want |= {p + "grid_" + b for b in base}
        want |= {p + "transform_" + t for t in tr}
        want |= {p + "multi_transform_" + m for m in multi}
    assert not (want - exported_symbols())


def test_cpp_classes_are_exported(lib):
    out = subprocess.run(["nm", "-DC", "--defined-only", str(sp.library_path())], capture_output=True,
                         text=True, check=True).stdout
    for sym in ["spfft::Grid::Grid(int, int, int, int, SpfftProcessingUnitType, int)",
                "spfft::Transform::backward(double const*, double*)",
                "spfft::TransformFloat::forward(float const*, float*, SpfftScalingType)",
                "spfft::multi_transform_backward(int, spfft::Transform*, double const* const*, double* const*)"]:
        assert sym in out, sym


HANDLE_TYPES = ("SpfftGrid", "SpfftFloatGrid", "SpfftTransform", "SpfftFloatTransform", "SpfftGb300Batch")


def handle_functions() -> list:
    """(name, [parameter declarations]) of every declared C function whose first parameter is a
    grid, transform or batch handle passed by value."""
    out = []
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for name, params in re.findall(r"SPFFT_EXPORT\s+SpfftError\s+(\w+)\s*\(([^)]*)\)", text):
            ps = [p.strip() for p in params.split(",") if p.strip()]
            if ps and ps[0].split()[0] in HANDLE_TYPES and "*" not in ps[0]:
                out.append((name, ps))
    return out


def test_null_handle_is_rejected_by_every_handle_function(lib):
    """Every C function taking a handle returns SPFFT_INVALID_HANDLE_ERROR for a null handle
    (transform.cpp:245-258 of the reference), before touching its other arguments, which here
    point at a zeroed buffer."""
    import ctypes

    scratch = (ctypes.c_char * 4096)()
    fns = handle_functions()
    assert len(fns) >= 60, len(fns)
    wrong = {}
    for name, params in fns:
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p if "*" in p else ctypes.c_int for p in params[1:]]
        fn.restype = ctypes.c_int
        # other pointers valid or null, other integers 0 or 1: the handle is checked first
        for ptr, num in ((ctypes.cast(scratch, ctypes.c_void_p), 0), (None, 1)):
            code = fn(None, *[ptr if "*" in p else num for p in params[1:]])
            if code != sp.ErrorCode.SPFFT_INVALID_HANDLE_ERROR:
                wrong[name] = code
    assert not wrong, wrong
