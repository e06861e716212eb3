"""Python binding of the GB300 SpFFT library.

The product is the C-ABI shared library ``libspfft_gb300.so`` (C interface identical to the
reference's ``include/spfft/*.h``). This module binds it with ctypes and mirrors the reference's
C++ classes (``spfft::Grid``, ``spfft::Transform``; include/spfft/grid.hpp, transform.hpp) with the
same method names, argument meaning and error behaviour: every failing call raises ``SpfftError``
carrying the C error code.

Buffers may be given as torch tensors (host or CUDA), numpy arrays, or raw integer addresses.
There is no CPU fallback: if the native library is missing, importing the library object fails.
"""
from __future__ import annotations

import ctypes
import enum
import os
from pathlib import Path
from typing import Any

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libspfft_gb300.so"

# ---- enums (values fixed by the reference ABI, include/spfft/types.h, errors.h) ----------------
SPFFT_PU_HOST = 1
SPFFT_PU_GPU = 2
SPFFT_INDEX_TRIPLETS = 0
SPFFT_TRANS_C2C = 0
SPFFT_TRANS_R2C = 1
SPFFT_NO_SCALING = 0
SPFFT_FULL_SCALING = 1
SPFFT_EXEC_SYNCHRONOUS = 0
SPFFT_EXEC_ASYNCHRONOUS = 1


class ErrorCode(enum.IntEnum):
    SPFFT_SUCCESS = 0
    SPFFT_UNKNOWN_ERROR = 1
    SPFFT_INVALID_HANDLE_ERROR = 2
    SPFFT_OVERFLOW_ERROR = 3
    SPFFT_ALLOCATION_ERROR = 4
    SPFFT_INVALID_PARAMETER_ERROR = 5
    SPFFT_DUPLICATE_INDICES_ERROR = 6
    SPFFT_INVALID_INDICES_ERROR = 7
    SPFFT_MPI_SUPPORT_ERROR = 8
    SPFFT_MPI_ERROR = 9
    SPFFT_MPI_PARAMETER_MISMATCH_ERROR = 10
    SPFFT_HOST_EXECUTION_ERROR = 11
    SPFFT_FFTW_ERROR = 12
    SPFFT_GPU_ERROR = 13
    SPFFT_GPU_PRECEDING_ERROR = 14
    SPFFT_GPU_SUPPORT_ERROR = 15
    SPFFT_GPU_ALLOCATION_ERROR = 16
    SPFFT_GPU_LAUNCH_ERROR = 17
    SPFFT_GPU_NO_DEVICE_ERROR = 18
    SPFFT_GPU_INVALID_VALUE_ERROR = 19
    SPFFT_GPU_INVALID_DEVICE_PTR_ERROR = 20
    SPFFT_GPU_COPY_ERROR = 21
    SPFFT_GPU_FFT_ERROR = 22


class SpfftError(RuntimeError):
    """A C call returned a code other than SPFFT_SUCCESS."""

    def __init__(self, code: int, func: str):
        self.code = ErrorCode(code)
        super().__init__(f"{func} failed: {self.code.name}")

    def error_code(self) -> int:
        return int(self.code)


_lib: ctypes.CDLL | None = None


def library_path() -> Path:
    return LIB_PATH


def load_library() -> ctypes.CDLL:
    """Load the native library (built by ``spfft_gb300.build.build()``). Fails loudly if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"native library {LIB_PATH} is missing; build it with "
            "`python -c 'import spfft_gb300.build as b; b.build()'`")
    lib = ctypes.CDLL(str(LIB_PATH))
    _declare(lib)
    _lib = lib
    return lib


_vp = ctypes.c_void_p
_i = ctypes.c_int
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)


def _declare(lib: ctypes.CDLL) -> None:
    for prefix in ("spfft_", "spfft_float_"):
        g = prefix + "grid_"
        getattr(lib, g + "create").argtypes = [ctypes.POINTER(_vp), _i, _i, _i, _i, _i, _i]
        getattr(lib, g + "destroy").argtypes = [_vp]
        for name in ("max_dim_x", "max_dim_y", "max_dim_z", "max_num_local_z_columns",
                     "max_local_z_length", "processing_unit", "device_id", "num_threads"):
            getattr(lib, g + name).argtypes = [_vp, _ip]
        t = prefix + "transform_"
        getattr(lib, t + "create").argtypes = [ctypes.POINTER(_vp), _vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp]
        getattr(lib, t + "create_independent").argtypes = [ctypes.POINTER(_vp), _i, _i, _i, _i, _i, _i, _i, _i, _vp]
        getattr(lib, t + "destroy").argtypes = [_vp]
        getattr(lib, t + "clone").argtypes = [_vp, ctypes.POINTER(_vp)]
        getattr(lib, t + "forward").argtypes = [_vp, _i, _vp, _i]
        getattr(lib, t + "forward_ptr").argtypes = [_vp, _vp, _vp, _i]
        getattr(lib, t + "backward").argtypes = [_vp, _vp, _i]
        getattr(lib, t + "backward_ptr").argtypes = [_vp, _vp, _vp]
        getattr(lib, t + "get_space_domain").argtypes = [_vp, _i, ctypes.POINTER(_vp)]
        for name in ("dim_x", "dim_y", "dim_z", "local_z_length", "local_slice_size", "local_z_offset",
                     "num_local_elements", "device_id", "num_threads", "execution_mode"):
            getattr(lib, t + name).argtypes = [_vp, _ip]
        for name in ("global_size", "num_global_elements"):
            getattr(lib, t + name).argtypes = [_vp, _llp]
        getattr(lib, t + "set_execution_mode").argtypes = [_vp, _i]
        m = prefix + "multi_transform_"
        getattr(lib, m + "forward").argtypes = [_i, ctypes.POINTER(_vp), _ip, ctypes.POINTER(_vp), _ip]
        getattr(lib, m + "forward_ptr").argtypes = [_i, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ip]
        getattr(lib, m + "backward").argtypes = [_i, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _ip]
        getattr(lib, m + "backward_ptr").argtypes = [_i, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]
    for prefix in ("spfft_gb300_", "spfft_gb300_float_"):
        getattr(lib, prefix + "transform_set_stream").argtypes = [_vp, _vp]
        getattr(lib, prefix + "transform_backward_device").argtypes = [_vp, _vp, _vp, _vp]
        getattr(lib, prefix + "transform_forward_device").argtypes = [_vp, _vp, _vp, _i, _vp]
        getattr(lib, prefix + "transform_path_info").argtypes = [_vp, _ip]
        getattr(lib, prefix + "transform_autotune").argtypes = [_vp, _i, ctypes.POINTER(ctypes.c_float)]
        getattr(lib, prefix + "transform_tuning").argtypes = [_vp, _ip]
        getattr(lib, prefix + "transform_x_backward_rows").argtypes = [_vp, _ip]
        getattr(lib, prefix + "transform_splits").argtypes = [_vp, _ip]
        getattr(lib, prefix + "transform_split_stages").argtypes = [_vp, _ip]
        getattr(lib, prefix + "transform_radix_plans").argtypes = [_vp, _ip, _ip]
        getattr(lib, prefix + "transform_adjoint_backward").argtypes = [_vp, _vp, _vp, _vp]
        getattr(lib, prefix + "transform_adjoint_forward").argtypes = [_vp, _vp, _vp, _i, _vp]
        getattr(lib, prefix + "transform_stage_times").argtypes = [_vp, _i, _vp, _vp, _i, _vp,
                                                                   ctypes.POINTER(ctypes.c_float)]
    lib.spfft_gb300_plan_indices.argtypes = [_i, _i, _i, _i, _i, _vp, _vp, _vp, _i, _ip, _ip]
    lib.spfft_gb300_plan_tables.argtypes = [_i, _i, _i, _i, _i, _i, _vp, _vp, ctypes.c_longlong,
                                            ctypes.POINTER(ctypes.c_longlong), _ip]
    lib.spfft_gb300_plan_cache_size.argtypes = [_ip]
    lib.spfft_gb300_inject_allocation_failure.argtypes = [_i, _ip]
    lib.spfft_gb300_batch_create.argtypes = [ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp)]
    lib.spfft_gb300_float_batch_create.argtypes = [ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp)]
    lib.spfft_gb300_batch_destroy.argtypes = [_vp]
    lib.spfft_gb300_batch_bind.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]
    lib.spfft_gb300_batch_backward.argtypes = [_vp, _vp]
    lib.spfft_gb300_batch_forward.argtypes = [_vp, _i, _vp]
    lib.spfft_gb300_batch_pair_graph.argtypes = [_vp, _i, _vp]
    lib.spfft_gb300_batch_info.argtypes = [_vp, _ip, _ip, _ip]
    lib.spfft_gb300_batch_transform_path.argtypes = [_vp, _i, _ip]
    lib.spfft_gb300_batch_row_groups.argtypes = [_vp, _i, _ip]
    lib.spfft_gb300_batch_autotune.argtypes = [_vp, _i, _vp, ctypes.POINTER(ctypes.c_float)]
    lib.spfft_gb300_multi_batched_calls.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
    lib.spfft_gb300_batch_stage_times.argtypes = [_vp, _i, _i, _vp, ctypes.POINTER(ctypes.c_float)]
    lib.spfft_gb300_transform_backward_noalloc.argtypes = [_vp, _vp, _vp, _vp]


def _check(code: int, func: str) -> None:
    if code != 0:
        raise SpfftError(code, func)


def _call(name: str, *args) -> None:
    lib = load_library()
    _check(getattr(lib, name)(*args), name)


def address(buf: Any) -> int | None:
    """Raw address of a torch tensor, numpy array, ctypes object or int (None stays None)."""
    if buf is None:
        return None
    if isinstance(buf, int):
        return buf
    if hasattr(buf, "data_ptr"):
        return int(buf.data_ptr())
    if hasattr(buf, "__array_interface__"):
        return int(buf.__array_interface__["data"][0])
    if isinstance(buf, ctypes.Array) or isinstance(buf, ctypes._SimpleCData):
        return ctypes.addressof(buf)
    raise TypeError(f"cannot take the address of {type(buf)!r}")


def _indices_arg(indices: Any) -> tuple[Any, int]:
    """Keep a contiguous int32 copy alive and return (owner, address)."""
    import numpy as np

    if indices is None:
        return None, 0
    if hasattr(indices, "detach"):
        indices = indices.detach().cpu().numpy()
    arr = np.ascontiguousarray(np.asarray(indices, dtype=np.int32).reshape(-1))
    return arr, int(arr.ctypes.data) if arr.size else 0


# ---- index planning without a GPU -------------------------------------------------------------

def plan_indices(transform_type: int, dim_x: int, dim_y: int, dim_z: int, indices: Any):
    """Host-only planner: (value_indices, stick_keys, zero_zero_stick) exactly as the transform
    uses them. Raises SpfftError like transform creation would."""
    import numpy as np

    owner, ptr = _indices_arg(indices)
    n = 0 if owner is None else owner.size // 3
    values = np.zeros(max(n, 1), dtype=np.int32)
    sticks = np.zeros(max(n, 1), dtype=np.int32)
    ns = ctypes.c_int(0)
    zz = ctypes.c_int(0)
    _call("spfft_gb300_plan_indices", transform_type, dim_x, dim_y, dim_z, n, ptr or None,
          int(values.ctypes.data), int(sticks.ctypes.data), int(sticks.size), ctypes.byref(ns),
          ctypes.byref(zz))
    return values[:n].copy(), sticks[: ns.value].copy(), zz.value


PLAN_TABLE_FIELDS = ("value_indices", "stick_keys", "stick_column", "stick_y", "stick_plane_pos",
                     "column_x", "column_stick_start", "entry_pos", "entry_user", "stick_entry_start",
                     "hermitian_weight")


def plan_tables(planner: int, transform_type: int, dim_x: int, dim_y: int, dim_z: int,
                indices: Any) -> dict:
    """Every table of the index plan from the host planner (0) or the device planner on the
    current device (1): a dict of int32 arrays named by PLAN_TABLE_FIELDS plus the scalars
    num_sticks, num_columns, zero_zero_stick, identity_order and used_device (0 where the device
    planner declined and the host planner ran)."""
    import numpy as np

    owner, ptr = _indices_arg(indices)
    n = 0 if owner is None else owner.size // 3
    size = ctypes.c_longlong(0)
    used = ctypes.c_int(0)
    args = (planner, transform_type, dim_x, dim_y, dim_z, n, ptr or None)
    _call("spfft_gb300_plan_tables", *args, None, 0, ctypes.byref(size), ctypes.byref(used))
    buf = np.zeros(max(size.value, 1), dtype=np.int32)
    _call("spfft_gb300_plan_tables", *args, int(buf.ctypes.data), int(buf.size), ctypes.byref(size),
          ctypes.byref(used))
    ns, nc, zz, ident = (int(v) for v in buf[:4])
    lengths = (n, ns, ns, ns, ns, nc, nc + 1, n, n, ns + 1, n if transform_type == SPFFT_TRANS_R2C else 0)
    out: dict = {"num_sticks": ns, "num_columns": nc, "zero_zero_stick": zz, "identity_order": ident,
                 "used_device": used.value}
    pos = 4
    for name, length in zip(PLAN_TABLE_FIELDS, lengths):
        out[name] = buf[pos:pos + length].copy()
        pos += length
    return out


def inject_allocation_failure(after_allocations: int) -> int:
    """Test hook: the allocation after `after_allocations` more successful ones fails once (-1 turns
    it off). Returns the previous countdown (-1 once an injected failure has fired)."""
    v = ctypes.c_int(0)
    _call("spfft_gb300_inject_allocation_failure", int(after_allocations), ctypes.byref(v))
    return v.value


def plan_cache_size() -> int:
    """Live index plans that transform creation can share."""
    v = ctypes.c_int(0)
    _call("spfft_gb300_plan_cache_size", ctypes.byref(v))
    return v.value


# ---- handles ------------------------------------------------------------------------------------

def _prefix(dtype: str) -> str:
    if dtype in ("float64", "double", "f64"):
        return "spfft_"
    if dtype in ("float32", "float", "f32"):
        return "spfft_float_"
    raise ValueError(f"unsupported dtype {dtype!r}")


class Grid:
    """Memory pool for transforms up to the given size (reference spfft::Grid)."""

    def __init__(self, max_dim_x: int, max_dim_y: int, max_dim_z: int, max_num_local_z_columns: int,
                 processing_unit: int = SPFFT_PU_GPU, max_num_threads: int = -1,
                 dtype: str = "float64"):
        self.dtype = dtype
        self._p = _prefix(dtype)
        h = _vp()
        _call(self._p + "grid_create", ctypes.byref(h), max_dim_x, max_dim_y, max_dim_z,
              max_num_local_z_columns, processing_unit, max_num_threads)
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            getattr(_lib, self._p + "grid_destroy")(h)
            self._h = None

    def _get(self, name: str) -> int:
        v = ctypes.c_int(0)
        _call(self._p + "grid_" + name, self._h, ctypes.byref(v))
        return v.value

    def max_dim_x(self) -> int: return self._get("max_dim_x")
    def max_dim_y(self) -> int: return self._get("max_dim_y")
    def max_dim_z(self) -> int: return self._get("max_dim_z")
    def max_num_local_z_columns(self) -> int: return self._get("max_num_local_z_columns")
    def max_local_z_length(self) -> int: return self._get("max_local_z_length")
    def processing_unit(self) -> int: return self._get("processing_unit")
    def device_id(self) -> int: return self._get("device_id")
    def num_threads(self) -> int: return self._get("num_threads")

    def create_transform(self, processing_unit: int, transform_type: int, dim_x: int, dim_y: int,
                         dim_z: int, local_z_length: int, num_local_elements: int,
                         index_format: int, indices: Any) -> "Transform":
        owner, ptr = _indices_arg(indices)
        h = _vp()
        _call(self._p + "transform_create", ctypes.byref(h), self._h, processing_unit, transform_type,
              dim_x, dim_y, dim_z, local_z_length, num_local_elements, index_format, ptr or None)
        return Transform._wrap(h, self.dtype, transform_type, keep=(self,))


class Transform:
    """Sparse 3D FFT plan on one GPU (reference spfft::Transform)."""

    def __init__(self, max_num_threads: int, processing_unit: int, transform_type: int, dim_x: int,
                 dim_y: int, dim_z: int, num_local_elements: int, index_format: int, indices: Any,
                 dtype: str = "float64"):
        owner, ptr = _indices_arg(indices)
        self.dtype = dtype
        self._p = _prefix(dtype)
        h = _vp()
        _call(self._p + "transform_create_independent", ctypes.byref(h), max_num_threads,
              processing_unit, transform_type, dim_x, dim_y, dim_z, num_local_elements, index_format,
              ptr or None)
        self._h = h
        self._type = transform_type
        self._keep: tuple = ()

    @classmethod
    def _wrap(cls, h: ctypes.c_void_p, dtype: str, transform_type: int, keep: tuple = ()) -> "Transform":
        obj = cls.__new__(cls)
        obj.dtype = dtype
        obj._p = _prefix(dtype)
        obj._h = h
        obj._type = transform_type
        obj._keep = keep
        return obj

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            getattr(_lib, self._p + "transform_destroy")(h)
            self._h = None

    @property
    def handle(self) -> int:
        return int(self._h.value)

    def _get(self, name: str) -> int:
        v = ctypes.c_int(0)
        _call(self._p + "transform_" + name, self._h, ctypes.byref(v))
        return v.value

    def _get_ll(self, name: str) -> int:
        v = ctypes.c_longlong(0)
        _call(self._p + "transform_" + name, self._h, ctypes.byref(v))
        return v.value

    def clone(self) -> "Transform":
        h = _vp()
        _call(self._p + "transform_clone", self._h, ctypes.byref(h))
        return Transform._wrap(h, self.dtype, self._type)

    def type(self) -> int:
        return self._type

    def dim_x(self) -> int: return self._get("dim_x")
    def dim_y(self) -> int: return self._get("dim_y")
    def dim_z(self) -> int: return self._get("dim_z")
    def local_z_length(self) -> int: return self._get("local_z_length")
    def local_slice_size(self) -> int: return self._get("local_slice_size")
    def local_z_offset(self) -> int: return self._get("local_z_offset")
    def num_local_elements(self) -> int: return self._get("num_local_elements")
    def device_id(self) -> int: return self._get("device_id")
    def num_threads(self) -> int: return self._get("num_threads")
    def execution_mode(self) -> int: return self._get("execution_mode")
    def global_size(self) -> int: return self._get_ll("global_size")
    def num_global_elements(self) -> int: return self._get_ll("num_global_elements")

    def set_execution_mode(self, mode: int) -> None:
        _call(self._p + "transform_set_execution_mode", self._h, mode)

    def space_domain_data(self, location: int) -> int:
        """Address of the internal space-domain buffer on the host (pinned) or the GPU."""
        p = _vp()
        _call(self._p + "transform_get_space_domain", self._h, location, ctypes.byref(p))
        return int(p.value or 0)

    def backward(self, input: Any, output: Any = SPFFT_PU_GPU) -> None:
        """Frequency -> space. ``output`` is a processing-unit location (internal buffer) or an
        external buffer."""
        if isinstance(output, int) and output in (SPFFT_PU_HOST, SPFFT_PU_GPU):
            _call(self._p + "transform_backward", self._h, address(input), output)
        else:
            _call(self._p + "transform_backward_ptr", self._h, address(input), address(output))

    def forward(self, input: Any, output: Any, scaling: int = SPFFT_NO_SCALING) -> None:
        """Space -> frequency. ``input`` is a processing-unit location or an external buffer."""
        if isinstance(input, int) and input in (SPFFT_PU_HOST, SPFFT_PU_GPU):
            _call(self._p + "transform_forward", self._h, input, address(output), scaling)
        else:
            _call(self._p + "transform_forward_ptr", self._h, address(input), address(output), scaling)

    # ---- extensions ----------------------------------------------------------------------------
    def path_info(self) -> dict:
        """Which kernels run: size-specialised z pass; fused plane pass or split specialised y and x
        passes (else the generic ones)."""
        v = ctypes.c_int(0)
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_path_info", self._h, ctypes.byref(v))
        return {"fast_z": bool(v.value & 1), "fused_plane": bool(v.value & 2),
                "split_plane": bool(v.value & 4)}

    def autotune(self, repetitions: int = 5) -> float:
        """Time every valid tile shape and plane strategy and keep the fastest; returns its time
        per backward + forward pair in ms (overwrites the grid's internal device space domain)."""
        ms = ctypes.c_float(0.0)
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_autotune", self._h, int(repetitions),
              ctypes.byref(ms))
        return float(ms.value)

    def tuning(self) -> dict:
        """The tile shapes the transform runs with."""
        v = (ctypes.c_int * 6)()
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_tuning", self._h, v)
        xb = ctypes.c_int(0)
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_x_backward_rows", self._h, ctypes.byref(xb))
        return {"sticks_per_z_block": v[0], "plane": ("generic", "fused", "split")[v[1]],
                "fused_half_rows": v[2], "fused_threads": v[3], "columns_per_y_block": v[4],
                "rows_per_x_block": v[5], "rows_per_x_backward_block": xb.value}

    def splits(self) -> dict:
        """Split of each size-specialised pass: (A, B) for a two-pass split, (A, B1, B2) for a
        three-pass split (None for a generic-kernel pass)."""
        v = (ctypes.c_int * 18)()
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_split_stages", self._h, v)
        out = {}
        for i, name in enumerate(["z_backward", "z_forward", "y_backward", "y_forward", "x_backward",
                                  "x_forward"]):
            st = [v[3 * i + j] for j in range(3)]
            out[name] = tuple(r for r in st if r > 0) if st[0] > 0 else None
        return out

    def radix_plans(self) -> list:
        """Radix stages of the z, y and x lengths ([[...], [...], [...]]): the generic kernels'
        plan, or the two radices of a size-specialised backward pass's split."""
        stages = (ctypes.c_int * 3)()
        radices = (ctypes.c_int * (3 * 24))()
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_radix_plans", self._h, stages, radices)
        return [[radices[d * 24 + i] for i in range(stages[d])] for d in range(3)]
    def set_stream(self, stream: Any) -> None:
        """Run every later call on this CUDA stream (torch.cuda.Stream, cudaStream_t int or None)."""
        ptr = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_set_stream", self._h, ptr)

    def adjoint_backward(self, grad_space: Any, grad_values: Any, stream: Any = None) -> None:
        """Gradient of the frequency values from the gradient of the space domain."""
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_adjoint_backward", self._h,
              address(grad_space), address(grad_values), _stream_handle(stream))

    def adjoint_forward(self, grad_values: Any, grad_space: Any, scaling: int = SPFFT_NO_SCALING,
                        stream: Any = None) -> None:
        """Gradient of the space domain from the gradient of the frequency values."""
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_adjoint_forward", self._h,
              address(grad_values), address(grad_space), scaling, _stream_handle(stream))

    def backward_device(self, values: Any, space: Any, stream: Any = None) -> None:
        s = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_backward_device", self._h,
              address(values), address(space), s)

    def forward_device(self, space: Any, values: Any, scaling: int = SPFFT_NO_SCALING,
                       stream: Any = None) -> None:
        s = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        _call("spfft_gb300_" + self._p[len("spfft_"):] + "transform_forward_device", self._h,
              address(space), address(values), scaling, s)


def stage_times(transform: "Transform", direction: int, input: Any, output: Any,
                scaling: int = SPFFT_NO_SCALING, stream: Any = None) -> list:
    """Kernel times (ms) of one backward (direction 0) or forward (1) pass: [z, y, x] for
    backward, [x, y, z] for forward."""
    ms = (ctypes.c_float * 3)()
    s = None if stream is None else int(getattr(stream, "cuda_stream", stream))
    _call("spfft_gb300_" + transform._p[len("spfft_"):] + "transform_stage_times", transform._h,
          direction, address(input), address(output), scaling, s, ms)
    return [float(v) for v in ms]


def _handles(transforms) -> ctypes.Array:
    arr = (_vp * len(transforms))()
    for i, t in enumerate(transforms):
        arr[i] = t._h.value
    return arr


def multi_transform_backward(transforms, inputs, outputs) -> None:
    """Reference spfft::multi_transform_backward: outputs are locations or buffers."""
    n = len(transforms)
    p = transforms[0]._p if n else "spfft_"
    ins = (_vp * n)(*[address(x) for x in inputs])
    if all(isinstance(o, int) and o in (SPFFT_PU_HOST, SPFFT_PU_GPU) for o in outputs):
        locs = (_i * n)(*outputs)
        _call(p + "multi_transform_backward", n, _handles(transforms), ins, locs)
    else:
        outs = (_vp * n)(*[address(x) for x in outputs])
        _call(p + "multi_transform_backward_ptr", n, _handles(transforms), ins, outs)


def multi_transform_forward(transforms, inputs, outputs, scalings=None) -> None:
    n = len(transforms)
    p = transforms[0]._p if n else "spfft_"
    sc = (_i * n)(*(scalings or [SPFFT_NO_SCALING] * n))
    outs = (_vp * n)(*[address(x) for x in outputs])
    if all(isinstance(i, int) and i in (SPFFT_PU_HOST, SPFFT_PU_GPU) for i in inputs):
        locs = (_i * n)(*inputs)
        _call(p + "multi_transform_forward", n, _handles(transforms), locs, outs, sc)
    else:
        ins = (_vp * n)(*[address(x) for x in inputs])
        _call(p + "multi_transform_forward_ptr", n, _handles(transforms), ins, outs, sc)


def multi_batched_calls() -> int:
    """How many multi-transform calls so far ran as one batched execution."""
    c = ctypes.c_longlong()
    _call("spfft_gb300_multi_batched_calls", ctypes.byref(c))
    return int(c.value)


def _stream_handle(stream: Any):
    return None if stream is None else int(getattr(stream, "cuda_stream", stream))


class Batch:
    """Many transforms executed together: each pass of each group of equally shaped transforms is
    one kernel launch, and a backward + forward pair can run as a captured CUDA graph
    (``spfft_gb300_batch_*`` in include/spfft/spfft_gb300.h)."""

    def __init__(self, transforms):
        if not transforms:
            raise ValueError("empty batch")
        dtypes = {t.dtype for t in transforms}
        if len(dtypes) != 1:
            raise ValueError("a batch holds transforms of one precision")
        self.dtype = dtypes.pop()
        self._transforms = list(transforms)
        h = _vp()
        fn = "spfft_gb300_float_batch_create" if _prefix(self.dtype) == "spfft_float_" else "spfft_gb300_batch_create"
        _call(fn, ctypes.byref(h), len(transforms), _handles(transforms))
        self._h = h
        self._bound = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.spfft_gb300_batch_destroy(h)
            self._h = None

    def bind(self, values, spaces) -> None:
        n = len(self._transforms)
        v = (_vp * n)(*[address(x) for x in values])
        s = (_vp * n)(*[address(x) for x in spaces])
        _call("spfft_gb300_batch_bind", self._h, v, s)
        self._bound = (list(values), list(spaces))  # keep the buffers alive

    def backward(self, stream: Any = None) -> None:
        _call("spfft_gb300_batch_backward", self._h, _stream_handle(stream))

    def forward(self, scaling: int = SPFFT_NO_SCALING, stream: Any = None) -> None:
        _call("spfft_gb300_batch_forward", self._h, scaling, _stream_handle(stream))

    def pair_graph(self, scaling: int = SPFFT_NO_SCALING, stream: Any = None) -> None:
        _call("spfft_gb300_batch_pair_graph", self._h, scaling, _stream_handle(stream))

    def stage_times(self, direction: int, scaling: int = SPFFT_NO_SCALING, stream: Any = None) -> list:
        """Pass times (ms) of one direction, the groups run pass by pass (z, y, x backward order)."""
        ms = (ctypes.c_float * 3)()
        _call("spfft_gb300_batch_stage_times", self._h, direction, scaling, _stream_handle(stream), ms)
        return [float(m) for m in ms]

    def info(self) -> dict:
        g, u, l = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _call("spfft_gb300_batch_info", self._h, ctypes.byref(g), ctypes.byref(u), ctypes.byref(l))
        return {"groups": g.value, "unbatched": u.value, "launches_per_pair": l.value}

    def autotune(self, repetitions: int = 3, stream: Any = None) -> float:
        """Per shape group, keep the fastest plane strategy and z block size (overwrites the bound
        buffers; drops captured graphs). Returns the sum of the groups' best ms per pair."""
        ms = ctypes.c_float(0.0)
        _call("spfft_gb300_batch_autotune", self._h, int(repetitions), _stream_handle(stream), ctypes.byref(ms))
        return float(ms.value)

    def transform_path(self, index: int) -> int:
        """0 unbatched, 1 batched with split y and x passes, 2 batched with the fused plane pass."""
        v = ctypes.c_int()
        _call("spfft_gb300_batch_transform_path", self._h, int(index), ctypes.byref(v))
        return v.value

    def row_groups(self, index: int) -> int:
        """Row groups of the fused plane passes of transform `index` (0 when not fused)."""
        v = ctypes.c_int()
        _call("spfft_gb300_batch_row_groups", self._h, int(index), ctypes.byref(v))
        return v.value
