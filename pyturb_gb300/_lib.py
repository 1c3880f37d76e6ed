"""ctypes binding of ``libpyturb_gb300.so`` (declared in ``include/pyturb_gb300.h``).

Every native call goes through :func:`call`, which raises ``RuntimeError`` (or
``ValueError`` for argument errors) with the library's message when the
status is not ``PT_OK``. The library is built on first use if it is missing;
if it cannot be built or loaded the import of the GPU path fails loudly —
there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import threading
from typing import Any

from . import _build

PT_OK, PT_ERR_ARG, PT_ERR_CUDA, PT_ERR_UNSUPPORTED, PT_ERR_NUMERIC = 0, 1, 2, 3, 4
PT_MAX_SPARSE = 64

_lock = threading.Lock()
_lib = None

vp = C.c_void_p
i32 = C.c_int
u64 = C.c_uint64
f32 = C.c_float
f64 = C.c_double
sz = C.c_size_t
dptr = C.POINTER(C.c_double)


class ExtrudeJob(C.Structure):
    """``pt_extrude_job``."""

    _fields_ = [
        ("screen", C.c_int32),
        ("group", C.c_int32),
        ("head", C.c_int32),
        ("step", C.c_int32),
        ("bscale", C.c_float),
        ("pad", C.c_int32),
        ("key", C.c_uint64),
        ("row", C.c_uint64),
        ("noise_off", C.c_int64),
    ]


class SparseStencil(C.Structure):
    """``pt_sparse_stencil``: sparse points (rows back, column) after the full rows."""

    _fields_ = [
        ("count", C.c_int32),
        ("depth", C.c_int32 * PT_MAX_SPARSE),
        ("column", C.c_int32 * PT_MAX_SPARSE),
    ]


def sparse_stencil(points):
    """A ``SparseStencil`` for ``points`` = [(depth, column), ...], or None if empty."""
    points = list(points)
    if not points:
        return None
    if len(points) > PT_MAX_SPARSE:
        raise ValueError(f"at most {PT_MAX_SPARSE} sparse stencil points")
    st = SparseStencil()
    st.count = len(points)
    for i, (d, c) in enumerate(points):
        st.depth[i] = int(d)
        st.column[i] = int(c)
    return st


class ExtrudeAnchor(C.Structure):
    """``pt_extrude_anchor``: device tables of the float32 form's low-order anchor."""

    _fields_ = [
        ("modes", C.c_int32),
        ("pad", C.c_int32),
        ("t_hi", C.c_void_p),
        ("t_lo", C.c_void_p),
        ("u", C.c_void_p),
    ]


class ReadoutLayer(C.Structure):
    """``pt_readout_layer``."""

    _fields_ = [
        ("screen", C.c_int32),
        ("row_max", C.c_int32),
        ("anchor_phys", C.c_int32),
        ("pad", C.c_int32),
        ("cos_t", C.c_double),
        ("sin_t", C.c_double),
        ("mag", C.c_double),
        ("shift_along", C.c_double),
        ("shift_perp", C.c_double),
    ]


# name -> (restype, argtypes); exactly the entry points of pyturb_gb300.h
SIGNATURES = {
    "pt_version": (i32, []),
    "pt_last_error": (C.c_char_p, []),
    "pt_launch_count": (u64, []),
    "pt_prof_enable": (i32, [i32]),
    "pt_prof_report": (i32, [C.c_char_p, sz]),
    "pt_device_error": (i32, [C.POINTER(C.c_int), i32]),
    "pt_selftest_wait_timeout": (i32, [C.c_longlong, C.POINTER(C.c_int)]),
    "pt_grid_create": (i32, [C.POINTER(vp), i32, f64, i32, dptr]),
    "pt_grid_destroy": (i32, [vp]),
    "pt_grid_workspace_bytes": (sz, [vp, i32]),
    "pt_grid_radices": (i32, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pt_grid_set_radices": (i32, [vp, i32, C.POINTER(C.c_int)]),
    "pt_grid_set_cols_variant": (i32, [vp, i32]),
    "pt_ifft2": (i32, [vp, vp, vp, i32, vp, sz, vp]),
    "pt_ifft2_noalloc": (i32, [i32, vp, vp, i32, vp]),
    "pt_ifft2_tc": (i32, [i32, vp, vp, i32, vp]),
    "pt_generate": (i32, [vp, i32, vp, vp, vp, vp, u64, u64, i32, i32, f32, i32, vp, vp, sz, vp]),
    "pt_generate_scaled": (i32, [vp, i32, vp, vp, u64, u64, i32, i32, f32, vp, vp, vp, sz, vp]),
    "pt_layers_fill": (i32, [vp, i32, vp, vp, vp, vp, C.POINTER(C.c_uint64), vp, vp, vp]),
    "pt_frames": (i32, [vp, i32, vp, vp, i32, dptr, dptr, i32, i32, i32, f32, vp, vp, sz, vp]),
    "pt_layers_translate": (i32, [vp, i32, vp, vp, dptr, dptr, vp, vp, vp]),
    "pt_lgs_zoom": (i32, [i32, i32, i32, i32, vp, vp, vp, f32, vp, vp]),
    "pt_boil_step": (i32, [vp, i32, vp, vp, vp, vp, vp, vp, f64, vp, vp, u64, u64, vp]),
    "pt_aw_workspace_bytes": (sz, [i32, i32, C.POINTER(SparseStencil)]),
    "pt_aw_build": (i32, [i32, i32, C.POINTER(SparseStencil), f64, f64, f64, i32, vp, vp, vp, vp,
                          vp, vp, sz, vp]),
    "pt_extrude_workspace_bytes": (sz, [i32, i32, i32, i32]),
    "pt_extrude_rows": (i32, [i32, i32, C.POINTER(SparseStencil), i32, i32, i32, vp, vp,
                              C.POINTER(ExtrudeAnchor), vp, i32, C.POINTER(ExtrudeJob), vp, vp,
                              sz, vp]),
    "pt_extrude_batch": (i32, [i32, i32, C.POINTER(SparseStencil), i32, i32, i32, vp, vp,
                               C.POINTER(ExtrudeAnchor), vp, i32, vp, vp, vp, vp, vp, vp, vp,
                               sz, vp]),
    "pt_extrude_lo_bytes": (sz, [i32, i32, i32, i32]),
    "pt_extrude_lo_prepare": (i32, [i32, i32, i32, i32, vp, vp, sz, vp]),
    "pt_readout": (i32, [i32, i32, i32, i32, i32, C.POINTER(ReadoutLayer), vp, f32, vp, vp]),
    "pt_rows_sample": (i32, [i32, i32, i32, i32, i32, f64, vp, vp, vp]),
    "pt_lr_fix": (i32, [i32, i32, i32, i32, i32, vp, dptr, vp, vp]),
    "pt_lr_forward": (i32, [i32, i32, i32, i32, i32, i32, dptr, vp, vp, vp, vp, vp]),
    "pt_lr_partial_count": (sz, [i32, i32, i32, i32, i32]),
    "pt_lr_grad_params": (i32, [i32, i32, i32, i32, i32, i32, dptr, vp, vp, vp, vp, vp, vp]),
    "pt_lr_grad_screens": (i32, [i32, i32, i32, i32, i32, i32, dptr, vp, vp, vp, i32, vp, vp]),
    "pt_structure_workspace_bytes": (sz, [i32, i32, i32, i32]),
    "pt_structure_function": (i32, [i32, i32, i32, vp, i32, vp, vp, sz, vp]),
    "pt_matmul_nt_workspace_bytes": (sz, [i32, i32, i32]),
    "pt_matmul_nt": (i32, [i32, i32, i32, vp, vp, vp, vp, sz, vp]),
    "pt_temporal_psd_workspace_bytes": (sz, [vp, i32]),
    "pt_temporal_psd": (i32, [vp, i32, vp, f64, vp, vp, sz, vp]),
    "pt_tc_probe": (i32, [i32, i32, vp, vp, vp, vp]),
    "pt_fill_normals": (i32, [u64, u64, i32, i32, C.POINTER(f32), vp, vp]),
    "pt_ring_blend": (i32, [i32, i32, vp, i32, i32, f32, f32, vp, vp]),
    "pt_extrude_tc_operator_bytes": (sz, [i32, i32, i32, i32, i32]),
    "pt_extrude_tc_prepare": (i32, [i32, i32, i32, i32, vp, i32, vp, sz, vp]),
    "pt_extrude_tc_workspace_bytes": (sz, [i32, i32, i32, i32, i32]),
    "pt_extrude_batch_tc": (i32, [i32, i32, C.POINTER(SparseStencil), i32, i32, i32, vp, i32, vp,
                                  i32, vp, vp, vp, vp, vp, vp, vp, sz, vp]),
    "pt_synth_adj_pack": (i32, [i32, i32, i32, i32, f32, vp, vp, vp]),
    "pt_synth_adj_phasors": (i32, [i32, f64, i32, i32, vp, vp, vp, vp]),
    "pt_synth_adj_spectra": (i32, [i32, i32, i32, vp, vp, vp, i32, vp, vp]),
    "pt_synth_adj_params": (i32, [i32, f64, i32, i32, vp, vp, vp, vp, vp, vp]),
    "pt_synth_adj_sh": (i32, [vp, i32, i32, i32, vp, vp, vp]),
}


def load(build: bool = True) -> C.CDLL:
    """Load (building first if needed) the native library and bind its symbols."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build else _build.library_path()
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return load().pt_last_error().decode(errors="replace")


def call(name: str, *args: Any) -> None:
    """Invoke a status-returning entry point; raise on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc == PT_OK:
        return
    msg = lib.pt_last_error().decode(errors="replace")
    if rc == PT_ERR_ARG:
        raise ValueError(f"{name}: {msg}")
    raise RuntimeError(f"{name} failed (status {rc}): {msg}")


def launch_count() -> int:
    return int(load().pt_launch_count())


def prof_enable(on: bool) -> None:
    load().pt_prof_enable(1 if on else 0)


def prof_report() -> dict:
    """{kernel: (launches, total_ms)} since the last report (synchronises)."""
    buf = C.create_string_buffer(1 << 16)
    call("pt_prof_report", buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, count, ms = line.split()
        out[name] = (int(count), float(ms))
    return out


def as_dptr(arr) -> Any:
    """ctypes double* view of a C-contiguous float64 numpy array."""
    return arr.ctypes.data_as(dptr)
