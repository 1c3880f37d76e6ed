"""The C-ABI library builds, loads and exports every entry point the header
declares; argument errors are reported before any device work (no GPU needed)."""

import ctypes as C
import re
from pathlib import Path

import pytest

from pyturb_gb300 import _build, _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "pyturb_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("pt_generate", "pt_frames", "pt_extrude_rows", "pt_readout", "pt_ifft2",
                 "pt_grid_create", "pt_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_the_header_exactly():
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_library_is_built_for_sm_103a_only():
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert _build.library_path().exists()


def test_struct_layouts_match_header():
    assert C.sizeof(_lib.ExtrudeJob) == 48
    assert C.sizeof(_lib.ReadoutLayer) == 56
    assert C.sizeof(_lib.SparseStencil) == 4 + 2 * 4 * _lib.PT_MAX_SPARSE
    assert C.sizeof(_lib.ExtrudeAnchor) == 32


def _status(name, *args):
    return getattr(_lib.load(), name)(*args)


def test_argument_errors_before_device_work():
    lib = _lib.load()
    h = C.c_void_p()
    assert _status("pt_grid_create", C.byref(h), 1, 0.1, 0, None) == _lib.PT_ERR_ARG
    assert "ns must be" in _lib.last_error()
    assert _status("pt_grid_create", C.byref(h), 64, -1.0, 0, None) == _lib.PT_ERR_ARG
    assert _status("pt_grid_create", C.byref(h), 64, 0.1, 17, None) == _lib.PT_ERR_ARG
    assert _status("pt_generate", None, 1, None, None, None, None, 0, 0, 0, 1, 1.0, 0, None,
                   None, 0, None) == _lib.PT_ERR_ARG
    assert _status("pt_readout", 0, 8, 8, 1, 1, None, None, 1.0, None, None) == _lib.PT_ERR_ARG
    assert _status("pt_lgs_zoom", 1, 8, 8, 7, None, None, None, 1.0, None, None) == _lib.PT_ERR_ARG
    assert _status("pt_rows_sample", 8, 8, 3, 0, 4, 0.0, None, None, None) == _lib.PT_ERR_ARG
    assert _status("pt_extrude_rows", 0, 2, None, 0, 8, 1, None, None, None, None, 0, None, None,
                   None, 0, None) == _lib.PT_ERR_ARG
    anchor = _lib.ExtrudeAnchor(modes=16)
    assert _status("pt_extrude_rows", 16, 2, None, 0, 8, 1, C.c_void_p(256), None, C.byref(anchor),
                   C.c_void_p(256), 0, None, None, None, 0, None) == _lib.PT_ERR_ARG
    assert "32 or 64 modes" in _lib.last_error()
    # sparse points must lie deeper than the full rows and inside the width
    bad = _lib.sparse_stencil([(2, 5)])
    assert _status("pt_extrude_batch", 64, 2, C.byref(bad), 0, 128, 1, C.c_void_p(256), None, None,
                   C.c_void_p(256), 1, None, None, None, None, None, None, None, 0,
                   None) == _lib.PT_ERR_ARG
    assert _status("pt_aw_build", 0, 2, None, 0.1, 25.0, 0.0, 0, None, None, None, None, None, None,
                   0, None) == _lib.PT_ERR_ARG
    assert _status("pt_aw_build", 16, 2, None, 0.1, float("inf"), 0.0, 0, C.c_void_p(256), None,
                   None, None, None, C.c_void_p(256), 1 << 20, None) == _lib.PT_ERR_ARG
    assert "finite L0" in _lib.last_error()
    assert _status("pt_aw_build", 16, 2, C.byref(bad), 0.1, 25.0, 0.0, 0, C.c_void_p(256), None,
                   None, None, None, C.c_void_p(256), 1 << 20, None) == _lib.PT_ERR_ARG
    assert _status("pt_extrude_lo_prepare", 16, 2, 0, 1, None, None, 0, None) == _lib.PT_ERR_ARG
    assert lib.pt_version() >= 100
    with pytest.raises(ValueError, match="pt_grid_create"):
        _lib.call("pt_grid_create", C.byref(h), 1, 0.1, 0, None)


def test_workspace_queries_are_pure():
    lib = _lib.load()
    assert lib.pt_extrude_workspace_bytes(100, 2, 0, 9) > 100 * 3 * 9 * 4
    assert lib.pt_extrude_workspace_bytes(100, 2, 18, 9) > lib.pt_extrude_workspace_bytes(100, 2,
                                                                                          0, 9)
    assert lib.pt_extrude_workspace_bytes(0, 2, 0, 9) == 0
    assert lib.pt_extrude_workspace_bytes(100, 2, 65, 9) == 0
    # the FP64 operator build: the joint (Kz + W)^2 matrix dominates
    st = _lib.sparse_stencil([(4, 10), (8, 90)])
    nbytes = lib.pt_aw_workspace_bytes(100, 2, C.byref(st))
    assert nbytes >= (3 * 100 + 2) ** 2 * 8
    assert lib.pt_aw_workspace_bytes(100, 2, None) >= (3 * 100) ** 2 * 8
    assert lib.pt_aw_workspace_bytes(100, 2, C.byref(_lib.sparse_stencil([(1, 10)]))) == 0


def test_tensor_core_dft_argument_errors():
    """pt_ifft2_tc rejects other sizes, misaligned buffers and oversized batches
    before any device work."""
    ok = 1 << 20  # a 16-byte aligned stand-in address, never dereferenced
    assert _status("pt_ifft2_tc", 256, ok, ok, 1, None) == _lib.PT_ERR_UNSUPPORTED
    assert _status("pt_ifft2_tc", 512, ok + 8, ok, 1, None) == _lib.PT_ERR_ARG
    assert "aligned" in _lib.last_error()
    assert _status("pt_ifft2_tc", 512, ok, ok, 5_000_000, None) == _lib.PT_ERR_ARG
    assert _status("pt_ifft2_tc", 512, ok, ok, -1, None) == _lib.PT_ERR_ARG
    assert _status("pt_ifft2_tc", 512, ok, ok, 0, None) == 0


def test_adjoint_argument_errors():
    ok = 1 << 20
    assert _status("pt_synth_adj_sh", None, 1, 0, 8, ok, ok, None) == _lib.PT_ERR_ARG
    assert "grid is NULL" in _lib.last_error()
    mag = (C.c_double * 1)(1.0)
    # pupil footprint wider than the screen
    assert _status("pt_lr_grad_screens", 1, 1, 16, 1, 1, 32, mag, ok, ok, ok, 0, ok,
                   None) == _lib.PT_ERR_ARG
    assert _status("pt_synth_adj_spectra", 0, 1, 1, ok, ok, ok, 1, ok, None) == _lib.PT_ERR_ARG
