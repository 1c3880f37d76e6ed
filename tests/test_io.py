"""npz round trip of screens and metadata in the reference's format (CPU)."""

import json
import sys
from pathlib import Path

import numpy as np
import pytest

from pyturb_gb300 import io as pio


def test_npz_round_trip(tmp_path):
    data = np.random.default_rng(0).standard_normal((3, 16, 16)).astype(np.float32)
    p = tmp_path / "screens.npz"
    pio.save(p, data, pixel_scale=0.0156, r0=0.15, L0=25.0, units="metres", seed=None)
    got, meta = pio.load(p)
    assert got.dtype == np.float32 and np.array_equal(got, data)
    assert meta["pixel_scale"] == 0.0156 and meta["units"] == "metres"
    assert "seed" not in meta and "pyturb_version" in meta


def test_file_layout_matches_the_reference_format(tmp_path):
    p = tmp_path / "x.npz"
    pio.save(p, np.zeros((4, 4)), r0=0.1)
    with np.load(p, allow_pickle=False) as h:
        assert set(h.files) == {"data", "__pyturb_meta__"}
        assert json.loads(str(h["__pyturb_meta__"]))["r0"] == 0.1


def test_fits_without_astropy_says_so(tmp_path):
    try:
        import astropy  # noqa: F401
        pytest.skip("astropy present")
    except ImportError:
        pass
    with pytest.raises(ImportError):
        pio.save(tmp_path / "x.fits", np.zeros((4, 4)))


def test_reference_reads_our_files_and_we_read_its(tmp_path):
    src = Path("/root/reference/src")
    if not src.exists():
        pytest.skip("reference sources not present")
    sys.path.insert(0, str(src))
    try:
        from pyturb import io as rio
    except Exception as exc:  # pragma: no cover
        pytest.skip(f"reference not importable: {exc}")
    finally:
        sys.path.remove(str(src))
    data = np.arange(16, dtype=np.float32).reshape(4, 4)
    ours = tmp_path / "ours.npz"
    pio.save(ours, data, r0=0.2, wavelength=5e-7)
    d, m = rio.load(ours)
    assert np.array_equal(d, data) and m["r0"] == 0.2
    theirs = tmp_path / "theirs.npz"
    rio.save(theirs, data, L0=30.0)
    d, m = pio.load(theirs)
    assert np.array_equal(d, data) and m["L0"] == 30.0
