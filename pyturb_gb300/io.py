"""Save and load screens with their metadata (drop-in for ``pyturb.io``).

The on-disk format is the reference's (``src/pyturb/io.py:25-87``): a NumPy
``.npz`` holding the array under ``data`` and a JSON string of the metadata
under ``__pyturb_meta__``; ``.fits``/``.fit`` paths go through astropy's
FITS writer. The key names and the JSON encoding are kept so that files move
freely between pyturb and this backend. Device tensors are copied to the
host first.
"""

from __future__ import annotations

import json
import os
from typing import Any, Dict, Tuple, Union

import numpy as np

from .backend import to_numpy

__all__ = ["save", "load"]

META_KEY = "__pyturb_meta__"


def _meta(metadata: Dict[str, Any]) -> Dict[str, Any]:
    from . import __version__

    out = {str(k): v for k, v in metadata.items() if v is not None}
    out.setdefault("pyturb_version", __version__)
    out.setdefault("backend", "pyturb_gb300")
    return out


def _is_fits(path: str) -> bool:
    return path.lower().endswith((".fits", ".fit"))


def _fits():
    try:
        from astropy.io import fits
    except ImportError as exc:
        raise ImportError("FITS support needs astropy (pip install astropy); "
                          "use a .npz path instead.") from exc
    return fits


def save(path: Union[str, os.PathLike], data: Any, **metadata: Any) -> None:
    """Write ``data`` (a screen or a stack; NumPy or a CUDA tensor) to ``path``
    with ``metadata`` (scalars and strings; ``None`` values are dropped)."""
    array = np.ascontiguousarray(to_numpy(data))
    meta = _meta(dict(metadata))
    path = os.fspath(path)
    if _is_fits(path):
        fits = _fits()
        hdu = fits.PrimaryHDU(data=array)
        hdu.header["BUNIT"] = str(meta.get("units", "radians"))
        for key, value in meta.items():
            if isinstance(value, (bool, int, float, str)):
                hdu.header["HIERARCH " + key.upper()] = value
        hdu.header["HIERARCH PYTURB_META"] = json.dumps(meta)
        hdu.writeto(path, overwrite=True)
        return
    np.savez(path, data=array, **{META_KEY: json.dumps(meta)})


def load(path: Union[str, os.PathLike]) -> Tuple[np.ndarray, Dict[str, Any]]:
    """``(array, metadata)`` from a file written by :func:`save` or by pyturb."""
    path = os.fspath(path)
    if _is_fits(path):
        fits = _fits()
        with fits.open(path) as hdul:
            data = np.asarray(hdul[0].data)
            raw = hdul[0].header.get("HIERARCH PYTURB_META")
        return data, (json.loads(raw) if raw else {})
    with np.load(path, allow_pickle=False) as handle:
        data = handle["data"]
        meta = json.loads(str(handle[META_KEY])) if META_KEY in handle.files else {}
    return data, meta
