"""Device selection, CUDA streams, noise streams and host/device conversion.

The reference chooses NumPy or CuPy from a ``device`` string
(``src/pyturb/backend.py:20-45``). This package *is* the GPU backend: the GPU
names select it, the CPU names are refused with a pointer back to the
reference's NumPy path, and there is no CPU fallback anywhere — if no CUDA
device or no native library is available the call fails loudly.
"""

from __future__ import annotations

import os
from typing import Any, Callable, Optional, Sequence

import numpy as np

_CPU_NAMES = frozenset({"cpu", "numpy"})
_GPU_NAMES = frozenset({"gpu", "cuda", "cupy", "gb300"})


def check_device(device: str) -> str:
    """Validate a device name (``src/pyturb/backend.py:20-45``); return ``"gpu"``."""
    name = str(device).lower()
    if name in _GPU_NAMES:
        return "gpu"
    if name in _CPU_NAMES:
        raise ValueError(
            f"device={device!r}: pyturb_gb300 is the GB300 GPU backend and has no "
            "CPU path; use pyturb itself for device='cpu'."
        )
    raise ValueError(
        f"Unknown device {device!r}. Expected one of {sorted(_GPU_NAMES)}."
    )


def torch_module():
    import torch

    return torch


def cuda_device():
    """The current CUDA device as a ``torch.device``; raises without a GPU."""
    torch = torch_module()
    if not torch.cuda.is_available():
        raise RuntimeError(
            "pyturb_gb300 needs a CUDA GPU (GB300, sm_103a); none is visible. "
            "There is no CPU fallback."
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle() -> int:
    """cudaStream_t of torch's current stream, so native work orders with torch's."""
    torch = torch_module()
    return torch.cuda.current_stream().cuda_stream


def to_numpy(array: Any) -> np.ndarray:
    """Copy a torch tensor (any device) or array-like to a host ``numpy.ndarray``."""
    if hasattr(array, "detach") and hasattr(array, "cpu"):
        return array.detach().cpu().numpy()
    if hasattr(array, "get"):
        return array.get()
    return np.asarray(array)


def seed_key(seed: Any) -> int:
    """64-bit Philox key for a user seed (int, SeedSequence, None = fresh entropy)."""
    if seed is None:
        return int.from_bytes(os.urandom(8), "little")
    if isinstance(seed, np.random.SeedSequence):
        state = seed.generate_state(2, dtype=np.uint32)
    elif isinstance(seed, np.random.Generator):
        state = seed.integers(0, 2**32, size=2, dtype=np.uint64).astype(np.uint32)
    else:
        state = np.random.SeedSequence(int(seed)).generate_state(2, dtype=np.uint32)
    return int(state[0]) | (int(state[1]) << 32)


HostNoise = Callable[[Any], Any]


class NoiseStream:
    """Gaussian noise for one object: in-kernel Philox, or injected host normals.

    With ``host_noise`` None the kernels draw Philox4x32-10 normals keyed by
    ``key`` and a per-call counter (``call``). With ``host_noise`` given (a
    factory ``seed -> generator`` whose ``standard_normal(shape)`` returns
    float64 normals, e.g. ``numpy.random.default_rng``) the normals are drawn
    on the host in the reference's own draw order and uploaded: this is the
    parity mode that reproduces the reference run on the same seed.
    """

    def __init__(self, seed: Any, host_noise: Optional[HostNoise]) -> None:
        self.key = seed_key(seed)
        self.call = 0
        self.host = host_noise(seed) if host_noise is not None else None

    @property
    def injected(self) -> bool:
        return self.host is not None

    def next_call(self) -> int:
        c = self.call
        self.call += 1
        return c

    def next_key(self) -> int:
        """A fresh 64-bit key derived from (key, call) for whole-array fills."""
        z = (self.key + 0x9E3779B97F4A7C15 * (self.next_call() + 1)) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def draw(self, shape: Sequence[int]) -> np.ndarray:
        """Host normals in the reference's order (parity mode only)."""
        assert self.host is not None
        return np.asarray(self.host.standard_normal(tuple(shape)), dtype=np.float64)


def upload(array: np.ndarray, dtype=None):
    """Host array -> contiguous CUDA tensor (float32 unless ``dtype`` given)."""
    torch = torch_module()
    t = torch.from_numpy(np.ascontiguousarray(array))
    return t.to(device=cuda_device(), dtype=dtype or torch.float32).contiguous()


def dptr(tensor) -> int:
    return 0 if tensor is None else int(tensor.data_ptr())
