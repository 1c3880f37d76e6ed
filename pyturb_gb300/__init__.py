"""pyturb_gb300 — the GB300-native (sm_103a) phase-screen hot path of pyturb.

Drop-in GPU backend for pyturb's ``PhaseScreen.generate``,
``InfinitePhaseScreen``, ``FourierFlowScreen`` and ``Atmosphere.frames`` /
``opd`` / ``evolve`` / ``sample``: same constructors and call surface, float32
CUDA ``torch.Tensor`` outputs, hand-written CUDA kernels reached through the
C-ABI library ``libpyturb_gb300.so`` (``include/pyturb_gb300.h``). There is no
CPU path: ``device="cpu"`` is refused and a missing GPU or library raises.
"""

from .atmosphere import Atmosphere, ExtrudeBoilingPerformanceWarning, FrameLoop, PeriodicWrapWarning
from .backend import to_numpy
from .extrude import ExtrudedAtmosphere, build_extrusion, phase_covariance
from .flow import FourierFlowScreen
from .fourier import PhaseScreen
from .infinite import InfinitePhaseScreen
from .io import load, save
from .optics import air_refractivity, r0_at_wavelength, seeing_from_r0, water_vapour_refractivity
from .profiles import Layer

__version__ = "0.1.0"

__all__ = [
    "Atmosphere",
    "FrameLoop",
    "PeriodicWrapWarning",
    "ExtrudeBoilingPerformanceWarning",
    "PhaseScreen",
    "FourierFlowScreen",
    "InfinitePhaseScreen",
    "ExtrudedAtmosphere",
    "Layer",
    "phase_covariance",
    "build_extrusion",
    "to_numpy",
    "save",
    "load",
    "air_refractivity",
    "water_vapour_refractivity",
    "r0_at_wavelength",
    "seeing_from_r0",
    "__version__",
]
