"""CPU oracle for pyturb's phase-screen hot path — TEST INFRASTRUCTURE ONLY.

A plain float64 NumPy/SciPy restatement of the reference algorithm
(jacotay7/pyturb ``src/pyturb``), each function citing the reference
``file:line`` it follows. It is the checker for the GPU path: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import it, and never as the thing measured or shipped. The product
package ``pyturb_gb300`` does not import this module.

Pinned against the reference: ``tests/golden/make_golden.py`` runs the real
reference (float64) in the build container on fixed seeds and stores the
inputs and outputs under ``tests/golden/``; ``tests/test_oracle_golden.py``
checks that this restatement reproduces every fixture.

Every random draw goes through a ``numpy.random.Generator``-like object
passed in by the caller, consumed in the reference's own order, so the same
seeds reproduce the reference run exactly.
"""

from .spectral import (OracleAtmosphere, OracleFlow, OraclePhaseScreen, band_amplitude,
                       build_filters, psd)
from .extrusion import (OracleExtruded, OracleInfinite, build_extrusion, phase_covariance,
                        compact_row_ring)

__all__ = [
    "OracleAtmosphere", "OracleFlow", "OraclePhaseScreen", "OracleExtruded", "OracleInfinite",
    "band_amplitude", "build_filters", "psd", "build_extrusion", "phase_covariance",
    "compact_row_ring",
]
