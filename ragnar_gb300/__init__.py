"""ragnar_gb300 -- GB300-native (sm_103a) synchrotron path of the ragnar library.

Drop-in for the reference's ``ragnar`` module on the synchrotron path::

    import ragnar_gb300 as rg
    rg.Initialize()
    prtls = rg.Particles_3D("e-")
    prtls.fromArrays({"U1": u1, "U2": u2, "U3": u3, "B3": b3})
    spec = rg.SynchrotronSpectrum_3D(prtls, rg.Logbins(1e-2, 1e7, 200, rg.EnergyUnits.mec2), 1, 1, 1)

The compute runs in the CUDA library behind ``include/ragnar_gb300.h``; there is
no CPU fallback: importing fails loudly if the native extension is missing.
"""

from __future__ import annotations

import os

_HERE = os.path.dirname(os.path.abspath(__file__))

try:
    from . import _ragnar  # noqa: F401
    from ._ragnar import *  # noqa: F401,F403
except ImportError as exc:  # pragma: no cover - exercised only on a broken install
    raise ImportError(
        "ragnar_gb300's native extension is not built or cannot be loaded "
        f"({exc}); build it with `python ragnar_gb300/build.py`"
    ) from exc

LIBRARY_PATH = os.path.join(_HERE, "_lib", "libragnar_gb300.so")
