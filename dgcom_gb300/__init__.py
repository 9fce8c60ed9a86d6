"""GB300-native FP64 2D shallow-water nodal-DG stage of DGCOM
(EmilLindfors/dgcom): the split-form `WetDry` right-hand side on
unstructured quads with its SSP-RK stage update, numerical flux, sources
and wet/dry limiter, as hand-written sm_103a CUDA behind a C ABI
(include/dgswe.h). This package is the host side above that ABI."""

from . import abi, cases, mesh, physics, tides  # noqa: F401
from .device import Cuda, DeviceError, DeviceRun, DeviceRunReport, SWEPhysics2D  # noqa: F401
from .physics import SWEDeviceForm2D, TidalBoundary, WallBoundary, at_rest  # noqa: F401


def build(force: bool = False) -> str:
    """Compile the CUDA library in place (nvcc, sm_103a)."""
    from ._build import build as _b

    return str(_b(force=force))
