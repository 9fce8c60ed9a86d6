"""Test infrastructure: the oracle (oracle/liboracle.so, the CPU
restatement of the reference path) bound through the same ABI wrapper as
the CUDA library, plus its pointwise entry points for the known-answer
tests."""

from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from dgcom_gb300 import abi  # noqa: E402
from dgcom_gb300.device import SWEPhysics2D  # noqa: E402

_dp = C.POINTER(C.c_double)
POINTWISE = {
    "set_threads": (C.c_int, [C.c_int]),
    "manning_cbrt": (C.c_double, [C.c_double]),
    "tidal_ramp": (C.c_double, [C.c_double, C.c_double]),
    "hypot": (C.c_double, [C.c_double, C.c_double]),
    "subcell_divergence": (C.c_int, [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp]),
    "drag_coefficient": (C.c_double, [C.c_int, C.c_double, C.c_double]),
    "atmosphere_source": (None, [C.c_double] * 5 + [C.c_int] + [C.c_double] * 4
                          + [C.POINTER(C.c_double)]),
    "inverse_barometer_level": (C.c_double, [C.c_double, C.c_double, C.c_double]),
    "characteristic_state": (None, [_dp, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_double, _dp]),
    "desingularized_velocity": (None, [C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
    "thin_layer_rate": (C.c_double, [C.c_double, C.c_double, C.c_double]),
    "correct_node": (None, [C.c_double, C.c_double, C.c_double, _dp]),
    "wintermeyer_flux": (None, [_dp, _dp, C.c_double, C.c_double, C.c_double, _dp]),
    "hydrostatic_hll": (None, [_dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double, _dp,
                               _dp]),
    "gll": (None, [C.c_int, _dp, _dp, _dp]),
    "positivity_cfl": (C.c_double, [C.c_int]),
    "positivity_bound": (None, [C.c_int, C.c_int, _dp]),
    "wet_dry_element": (C.c_int, [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double]),
    "damp_nodes": (None, [C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                          C.c_double, C.c_double, C.c_double]),
    "tide_elevation": (C.c_double, [C.POINTER(abi.Boundary), C.c_double]),
    "multirate_stats_get": (C.c_int, [C.c_void_p, C.POINTER(abi.MultirateStats)]),
    "time_stencil": (C.c_int, [_dp, C.c_int64, C.c_double, C.c_int, C.POINTER(C.c_int64), _dp]),
}

_libs: dict = {}


def oracle_library(contract: bool = False) -> abi.Library:
    """The oracle's library: the parity build, or with ``contract`` the
    FMA-contracted build (timed as a second CPU figure, never a checker)."""
    if contract not in _libs:
        sys.path.insert(0, str(ROOT / "oracle"))
        import build as oracle_build  # oracle/build.py

        path = oracle_build.build(contract=contract)
        _libs[contract] = abi.Library(C.CDLL(str(path)), "oracle", POINTWISE)
    return _libs[contract]


def oracle(form, threads: int | None = None, contract: bool = False) -> SWEPhysics2D:
    """The oracle's physics on ``form`` (the CUDA library's wrapper, bound
    to the oracle)."""
    lib = oracle_library(contract)
    if threads:
        lib.set_threads(threads)
    return SWEPhysics2D(form, 0, library=lib)


def arr(values):
    a = (C.c_double * len(values))(*values)
    return a
