"""The case-file front end (dgcom_gb300/case.py) on the host: the
reference's own example case (cases/tidal_channel/case.toml, read in place
where present) and small case files written here, for the schema's
defaults, its strictness, what the device path refuses by name, the
domain (drop_land, tags, boundaries), the stations' probes, and a short
run of a case on the oracle."""

import math
import textwrap

import numpy as np
import pytest

from dgcom_gb300 import abi, gmsh
from dgcom_gb300 import case as C
from dgcom_gb300.astronomy import ModelClock
from dgcom_gb300.device import DeviceRun
from dgcom_gb300.mesh import TAG_OPEN, TAG_TIDAL, TAG_WALL, custom_tag, graded_jittered_box
from oracle_lib import oracle

BASIN = """
[run]
name = "basin"
duration_hours = 0.05

[mesh]
order = 2
drop_land = true

[mesh.rectangle]
x_m = [0.0, 8000.0]
y_m = [0.0, 2000.0]
nx = 16
ny = 4
west = "tidal"

[bathymetry.ramp]
from_m = [0.0, 1000.0]
to_m = [8000.0, 1000.0]
depth_m = [20.0, -6.0]

[physics]
coriolis = { f_plane = 1.1e-4 }
friction = { manning = 0.03 }

[[boundary]]
tag = "tidal"
velocity = "incoming_wave"
[boundary.tide]
ramp_hours = 0.0
constituents = [{ name = "m2", amplitude_m = 0.5, phase_deg = 10.0 }]

[numerics]
integrator = "ssp_rk3"

[output]
interval_minutes = 1.0

[[output.station]]
name = "mouth"
x_m = 300.0
y_m = 1000.0

[[output.station]]
name = "flats"
x_m = 5900.0
y_m = 1000.0
open_water_depth_m = 2.0
"""


def write(tmp_path, text, name="case.toml"):
    p = tmp_path / name
    p.write_text(textwrap.dedent(text))
    return p


def test_the_reference_tidal_channel_case(reference_data):
    case = C.load_case(reference_data("cases/tidal_channel/case.toml"))
    assert (case.name, case.duration_s, case.order) == ("tidal_channel", 25 * 3600.0, 2)
    assert case.scheme == abi.SSP_RK43 and abs(case.cfl - 0.9 * 1.51) < 1e-15
    assert case.rectangle["sides"] == (TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN)
    assert not case.drop_land and case.manning == 0.025
    assert abs(case.coriolis_f - 2 * 7.2921e-5 * math.sin(math.radians(63.5))) < 1e-8
    tide = case.boundaries[TAG_OPEN]
    assert tide.ramp_duration == 7200.0 and not tide.incoming_wave
    m2, s2 = tide.constituents
    clock = ModelClock("2025-06-15T00:00:00Z")
    d = clock.nodal_drift("M2")
    assert (m2.f, m2.u_deg, m2.v0_deg) == (d.at_start.f, d.at_start.u_deg, d.at_start.v0_deg)
    assert s2.amplitude == 0.35 and abs(s2.phase + math.radians(30.0)) < 1e-15
    assert min(s2.v0_deg, 360.0 - s2.v0_deg) < 1e-6  # S2's V₀ is 0 at UT midnight
    assert case.station_interval_s == case.interval_s == 1800.0
    form, q = C.build_form(case)
    assert form.mesh.n_elements == 160 and abs(q[0].max() - 30.0) < 1e-12
    bed = form.bathymetry.reshape(160, 9)
    depths = {s.name: -C.station_probe(form.mesh, 2, bed, s).value(bed) for s in case.stations}
    assert abs(depths["mouth"] - 28.4) < 1e-9 and abs(depths["middle"] - 14.0) < 1e-9
    assert abs(depths["head"] - 2.8) < 1e-9  # open_water_depth_m = 1 keeps it in place


def test_defaults_and_drop_land(tmp_path):
    case = C.load_case(write(tmp_path, BASIN))
    assert case.scheme == abi.SSP_RK3 and abs(case.cfl - 0.9 * 1.04) < 1e-15
    assert case.levels == 0 and case.dt_max is None and case.gravity == 9.81
    assert case.wetting_drying and case.eta0 == 0.0 and case.ordinal == 0
    assert case.output_dir == tmp_path / "output" / "basin"
    form, q = C.build_form(case)
    # depth 20 → −6 m along x: columns whose nodes are all above the datum
    # (x ≥ 6154 m) are dropped; their faces to the kept ones become walls
    x, _ = form.positions()
    assert form.mesh.n_elements == 13 * 4
    assert x.max() <= 6500.0 + 1e-9
    rows = gmsh.boundary_edges(form.mesh)
    east = rows[np.isclose(form.mesh.vertices[rows[:, 2], 0], 6500.0)
                & np.isclose(form.mesh.vertices[rows[:, 3], 0], 6500.0)]
    assert len(east) == 4 and (east[:, 4] == TAG_WALL).all()
    assert set(form.boundaries) == {TAG_WALL, TAG_TIDAL}
    assert form.boundaries[TAG_TIDAL].incoming_wave
    bed = form.bathymetry.reshape(-1, 9)
    probes = {s.name: C.station_probe(form.mesh, 2, bed, s) for s in case.stations}
    assert (probes["mouth"].x, probes["mouth"].y) == (300.0, 1000.0)
    flats = probes["flats"]  # 5900 m is under 2 m at some node: moved west into deeper water
    assert flats.x < 5900.0 and (-bed[flats.element] >= 2.0).all()


@pytest.mark.parametrize("text, message", [
    ("[run]\nduration_hours = 1\nbogus = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n", "unknown key run.bogus"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[waves]\n", "spectral waves is not on the device path"),
    ("[run]\nduration_hours = 1\n[mesh]\norigin = { lat = 63.0, lon = 8.0 }\n"
     "[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n[bathymetry]\ndepth_m = 1\n",
     "mesh.origin: a mesh placed on the Earth"),
    ("[run]\nduration_hours = 1\n[mesh]\norder = 6\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\n"
     "nx=1\nny=1\n[bathymetry]\ndepth_m = 1\n", "mesh.order must be 1–4"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\nramp = { from_m=[0,0], to_m=[1,0], depth_m=[1,2] }\n",
     "exactly one of `depth_m` and `ramp`"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[physics]\nfriction = { drag_coefficient = 0.0025 }\n",
     "quadratic drag"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[physics]\nsmagorinsky = 0.1\n", "horizontal viscosity"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[[boundary]]\ntag = \"open\"\n[boundary.atlas]\nfile = \"a.txt\"\n",
     "tidal atlas"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[output]\ninterval_minutes = 10\nstation_interval_minutes = 4\n",
     "whole multiple"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[numerics]\nlocal_time_stepping_levels = 12\n", "at most 8"),
    ("[run]\nduration_hours = 1\n[mesh]\n[mesh.rectangle]\nx_m=[0,1]\ny_m=[0,1]\nnx=1\nny=1\n"
     "[bathymetry]\ndepth_m = 1\n[compute]\ndevice = \"tpu\"\n", "compute.device"),
])
def test_refusals_name_the_key(tmp_path, text, message):
    with pytest.raises(C.CaseError, match=message):
        C.load_case(write(tmp_path, text))


def test_open_faces_need_a_boundary(tmp_path):
    text = BASIN.replace('west = "tidal"', 'west = "open"')
    with pytest.raises(C.CaseError, match="no \\[\\[boundary\\]\\]"):
        C.build_form(C.load_case(write(tmp_path, text)))


def test_a_gmsh_mesh_through_a_case(tmp_path):
    m = graded_jittered_box(3000.0, 2000.0, 8, 6, size_range=(250.0, 500.0), seed=2,
                            sides=(TAG_WALL, custom_tag(13), TAG_WALL, TAG_OPEN))
    gmsh.write_gmsh_mesh(m, tmp_path / "box.msh")
    text = """
    [run]
    duration_hours = 1.0
    [mesh]
    order = 3
    gmsh = "box.msh"
    [bathymetry]
    depth_m = 15.0
    [[boundary]]
    tag = "open"
    still = { eta_m = 0.25 }
    """
    case = C.load_case(write(tmp_path, text))
    form, q = C.build_form(case)
    assert form.mesh.n_elements == 48 and form.order == 3
    assert set(form.boundaries) == {TAG_WALL, TAG_OPEN, custom_tag(13)}
    still = form.boundaries[TAG_OPEN]
    assert still.constituents == [] and still.mean_elevation == 0.25
    assert np.allclose(q[0], 15.0)


def test_a_case_runs_on_the_oracle(tmp_path):
    """The case's form, state and run on the oracle: the stations sampled
    at every interval, the tide entering at the mouth."""
    case = C.load_case(write(tmp_path, BASIN))
    form, q = C.build_form(case)
    bed = form.bathymetry.reshape(form.mesh.n_elements, 9)
    probes = [C.station_probe(form.mesh, 2, bed, s) for s in case.stations]
    times = []
    ref = oracle(form)
    try:
        ref.upload(*q)
        rep = ref.run_with_callback(
            DeviceRun(span=(0.0, case.duration_s), cfl=case.cfl, interval=case.station_interval_s,
                      scheme=case.scheme),
            lambda t, h, hu, hv: times.append((t, probes[0].value(h.reshape(-1, 9)))))
        assert rep.success, rep.message
    finally:
        ref.close()
    assert [t for t, _ in times] == pytest.approx([0.0, 60.0, 120.0, 180.0])
    assert abs(times[0][1] - 19.025) < 1e-9  # still water at the mouth: depth 20 − 26·300/8000
    assert times[-1][1] != times[0][1]
