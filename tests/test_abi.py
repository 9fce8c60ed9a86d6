"""The C ABI on the CPU: the library loads and exports every entry point the
header declares, and its host-only set-up (dgswe_check_form) builds the
connectivity, geometry and tables of the reference's meshes. No kernel runs
here."""

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from dgcom_gb300 import abi, cases
from dgcom_gb300.mesh import TAG_OPEN, TAG_WALL, uniform_periodic, uniform_rectangle
from dgcom_gb300.physics import SWEDeviceForm2D, TidalBoundary, WallBoundary

HEADER = Path(__file__).resolve().parents[1] / "include" / "dgswe.h"


def declared():
    text = HEADER.read_text()
    # declarations start a line with their return type
    return sorted(set(re.findall(r"^(?:const\s+)?[a-z_0-9]+[\s*]+(dgswe_[a-z_0-9]+)\s*\(",
                                 text, flags=re.M)))


def test_library_exports_every_declared_entry_point(cuda_lib):
    names = declared()
    assert len(names) >= 17
    for name in names:
        assert hasattr(cuda_lib.cdll, name), name
    assert sorted(abi.exported_symbols()) == names
    assert cuda_lib.abi_version() == abi.ABI_VERSION
    assert cuda_lib.status_string(abi.ERR_NONFINITE).decode() == "the state is not finite"


def check(cuda_lib, form):
    c_form, keep = form.to_c()
    info = abi.FormInfo()
    msg = C.create_string_buffer(256)
    status = cuda_lib.check_form(C.byref(c_form), C.byref(info), msg, 256)
    return status, info, msg.value.decode()


def test_check_form_counts_a_walled_rectangle(cuda_lib):
    for order in (1, 2, 3, 4):
        form = SWEDeviceForm2D(mesh=uniform_rectangle(0.0, 4000.0, 0.0, 2000.0, 8, 5), order=order,
                               bathymetry=None)
        status, info, _ = check(cuda_lib, form)
        assert status == abi.OK
        assert info.n_elements == 40
        assert info.n_interior_edges == 7 * 5 + 8 * 4
        assert info.n_boundary_faces == 2 * 8 + 2 * 5
        assert info.n_periodic_edges == 0 and info.n_affine == 40
        assert abs(info.area - 4000.0 * 2000.0) < 1e-6
        assert abs(info.min_jacobian - (500.0 * 400.0) / 4.0) < 1e-6


def test_check_form_pairs_periodic_faces(cuda_lib):
    form = SWEDeviceForm2D(mesh=uniform_periodic(0.0, 1.0, 0.0, 1.0, 3, 2), order=2)
    status, info, _ = check(cuda_lib, form)
    assert status == abi.OK
    assert info.n_boundary_faces == 0
    assert info.n_interior_edges == 2 * 3 * 2  # every face paired once
    assert info.n_periodic_edges == 2 + 3


def test_check_form_refuses_bad_forms(cuda_lib):
    # a clockwise element
    mesh = uniform_rectangle(0.0, 1.0, 0.0, 1.0, 1, 1)
    mesh.elements = mesh.elements[:, ::-1].copy()
    status, _, msg = check(cuda_lib, SWEDeviceForm2D(mesh=mesh, order=2))
    assert status == abi.ERR_INVALID and "Jacobian" in msg
    # a boundary tag without a condition
    form = SWEDeviceForm2D(mesh=uniform_rectangle(0.0, 1.0, 0.0, 1.0, 2, 2,
                                                  sides=(TAG_WALL, TAG_WALL, TAG_WALL, TAG_OPEN)),
                           order=2)
    status, _, msg = check(cuda_lib, form)
    assert status == abi.ERR_INVALID and "tagged 1" in msg
    form.boundaries[TAG_OPEN] = TidalBoundary([])
    assert check(cuda_lib, form)[0] == abi.OK
    # an order the device does not run
    assert check(cuda_lib, SWEDeviceForm2D(mesh=uniform_rectangle(0, 1, 0, 1, 1, 1), order=5))[0] \
        == abi.ERR_UNSUPPORTED
    # three elements on one edge
    mesh = uniform_rectangle(0.0, 2.0, 0.0, 1.0, 2, 1)
    mesh.vertices = np.vstack([mesh.vertices, [[1.5, 0.5], [1.5, 0.7]]])
    mesh.elements = np.vstack([mesh.elements, [[4, 1, 6, 7]]])
    mesh.face_tags = np.zeros((3, 4), np.int32)
    status, _, msg = check(cuda_lib, SWEDeviceForm2D(mesh=mesh, order=1))
    assert status == abi.ERR_INVALID


def test_check_form_of_the_workloads(cuda_lib):
    case = cases.tidal_channel()
    status, info, _ = check(cuda_lib, case.form)
    assert status == abi.OK and info.n_elements == 4000 and info.n_affine == 4000
    assert info.n_boundary_faces == 2 * 200 + 2 * 20
    case = cases.coastal_box(n_elements=20_000, order=3)
    status, info, _ = check(cuda_lib, case.form)
    assert status == abi.OK and info.n_affine < info.n_elements // 10  # jittered: general quads
    assert info.min_jacobian > 0.0
    assert abs(info.area - 200_000.0 * 150_000.0) < 1e-3 * 200_000.0 * 150_000.0


def test_create_without_a_gpu_says_so(cuda_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    form = SWEDeviceForm2D(mesh=uniform_rectangle(0.0, 1.0, 0.0, 1.0, 2, 2), order=2)
    c_form, keep = form.to_c()
    handle = C.c_void_p()
    status = cuda_lib.create(C.byref(c_form), 0, C.byref(handle))
    assert status == abi.ERR_NO_DEVICE
    assert "no CUDA device" in cuda_lib.last_error(handle).decode()
    cuda_lib.destroy(handle)


def test_ensemble_create_checks_the_members_before_the_device():
    """Members must share every physics option but the mesh, bed, Manning
    and boundary data; the check needs no GPU."""
    import ctypes as C

    from dgcom_gb300 import cases

    lib = abi.cuda_library()
    a = cases.tidal_channel(nx=4, ny=2)
    b = cases.tidal_channel(nx=6, ny=2, order=3)
    b.form.manning_n = 0.03
    keep = []
    forms = (abi.Form * 2)()
    for i, c in enumerate((a, b)):
        f, k = c.form.to_c()
        forms[i] = f
        keep.append(k)
    handle = C.c_void_p()
    status = lib.ensemble_create(forms, 2, 0, C.byref(handle))
    # the same physics: only the device can refuse (no GPU here), or it runs
    assert status in (abi.OK, abi.ERR_NO_DEVICE)
    lib.ensemble_destroy(handle)
    c2 = cases.tidal_channel(nx=6, ny=2)
    c2.form.h_min = 2e-6
    f, k = c2.form.to_c()
    forms[1] = f
    keep.append(k)
    handle = C.c_void_p()
    status = lib.ensemble_create(forms, 2, 0, C.byref(handle))
    assert status == abi.ERR_INVALID
    assert b"physics options differ" in lib.ensemble_last_error(handle)
    lib.ensemble_destroy(handle)
    assert lib.ensemble_create(forms, 0, 0, C.byref(handle)) == abi.ERR_INVALID
    lib.ensemble_destroy(handle)
