"""The C ABI library loads, exports every symbol include/bpm_gb300.h declares, and
validates its arguments on the host (no kernel launches: these run without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bpm_gb300.h")


@pytest.fixture(scope="module")
def native():
    from bpm_gb300 import build, _native
    build.build(verbose=False)
    return _native


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\*?\s*\**\s*(bpm_\w+|debye_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ["bpm_version", "bpm_plan_create", "bpm_propagate", "debye_focus_field"]:
        assert n in names


def test_library_exports_every_declared_symbol(native):
    L = ctypes.CDLL(native.LIB_PATH)
    for n in header_functions():
        assert hasattr(L, n), n
    assert set(header_functions()) <= set(native.SIGNATURES)


def test_version_and_error_text(native):
    L = native.lib()
    assert L.bpm_version() == 1
    assert isinstance(native.last_error(), str)


def desc(native, **kw):
    d = dict(nx=64, ny=32, nz=8, dx=.1, dy=.1, dz=.1, lam=.5, n0=1.33, absorbing_width=0,
             mean_mode=2, prop_kind=0, use_fresnel_approx=0)
    d.update(kw)
    return native.GridDesc(**d)


@pytest.mark.parametrize("kw,code", [
    (dict(), 0),
    (dict(nx=100), -2), (dict(ny=8), -2), (dict(nx=2048), -2), (dict(nz=0), -2),
    (dict(dx=0.), -1), (dict(lam=-1.), -1), (dict(n0=0.), -1), (dict(absorbing_width=-1), -1),
    (dict(mean_mode=7), -2), (dict(prop_kind=3), -1),
])
def test_grid_check(native, kw, code):
    rc = native.lib().bpm_grid_check(ctypes.byref(desc(native, **kw)))
    assert rc == code
    if code:
        assert native.last_error()


def test_status_to_exception(native):
    with pytest.raises(NotImplementedError):
        native.check(native.BPM_ERR_SHAPE)
    with pytest.raises(ValueError):
        native.check(native.BPM_ERR_ARG)
    with pytest.raises(MemoryError):
        native.check(native.BPM_ERR_OOM)
    with pytest.raises(RuntimeError):
        native.check(native.BPM_ERR_CUDA)


def test_debye_workspace_rejects_bad_shapes(native):
    na = (ctypes.c_double * 2)(0., .8)
    d = native.DebyeDesc(16, 16, 15, .1, .1, .1, .5, 1., ctypes.cast(na, ctypes.POINTER(ctypes.c_double)),
                         2, 50, 1., 0.)
    assert native.lib().debye_workspace_bytes(ctypes.byref(d)) == 0
    d.nz = 16
    assert native.lib().debye_workspace_bytes(ctypes.byref(d)) > 0
    d.n_integration_steps = 1
    assert native.lib().debye_workspace_bytes(ctypes.byref(d)) == 0


def test_null_plan_calls(native):
    L = native.lib()
    assert L.bpm_workspace_bytes(None, 1, 0) == 0
    assert L.bpm_propagate(None, None, None, 0, None) == native.BPM_ERR_ARG
    assert L.bpm_plan_destroy(None) == 0
    assert L.bpm_exec_destroy(None) == 0


def test_autotune_pick_group():
    """The tuner keeps the largest group within 3 % of the fastest probe time."""
    from bpm_gb300.autotune import pick_group
    assert pick_group({1: 10., 2: 8., 4: 7.9, 8: 7.95, 16: 9.}) == 8
    assert pick_group({4: 7.0, 8: 7.5, 16: 7.6}) == 4
    assert pick_group({8: 5.}) == 8
    assert pick_group({2: 3., 4: 3.09}, tol=.03) == 4


def test_psf_request_footprint_covers_the_workspace(native):
    """The serving loop admits a PSF request by its footprint: never less than the
    library's workspace plus the outputs; a request the library rejects still gets one."""
    from bpm_gb300.psf import _desc
    from bpm_gb300.serve import PsfRequest
    for shape, NA, steps, field in (((128, 128, 128), .8, 200, True), ((256, 256, 256), 1.1, 512, False),
                                    ((130, 96, 200), [.2, .5, .6, .9], 100, True), ((16, 16, 16), .5, 20, False)):
        desc, _na = _desc(shape, (.1, .1, .1), .5, NA, 1.33, steps)
        ws = native.lib().debye_workspace_bytes(ctypes.byref(desc))
        out = shape[0] * shape[1] * shape[2] * (28 if field else 4)
        assert ws > 0
        assert PsfRequest(shape, (.1, .1, .1), .5, NA, 1.33, steps, return_field=field).footprint() == ws + out
    assert PsfRequest((15, 16, 16), (.1, .1, .1)).footprint() > 0          # odd shape: rejected at launch
    assert PsfRequest((16, 16, 16), (.1, .1, .1), NA=[.1, .2, .3]).footprint() > 0


def test_mask_policy():
    """Phase masks are precomputed for several fields through one dn, and for one field
    from 64 x 64 points up."""
    from bpm_gb300.bpm3d import mask_pays
    assert mask_pays(2, 64, 32) and mask_pays(2, 16, 16) and mask_pays(64, 512, 512)
    assert mask_pays(1, 512, 512) and mask_pays(1, 1024, 256) and mask_pays(1, 1024, 1024)
    assert mask_pays(1, 256, 256) and mask_pays(1, 512, 256) and mask_pays(1, 64, 64)
    assert not mask_pays(1, 32, 64) and not mask_pays(1, 16, 16)


def test_serve_request_keys_and_footprint():
    """Requests merge into one launch when grid, physics, dn kind and output form agree
    (each field may bring its own dn); the admission footprint counts u0, last plane and
    workspace plane, the dn volume, its phase masks and the output volume."""
    import numpy as np
    from bpm_gb300.serve import BpmRequest
    size, units = (64, 32, 8), (.1, .1, .1)
    dn = np.zeros((8, 32, 64), np.float32)
    a = BpmRequest(size, units, dn=dn)
    assert a.key() == BpmRequest(size, units, dn=dn.copy()).key()
    for other in (BpmRequest(size, units, lam=.6, dn=dn), BpmRequest(size, units, n0=1.33, dn=dn),
                  BpmRequest(size, units, dn=dn.astype(np.complex64)), BpmRequest(size, units),
                  BpmRequest(size, units, dn=dn, mean_mode="ignore"), BpmRequest(size, units, dn=dn, return_field=True),
                  BpmRequest((64, 32, 9), units, dn=np.zeros((9, 32, 64), np.float32))):
        assert other.key() != a.key()
    plane = 64 * 32
    assert a.voxel_updates() == plane * 7
    assert a.footprint() == plane * 8 * 3 + 8 * plane * 4 + 8 * plane * 8 + 8 * plane * 4
    assert BpmRequest(size, units, dn=dn.astype(np.complex64)).footprint() - a.footprint() == 8 * plane * 4
    assert BpmRequest(size, units, dn=dn, return_field=True).footprint() - a.footprint() == 8 * plane * 4
    assert BpmRequest(size, units, return_full=False).footprint() == plane * 8 * 3


def test_serve_overlap_count():
    """The server's count of launches whose device intervals overlap another's."""
    from bpm_gb300.serve import overlapped
    assert overlapped([]) == 0
    assert overlapped([(0., 1.), (1., 2.)]) == 0            # touching intervals do not overlap
    assert overlapped([(0., 2.), (1., 3.), (4., 5.)]) == 2
    assert overlapped([(0., 10.), (1., 2.), (3., 4.), (11., 12.)]) == 3


def test_autotune_shape_choices():
    """The launch-shape search: an option replaces the current choice only when more than 3 %
    faster; the choices offered depend on the grid, the number of groups and the mode."""
    from bpm_gb300.autotune import pick_option, shape_candidates
    assert pick_option(0, 10., {1: 9.8, 2: 9.9}) == (0, 10.)          # within 3 %: keep
    assert pick_option(0, 10., {1: 9.0, 8: 9.5}) == (1, 9.0)
    c = shape_candidates((512, 512), 64, 8, "weighted")
    assert c == {"conc": [1, 2, 4, 8], "col_fuse": [1, 2]}             # weighted passes keep 16 columns
    c = shape_candidates((256, 256), 4, 4, "ignore")
    assert c == {"col_block": [4, 8, 16], "cluster": [1, 2]}              # one group: no concurrency choice
    assert "cluster" not in shape_candidates((512, 256), 8, 2, "ignore")
