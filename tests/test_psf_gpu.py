"""Parity of the CUDA Debye-Wolf focus field with the reference (golden vectors from the
reference's own kernel) and with the FP64 oracle. Tolerance: relative L2 <= 1e-4."""
import numpy as np
import pytest

from conftest import PSF_GOLDEN, debye_point_fp64, golden_psf_case, rel_l2
from oracle import debye_ref

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    return bpm_gb300


@pytest.mark.parametrize("name", PSF_GOLDEN)
def test_golden_reference_kernel(bpm, golden, name):
    c = golden_psf_case(golden, name)
    u, ex, ey, ez = bpm.psf(c["shape"], c["units"], c["lam"], c["NA"], c["n0"], c["steps"], return_field=True)
    assert u.shape == c["u"].shape and u.dtype == np.float32 and ex.dtype == np.complex64
    for a, k in zip((u, ex, ey, ez), ("u", "ex", "ey", "ez")):
        assert rel_l2(a, c[k]) < TOL, k


@pytest.mark.parametrize("shape,units,lam,NA,n0,steps", [
    ((64, 64, 64), (.1, .1, .1), .5, 1.1, 1.33, 200),
    ((96, 64, 32), (.05, .08, .1), .488, .8, 1.0, 100),
    ((128, 128, 64), (.1, .1, .1), .5, [.2, .4, .6, .8], 1.33, 64),
    ((2, 2, 2), (.1, .1, .1), .5, .5, 1.0, 20),
])
def test_oracle_parity(bpm, shape, units, lam, NA, n0, steps):
    u, ex, ey, ez = bpm.focus_field_debye(shape, units, lam, NA, n0, steps)
    o = debye_ref.focus_field_debye(shape, units, lam, NA, n0, steps,
                                    real_dtype=np.float64, complex_dtype=np.complex128)
    for a, b, k in zip((u, ex, ey, ez), o, ("u", "ex", "ey", "ez")):
        assert rel_l2(a, b) < TOL, k


def test_config2_psf_256(bpm):
    """256^3 vectorial PSF, NA 1.1, n0 1.33, lam 0.5, x-polarised, 512 steps: the intensity
    agrees with the FP64 oracle on a set of full-resolution slices."""
    shape = (256, 256, 256)
    u, ex, ey, ez = bpm.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 512, return_field=True)
    params = debye_ref.octant_params(shape, (.1, .1, .1), .5, 1.1, 1.33)
    octant = debye_ref.debye_octant(params, 512)
    c = 128
    # full index c + k (k >= 1 along z, >= 0 along x, y) holds octant sample k, unconjugated
    for a, b, k in zip((u, ex, ey, ez), octant, ("u", "ex", "ey", "ez")):
        print("psf 256^3 %s: relative L2 %.2e against the FP64 oracle" % (k, rel_l2(a[c + 1:, c:, c:], b[1:c, :c, :c])))
        assert rel_l2(a[c + 1:, c:, c:], b[1:c, :c, :c]) < TOL, k
        # full index m <= c holds octant sample c - m, conjugated: index 0 is the octant's
        # last plane (z = 12.8 um), the one the plane-remainder kernel computes
        assert rel_l2(a[:c, c:, c:], np.conj(b[c:0:-1, :c, :c])) < TOL, k
        # that plane alone is far from focus, where the node sum cancels more: 1e-3
        assert rel_l2(a[0, c:, c:], np.conj(b[c, :c, :c])) < 1e-3, k
    assert np.all(np.isfinite(u))
    u_only = bpm.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 512)
    assert np.array_equal(u_only, u)


def test_psf_u0_matches_oracle(bpm):
    a = bpm.psf_u0((256, 256), (.1, .1), zfoc=12.8, NA=.4, lam=.5, n0=1.33)
    b = debye_ref.psf_u0((256, 256), (.1, .1), zfoc=12.8, NA=.4, lam=.5, n0=1.33)
    assert a.shape == (256, 256) and a.dtype == np.complex64
    assert rel_l2(a, b) < TOL


def test_psf_lightsheet_matches_oracle(bpm):
    a = bpm.psf_lightsheet((32, 32, 32), (.1, .1, .1), .5, .2, .5, .8, n0=1.33, n_integration_steps=50)
    b = debye_ref.psf_lightsheet((32, 32, 32), (.1, .1, .1), .5, .2, .5, .8, n0=1.33, n_integration_steps=50)
    assert rel_l2(a, b) < TOL


def test_psf_errors(bpm):
    with pytest.raises(NotImplementedError):
        bpm.psf((16, 16, 15), (.1, .1, .1), .5, .8)
    with pytest.raises(AssertionError):
        bpm.psf((16, 16, 16), (.1, .1, .1), .5, [.1, .2, .3])


# --- variants: Gaussian pupil, single plane, arbitrary points ---------------------------

@pytest.mark.parametrize("name", ["gauss_a", "gauss_b"])
def test_gauss_golden_reference_kernel(bpm, golden, name):
    a = golden[name + "_args"]
    shape = tuple(int(v) for v in a[:3])
    res = bpm.focus_field_debye_gauss(shape, tuple(a[3:6]), a[6], list(golden[name + "_NA"]), a[7], int(a[8]))
    for v, k in zip(res, ("u", "ex", "ey", "ez")):
        assert v.shape == shape[::-1]
        assert rel_l2(v, golden["%s_%s" % (name, k)]) < TOL, k


@pytest.mark.parametrize("shape,units,lam,NAs,sig,steps", [
    ((64, 48, 33), (.1, .1, .1), .5, [0., .9], 1. / np.sqrt(2), 200),
    ((101, 64, 40), (.08, .1, .15), .488, [.3, .5, .7, .95], .5, 128),
])
def test_gauss_oracle_parity(bpm, shape, units, lam, NAs, sig, steps):
    res = bpm.focus_field_debye_gauss(shape, units, lam, NAs, sig, steps)
    o = debye_ref.focus_field_debye_gauss(shape, units, lam, NAs, sig, steps)
    for v, b, k in zip(res, o, ("u", "ex", "ey", "ez")):
        assert rel_l2(v, b) < TOL, k


@pytest.mark.parametrize("name", ["plane_a", "plane_b"])
def test_plane_golden_reference_kernel(bpm, golden, name):
    Nx, Ny, dx, dy, z, lam, NA, n0, steps = golden[name + "_args"]
    ex = bpm.focus_field_debye_plane((int(Nx), int(Ny)), (dx, dy), z, lam, NA, n0, n_integration_steps=int(steps))
    assert ex.shape == (int(Ny), int(Nx)) and ex.dtype == np.complex64
    assert rel_l2(ex, golden[name + "_ex"]) < TOL


@pytest.mark.parametrize("shape,z,NA,n0", [((256, 256), 0., 1.1, 1.33), ((200, 120), 3.7, .8, 1.),
                                           ((64, 64), -2.5, [.2, .4, .6, .8], 1.)])
def test_plane_oracle_parity(bpm, shape, z, NA, n0):
    ex = bpm.focus_field_debye_plane(shape, (.1, .1), z, .5, NA, n0, n_integration_steps=150)
    o = debye_ref.focus_field_debye_plane(shape, (.1, .1), z, .5, NA, n0, 150)
    assert rel_l2(ex, o) < TOL


def test_plane_fills_buffer(bpm):
    import torch
    buf = torch.zeros((24, 32), dtype=torch.complex64, device="cuda")
    assert bpm.focus_field_debye_plane((32, 24), (.1, .1), 1., .5, .8, ex_g=buf) is None
    ref = bpm.focus_field_debye_plane((32, 24), (.1, .1), 1., .5, .8)
    assert np.array_equal(buf.cpu().numpy(), ref)


def test_at_golden_reference_kernel(bpm, golden):
    p = golden["at_a_pts"]
    lam, n0, steps = golden["at_a_args"]
    res = bpm.focus_field_debye_at(p[0], p[1], p[2], lam, list(golden["at_a_NA"]), n0, int(steps))
    for v, k in zip(res, ("u", "ex", "ey", "ez")):
        assert v.shape == p[0].shape
        assert rel_l2(v, golden["at_a_" + k]) < TOL, k


def test_at_oracle_parity_and_grid_consistency(bpm):
    """Random points, including far from focus (large kz cos t phases), against the FP64
    oracle; and the grid samples of focus_field_debye re-evaluated as free points."""
    import torch
    rng = np.random.default_rng(7)
    x, y = rng.uniform(-3, 3, (2, 4000)).astype(np.float32)
    z = rng.uniform(-40, 40, 4000).astype(np.float32)
    res = bpm.focus_field_debye_at(x, y, z, .5, 1.1, 1.33, 200)
    o = debye_ref.focus_field_debye_at(x, y, z, .5, 1.1, 1.33, 200)
    for v, b, k in zip(res, o, ("u", "ex", "ey", "ez")):
        assert rel_l2(v, b) < TOL, k
    # torch inputs on the device, device outputs
    t = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    res_d = bpm.focus_field_debye_at(*t, .5, 1.1, 1.33, 200, device=True)
    assert res_d[1].is_cuda and np.array_equal(res_d[1].cpu().numpy(), res[1])


def test_variant_errors(bpm):
    with pytest.raises(NotImplementedError):
        bpm.focus_field_debye_gauss((2, 16, 16), (.1, .1, .1), .5, [0., .8])
    with pytest.raises(AssertionError):
        bpm.focus_field_debye_gauss((16, 16, 16), (.1, .1, .1), .5, [0., .8], sig=0.)
    with pytest.raises(NotImplementedError):
        bpm.focus_field_debye_plane((1, 16), (.1, .1), 0., .5, .8)
    with pytest.raises(AssertionError):
        bpm.focus_field_debye_at(np.zeros(3), np.zeros(3), np.zeros(4), .5, .8)
    u, ex, ey, ez = bpm.focus_field_debye_at(np.zeros(0), np.zeros(0), np.zeros(0), .5, .8)
    assert u.shape == (0,)


def test_tensor_core_quadrature_matches_fma(bpm, tmp_path):
    """The octant quadrature as a 3xTF32 tensor-core product (tcgen05, TMA-staged operands,
    the default) against the FP32 FMA kernels (BPM_GB300_DEBYE=fma), each in a child
    process: symmetric octants (radius rows deduplicated) and non-square ones, annuli, the
    Gaussian pupil with odd shapes, the 256^3 PSF of the single-request configuration. Both
    evaluate the same node tables; the sums differ only by rounding (relative L2 < 5e-5 on
    every output; each path is within 1e-4 of the FP64 oracle in the parity tests), and no
    bounded tensor-core wait gave up."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    script = os.path.join(here, "_psf_cases.py")
    a, b = str(tmp_path / "tc.npz"), str(tmp_path / "fma.npz")
    env = {k: v for k, v in os.environ.items() if k != "BPM_GB300_DEBYE"}
    subprocess.run([sys.executable, script, a], check=True, timeout=600, env=env)
    subprocess.run([sys.executable, script, b], check=True, timeout=600, env=dict(env, BPM_GB300_DEBYE="fma"))
    A, B = np.load(a), np.load(b)
    assert int(A["device_status"][0]) == 0 and int(B["device_status"][0]) == 0
    keys = [k for k in A.files if k != "device_status"]
    assert sorted(keys) == sorted(k for k in B.files if k != "device_status") and len(keys) == 28
    errs = {k: rel_l2(A[k], B[k]) for k in keys}
    print("tensor cores vs FMA, largest relative L2: %s %.2e" % max(errs.items(), key=lambda kv: kv[1]))
    bad = [(k, e) for k, e in errs.items() if not e < 5e-5]
    assert not bad, bad


def test_tensor_core_status_is_clear(bpm):
    """After a PSF on the tensor cores the library's sticky device status is 0 (no bounded
    wait gave up)."""
    from bpm_gb300 import _native as N
    bpm.psf((128, 128, 128), (.1, .1, .1), .5, 1.1, 1.33, 200)
    assert N.lib().bpm_device_status(0) == 0


@pytest.mark.parametrize("n_int", [200, 1000])
def test_physical_quadrature_against_the_debye_integral(bpm, n_int):
    """quadrature="physical" (sin t included, exact trapezoid) against the reference test
    script's own point formula (NA 0.95, lambda 0.5, n0 1, dx 0.008 um as there) along the x
    and y axes near the focus and off the focal plane, and against the oracle's octant;
    relative L2 <= 1e-4. The default rule stays the reference kernel's (no sin t)."""
    NA, lam, dx = .95, .5, .008
    shape = (128, 96, 64)
    u, ex, ey, ez = bpm.psf(shape, (dx,) * 3, lam, NA, 1., n_int, return_field=True, quadrature="physical")
    c = (shape[0] // 2, shape[1] // 2, shape[2] // 2)
    k = 2 * np.pi / lam
    got, want = [], []
    # grid index (cx + i, cy + j, cz + l) sits at (i dx, j dx, l dx) for i, j, l >= 0, l >= 1
    for i, j, l in [(i, 0, 1) for i in range(0, 64, 3)] + [(0, j, 1) for j in range(0, 48, 3)] + \
                   [(i, i // 2, l) for i in range(0, 40, 5) for l in (4, 17, 31)]:
        got.append([ex[c[2] + l, c[1] + j, c[0] + i], ey[c[2] + l, c[1] + j, c[0] + i],
                    ez[c[2] + l, c[1] + j, c[0] + i]])
        want.append(debye_point_fp64(i * dx, j * dx, l * dx, k, NA, n_int))
    got, want = np.array(got), np.array(want)
    for comp in range(3):
        if comp == 1:   # ey vanishes on the axes: compare where it does not
            sel = np.abs(want[:, 1]) > 1e-3 * np.abs(want[:, 0]).max()
            assert rel_l2(got[sel, 1], want[sel, 1]) < TOL
        else:
            assert rel_l2(got[:, comp], want[:, comp]) < TOL, comp
    o = debye_ref.focus_field_debye(shape, (dx,) * 3, lam, NA, 1., n_int, real_dtype=np.float64,
                                    complex_dtype=np.complex128, quadrature="physical")
    for a, b, name in zip((u, ex, ey, ez), o, ("u", "ex", "ey", "ez")):
        assert rel_l2(a, b) < TOL, name
    ref = bpm.psf(shape, (dx,) * 3, lam, NA, 1., n_int)
    assert rel_l2(ref, u) > 1e-2          # the reference rule (no sin t) is another PSF
    with pytest.raises(ValueError):
        bpm.psf(shape, (dx,) * 3, lam, NA, 1., n_int, quadrature="midpoint")


def test_tensor_core_wait_runs_out_and_reports(bpm):
    """A bounded wait of the tensor-core quadrature that cannot be met (its loads announce 16
    bytes that never arrive, debye_tc_timeout_selftest) gives up after 20 ms and reports
    BPM_ERR_TIMEOUT through the device status; the context stays usable: a PSF afterwards
    is correct and leaves the status clear."""
    import time
    from bpm_gb300 import _native as N
    t0 = time.perf_counter()
    assert N.lib().debye_tc_timeout_selftest(20.) == N.BPM_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30
    assert N.lib().bpm_device_status(0) == 0
    shape = (32, 32, 32)
    u = bpm.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 100)
    o = debye_ref.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 100)
    assert rel_l2(u, o) < TOL
    assert N.lib().bpm_device_status(0) == 0


@pytest.mark.parametrize("shape", [(64, 48, 32), (128, 96, 64)])
def test_assembly_forms_agree(bpm, shape):
    """The two forms of the full-volume assembly give the same bits: the gather form (16-byte
    aligned field buffers of even nx: paired stores) and the scatter form (one octant sample
    per thread to its mirrored voxels: taken here by field buffers 8 bytes off a 16-byte
    boundary, and by the intensity alone). Odd shapes (Gaussian pupil) take the scatter form
    and are checked against the reference kernel's goldens above."""
    import ctypes
    import torch
    from bpm_gb300 import _native as N
    from bpm_gb300.bpm3d import _ptr, _stream_ptr
    from bpm_gb300.psf import _desc
    Nx, Ny, Nz = shape
    desc, _na = _desc(shape, (.1, .1, .1), .5, .9, 1.33, 100)
    L = N.lib()
    wsb = int(L.debye_workspace_bytes(ctypes.byref(desc)))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    n = Nx * Ny * Nz

    def run(off, fields=True):
        u = torch.empty(n, dtype=torch.float32, device="cuda")
        bufs = [torch.zeros(n + 1, dtype=torch.complex64, device="cuda") for _ in range(3)]
        f = [b[off:off + n] for b in bufs] if fields else [None] * 3
        N.check(L.debye_focus_field(ctypes.byref(desc), _ptr(u), *(_ptr(t) for t in f), _ptr(ws), wsb,
                                    _stream_ptr()), "debye_focus_field")
        torch.cuda.synchronize()
        return [u] + [t for t in f if t is not None]

    gathered, scattered = run(0), run(1)
    assert scattered[1].data_ptr() % 16 == 8
    for a, b in zip(gathered, scattered):
        assert torch.equal(a, b)
    assert torch.equal(run(0, fields=False)[0], gathered[0])
