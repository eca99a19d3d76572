"""Physical checks of the split-step march and the Debye-Wolf field, on the oracle (CPU,
FP64 and FP32). The reference's own test scripts make these comparisons by eye
(tests/test_gaussian.py, test_energy.py, test_refraction.py, test_single_focus.py,
test_focus_reflect.py, test_psf.py, test_psf_vectorial.py); here each one asserts a bound. The CUDA path is held
to the oracle at 1e-4 by the GPU parity tests, so these bounds carry over to it."""
import numpy as np
import pytest
from scipy.special import jn

from conftest import rel_l2
from oracle import bpm_ref, debye_ref


def gaussian_beam(x, y, z, lam, NA):
    """Paraxial Gaussian beam with waist lam / (pi asin NA) at z = 0, in bpm_3d's phase
    convention exp(-i k z) (the form of tests/test_gaussian.py)."""
    r2 = x ** 2 + y ** 2
    k = 2 * np.pi / lam
    w0 = lam / np.pi / np.arcsin(NA)
    zr = np.pi * w0 ** 2 / lam
    w = w0 * np.sqrt(1 + (z / zr) ** 2)
    R = z * (1 + (zr / z) ** 2)
    return w0 / w * np.exp(-r2 / w ** 2) * np.exp(-1j * (k * z + k * r2 / 2. / R - np.arctan(z / zr)))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gaussian_beam_free_space(precision):
    """A Gaussian beam started at z = -Nz dz / 2 and marched through free space follows the
    paraxial formula, the closer the smaller its NA (the formula's error grows as NA^4)."""
    errs = []
    for (Nx, Ny, Nz), (dx, dy, dz), NA in (((128, 128, 128), (.2, .2, .2), .1),
                                          ((64, 128, 96), (.2, .1, .1), .15)):
        x = dx * (np.arange(-Nx / 2, Nx / 2) + .5)
        y = dy * (np.arange(-Ny / 2, Ny / 2) + .5)
        z = dz * (np.arange(-Nz / 2, Nz / 2) + .5)
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        ua = gaussian_beam(X, Y, Z, .5, NA)
        u = bpm_ref.bpm_3d((Nx, Ny, Nz), (dx, dy, dz), lam=.5, n0=1., u0=ua[0].astype(np.complex64),
                           precision=precision)
        errs.append(rel_l2(u, ua))
    assert errs[0] < .005 and errs[1] < .01, errs     # observed 0.0029 and 0.0056
    assert errs[0] < errs[1]


@pytest.mark.parametrize("mode", ["ignore", "simple", "weighted"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_energy_never_grows(mode, precision):
    """Real dn and no absorbing taper: the propagator has modulus <= 1 (0 past the
    evanescent cut), the phase mask modulus 1 and the FFT pair is unitary up to its
    1/(Nx Ny), so sum |u|^2 cannot grow from one plane to the next; over smooth dn it
    barely falls."""
    Nx, Ny, Nz = 64, 32, 40
    rng = np.random.default_rng(11)
    dn = (.05 * rng.uniform(-1, 1, (Nz, Ny, Nx))).astype(np.float32)
    x = .1 * np.arange(Nx)
    # a frequency of the grid (3 periods across it): no spectral leakage past the
    # evanescent cut, which would take energy out in the first step
    u0 = np.exp(-1j * 2 * np.pi * 3 / (Nx * .1) * x)[None, :].repeat(Ny, 0).astype(np.complex64)
    I = bpm_ref.bpm_3d((Nx, Ny, Nz), (.1, .1, .1), lam=.5, n0=1.33, u0=u0, dn=dn, mean_mode=mode,
                       return_field=False, precision=precision)
    E = I.reshape(Nz, -1).sum(1).astype(np.float64)
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert np.all(E[1:] <= E[:-1] * (1 + tol)), np.diff(E) / E[:-1]
    assert E[-1] > .9 * E[0]
    # the same march through the uniform dn mean keeps the energy to rounding
    I0 = bpm_ref.bpm_3d((Nx, Ny, Nz), (.1, .1, .1), lam=.5, n0=1.33, u0=u0, mean_mode=mode,
                        return_field=False, precision=precision)
    E0 = I0.reshape(Nz, -1).sum(1).astype(np.float64)
    assert np.allclose(E0, E0[0], rtol=10 * tol, atol=0)


@pytest.mark.parametrize("mode", ["ignore", "simple", "weighted"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_refraction_in_a_uniform_medium(mode, precision):
    """A tilted plane wave in a medium of index n0 + dn keeps its transverse wavenumber kx
    and advances exp(-i kz dz) per step. With the mean-index correction (simple and
    weighted modes) the propagator runs at n0 + dn, so kz = sqrt((n0 + dn)^2 k0^2 - kx^2):
    Snell's law in the refracted medium. Without it (ignore) the step splits into the
    free-space propagator at n0 and the phase mask: kz = sqrt(n0^2 k0^2 - kx^2) + k0 dn."""
    Nx, Ny, Nz = 64, 16, 30
    dx = dz = .1
    lam, n0, dnv = .5, 1.33, .05
    k0 = 2 * np.pi / lam
    kx = 2 * np.pi * 9 / (Nx * dx)      # a frequency of the grid: an exact mode of the march
    x = dx * np.arange(Nx)
    u0 = np.exp(-1j * kx * x)[None, :].repeat(Ny, 0).astype(np.complex64)
    dn = np.full((Nz, Ny, Nx), dnv, np.float32)
    u = bpm_ref.bpm_3d((Nx, Ny, Nz), (dx, dx, dz), lam=lam, n0=n0, u0=u0, dn=dn, mean_mode=mode,
                       precision=precision)
    if mode == "ignore":
        kz = np.sqrt((n0 * k0) ** 2 - kx ** 2) + k0 * float(np.float32(dnv))
    else:
        kz = np.sqrt(((n0 + float(np.float32(dnv))) * k0) ** 2 - kx ** 2)
    want = u0[None] * np.exp(-1j * kz * dz * np.arange(Nz))[:, None, None]
    # the FP64 flavour still takes the reference's float32 inputs (dn, simple mode's dn0 as a
    # float32 mean): observed up to 3e-7
    assert rel_l2(u, want) < (2e-6 if precision == "fp64" else 1e-4)
    # the refracted direction: sin(theta) = kx / kz' scales as 1 / n
    if mode != "ignore":
        th0 = np.arcsin(kx / (n0 * k0))
        th1 = np.arctan(kx / kz)
        assert np.isclose(n0 * np.sin(th0), (n0 + dnv) * np.sin(th1), rtol=1e-6)


def test_bpm_carries_the_debye_focus():
    """The two hot paths agree: marching the Debye field of the first plane with the
    split-step propagator reproduces the Debye field of every later plane (each quadrature
    node is a cone of plane waves with kz = k cos t). The Debye kernel's phase is
    exp(+i k z cos t) and bpm_3d's exp(-i k z), so the march takes conjugated fields:
    conj(psf_u0) focuses zfoc downstream in bpm_3d, psf_u0 itself (as in the reference)
    moves away from the focus."""
    for size, units, lam, NA, n0, err in (((64, 64, 64), (.1, .1, .1), .5, .3, 1., .05),
                                          ((128, 128, 64), (.1, .1, .1), .5, .5, 1.33, .025)):
        _, ex, _, _ = debye_ref.focus_field_debye(size, units, lam, NA, n0, 200, real_dtype=np.float64,
                                                  complex_dtype=np.complex128)
        u0 = debye_ref.psf_u0(size[:2], units[:2], zfoc=.5 * units[2] * size[2], NA=NA, lam=lam, n0=n0)
        assert rel_l2(u0, ex[0]) < 1e-6
        u = bpm_ref.bpm_3d(size, units, lam=lam, n0=n0, u0=np.conj(u0), precision="fp64")
        assert rel_l2(u, np.conj(ex)) < err, size      # observed 0.038, 0.017
        assert rel_l2(np.abs(u) ** 2, np.abs(ex) ** 2) < err / 2, size
        away = bpm_ref.bpm_3d(size, units, lam=lam, n0=n0, u0=u0, precision="fp64")
        assert rel_l2(np.abs(away[-1]) ** 2, np.abs(ex[-1]) ** 2) > .3


def _airy(r, lam, NA):
    v = 2. * np.pi * NA / lam * np.abs(r)
    safe = np.where(v > 1e-12, v, 1.)
    return np.where(v > 1e-12, (2 * jn(1, safe) / safe) ** 2, 1.)


@pytest.mark.parametrize("NA,n0", [(.1, 1.), (.2, 1.), (.2, 1.3), (.4, 1.)])
def test_focal_plane_and_the_airy_disk(NA, n0):
    """The scalar limit of tests/test_psf.py, in the focal plane. The plane kernel
    (debye_wolf_plane) weights its nodes with sqrt(cos t) sin t, the aperture's area
    element, and its intensity is the Airy disk (2 J1(v)/v)^2 within 1.2 %. The octant
    kernel behind psf (debye_wolf) drops sin t (psf_debye.cl:77-78), which weighs the small
    angles more: its focal plane departs from the Airy disk by 15 % or more. Both are the
    reference's behaviour and both are kept."""
    N, dx, lam = 64, .05, .5
    ex = debye_ref.focus_field_debye_plane((N, N), (dx, dx), z=0., lam=lam, NA=NA, n0=n0)
    x = -(N // 2) * dx + np.arange(N) * (N * dx) / (N - 1)   # the plane kernel's grid
    Y, X = np.meshgrid(x, x, indexing="ij")
    I, th = np.abs(ex) ** 2, _airy(np.hypot(X, Y), lam, NA)
    assert rel_l2(I, th * (I * th).sum() / (th * th).sum()) < .012       # observed 0.004-0.011
    u = debye_ref.psf((N, N, 8), (dx, dx, .1), lam, NA, n0=n0)[4]        # focal plane, index N/2
    xo = dx * (np.arange(N) - N // 2)
    Yo, Xo = np.meshgrid(xo, xo, indexing="ij")
    tho = _airy(np.hypot(Xo, Yo), lam, NA)
    assert rel_l2(u, tho * (u * tho).sum() / (tho * tho).sum()) > .1      # observed 0.14-0.31


@pytest.mark.parametrize("n0", [1., 1.3, 1.5])
def test_axial_profile_scalar_limit(n0):
    """tests/test_psf.py's axial profile: at NA 0.2 the on-axis intensity of psf follows
    the scalar paraxial form 16 sin^2(u/4) / u^2, u = 2 pi NA^2 z / (lam n0)."""
    Nx, Ny, Nz, dx, lam, NA = 64, 64, 256, .05, .5, .2
    u = debye_ref.psf((Nx, Ny, Nz), (dx,) * 3, lam, NA, n0=n0)
    prof = u[:, Ny // 2, Nx // 2] / u.max()
    z = dx * (np.arange(Nz) - Nz // 2)
    a = 2. * np.pi / lam * NA ** 2 / n0 * z
    safe = np.where(a != 0, a, 1.)
    theory = np.where(a != 0, 16. / safe ** 2 * np.sin(safe / 4.) ** 2, 1.)
    assert np.argmax(u) == np.ravel_multi_index((Nz // 2, Ny // 2, Nx // 2), u.shape)
    assert np.sqrt(np.mean((prof - theory / theory.max()) ** 2)) < .015   # observed 0.004-0.009


def _debye_trapezoid(x, y, z, k, NA, n_int=4001):
    """The vectorial Debye integral of an x-polarised aperture (sqrt(cos t) apodisation, area
    element sin t) by the trapezoid rule on n_int nodes over [0, asin NA], in FP64."""
    a = np.arcsin(NA)
    t = np.linspace(0., a, n_int)
    dt = a / (n_int - 1.)
    kr = k * np.hypot(x, y)[:, None]
    phi = np.arctan2(y, x)
    c, s = np.cos(t), np.sin(t)
    e = np.exp(1j * k * z[:, None] * c)

    def trap(f):
        return dt * (f.sum(1) - .5 * (f[:, 0] + f[:, -1]))
    I0 = trap(np.sqrt(c) * s * (c + 1) * jn(0, kr * s) * e)
    I1 = trap(np.sqrt(c) * s ** 2 * jn(1, kr * s) * e)
    I2 = trap(np.sqrt(c) * s * (c - 1) * jn(2, kr * s) * e)
    return I0 + I2 * np.cos(2 * phi), I2 * np.sin(2 * phi), -2j * I1 * np.cos(phi)


@pytest.mark.parametrize("NA", [.5, .95])
def test_free_points_match_an_independent_quadrature(NA):
    """tests/test_psf_vectorial.py: the free-point kernel (debye_wolf_at) against the Debye
    integral evaluated independently on a fine trapezoid grid. Its nodes run one step past
    the aperture edge (i = 0..INT_STEPS with dt = (a2 - a1) / (INT_STEPS - 1)), so the fields
    agree to O(1 / INT_STEPS). Its intensity output is |ex|^2 alone, as the reference kernel
    writes it (psf_debye.cl:267)."""
    rng = np.random.default_rng(3)
    x, y = (rng.uniform(-1, 1, 200).astype(np.float32) for _ in range(2))
    z = rng.uniform(-1.5, 1.5, 200).astype(np.float32)
    want = _debye_trapezoid(x.astype(np.float64), y.astype(np.float64), z.astype(np.float64),
                            2 * np.pi / .5, NA)
    errs = []
    for steps in (200, 1000):
        u, ex, ey, ez = debye_ref.focus_field_debye_at(x, y, z, .5, NA, n0=1., n_integration_steps=steps)
        e = [rel_l2(g, w) for g, w in zip((ex, ey, ez), want)]
        assert max(e) < 10. / steps, (steps, e)      # observed at most 5 / steps
        errs.append(max(e))
        assert np.allclose(u, np.abs(ex) ** 2, rtol=1e-5, atol=0)
    assert errs[1] < errs[0] / 3


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_absorbing_boundary(precision):
    """tests/test_focus_reflect.py's absorbing layer: the taper 0.5 (1 - cos(pi d / w)) is 0
    at the grid's edge (d = 0), so every plane after u0 has its outermost ring at exactly 0,
    and a beam spreading from focus loses energy into the layer instead of wrapping round
    the periodic grid. Complex dn takes no taper (bpm_3d_kernels.cl:174-195)."""
    N, Nz, w = 64, 48, 8
    _, ex, _, _ = debye_ref.focus_field_debye((N, N, 2), (.1, .1, .1), .5, .7, 1., 100)
    u0 = ex[1].astype(np.complex64)                          # the focal plane
    kw = dict(lam=.5, n0=1., u0=u0, precision=precision)
    free = bpm_ref.bpm_3d((N, N, Nz), (.1, .1, .1), dn=np.zeros((Nz, N, N), np.float32), **kw)
    damp = bpm_ref.bpm_3d((N, N, Nz), (.1, .1, .1), dn=np.zeros((Nz, N, N), np.float32),
                          absorbing_width=w, **kw)
    ring = np.ones((N, N), bool)
    ring[1:-1, 1:-1] = False
    assert np.all(damp[1:, ring] == 0)
    E_free = (np.abs(free) ** 2).sum((1, 2))
    E_damp = (np.abs(damp) ** 2).sum((1, 2))
    assert np.all(E_damp[1:] <= E_damp[:-1] * (1 + 1e-6))
    assert E_damp[-1] < .9 * E_free[-1]                      # the spread beam reached the layer
    cplx = bpm_ref.bpm_3d((N, N, Nz), (.1, .1, .1), dn=np.zeros((Nz, N, N), np.complex64),
                          absorbing_width=w, mean_mode="ignore", **kw)
    assert rel_l2(cplx, free) < (1e-12 if precision == "fp64" else 1e-5)


def test_oracle_physical_quadrature_is_the_debye_integral():
    """The oracle's quadrature="physical" octant equals the Debye integral evaluated point by
    point with the reference test script's formula (tests/test_psf_vectorial.py:15-42 there),
    to FP32 grid-coordinate rounding."""
    from conftest import debye_point_fp64, rel_l2
    NA, lam, dx = .95, .5, .008
    shape = (64, 48, 32)
    o = debye_ref.focus_field_debye(shape, (dx,) * 3, lam, NA, 1., 200, real_dtype=np.float64,
                                    complex_dtype=np.complex128, quadrature="physical")
    c, k = (32, 24, 16), 2 * np.pi / lam
    pts = [(i, i // 2, l) for i in range(0, 32, 3) for l in (1, 7, 15)]
    got = np.array([[o[q][c[2] + l, c[1] + j, c[0] + i] for q in (1, 2, 3)] for i, j, l in pts])
    want = np.array([debye_point_fp64(i * dx, j * dx, l * dx, k, NA, 200) for i, j, l in pts])
    for q in range(3):
        assert rel_l2(got[:, q], want[:, q]) < 1e-6
