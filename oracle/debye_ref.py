"""CPU oracle for the vectorial Debye-Wolf focus field. TEST INFRASTRUCTURE ONLY.

Restates bpm/psf/_focus_fields_debye.py:focus_field_debye (:48-146) with the kernel
bpm/psf/kernels/psf_debye.cl:debye_wolf (:24-113), and the public wrappers
bpm/psf/psf_functions.py:psf (:18-71), psf_u0 (:104-120) and psf_lightsheet (:75-98).

The octant kernel is evaluated in FP64 with scipy's Bessel functions, from the float32
parameters the reference passes to its kernel (octant extents x2,y2,z2, lam/n0, the
aperture angles). Grid coordinates follow the kernel's FP32 recipe
x = x1 + i*(x2-x1)/(Nx-1.f). The quadrature is the kernel's (quirk Q14): INT_STEPS+1
nodes t = a1 + i*dt with dt = (a2-a1)/(INT_STEPS-1) (so the last node lies past a2),
weight 1/2 at i=0 and i=INT_STEPS, prefactor dt*sqrt(cos t) without sin t.

Mirroring to the full volume is the reference's literal slice loop (:116-144): x/y
mirrors copy values unchanged, the z <= Nz0/2 half is conjugated (quirk Q15).

The variants focus_field_debye_gauss (:361-441), _plane (:149-214) and _at (:315-358)
follow their kernels (psf_debye.cl:273-362, :117-183, :187-269): pupil weight
dt*sqrt(cos t)*sin t (times the Gaussian envelope), half weights decided by the float32
test t == a1 || t == a2, and each variant's own grid, outputs and spreading.
"""
import itertools

import numpy as np
from scipy.special import jv


def octant_params(shape, units, lam, NA, n0):
    """The float32 arguments of the debye_wolf launch (_focus_fields_debye.py:74-109)."""
    if np.isscalar(NA):
        NA = [0., NA]
    Nx0, Ny0, Nz0 = shape
    dx, dy, dz = units
    if not Nx0 % 2 + Ny0 % 2 + Nz0 % 2 == 0:
        raise NotImplementedError("odd shapes not supported yet")
    alphas = np.arcsin(np.array(NA) / n0)
    assert len(alphas) % 2 == 0
    Nx, Ny, Nz = Nx0 // 2 + 1, Ny0 // 2 + 1, Nz0 // 2 + 1
    return dict(Nx=Nx, Ny=Ny, Nz=Nz,
                x2=np.float32(dx * (Nx - 1.)), y2=np.float32(dy * (Ny - 1.)),
                z2=np.float32(dz * (Nz - 1.)), lam=np.float32(1. * lam / n0),
                alphas=alphas.astype(np.float32))


def coord_f32(N, x2, x1=0.):
    """x = x1 + i*(x2-x1)/(N-1.f) in float32 (psf_debye.cl:46-48, :137-138, :299-301)."""
    i = np.arange(N, dtype=np.float32)
    x1 = np.float32(x1)
    return x1 + (i * (np.float32(x2) - x1)) / np.float32(N - 1.)


def quadrature_nodes(alphas, int_steps, quadrature="reference"):
    """Nodes and end weights of the kernel's trapezoid rule per annulus (psf_debye.cl:62-78):
    int_steps+1 nodes, dt = (a2-a1)/(int_steps-1), half weights at i = 0 and i = int_steps.
    quadrature="physical": the exact trapezoid of int_steps nodes over [a1, a2] (half weights
    at both ends), the rule of the reference's tests/test_psf_vectorial.py:15-42."""
    ts, ws = [], []
    for a1, a2 in zip(alphas[0::2], alphas[1::2]):
        a1 = float(a1)
        a2 = float(a2)
        dt = (a2 - a1) / (int_steps - 1.)
        n = int_steps + 1 if quadrature == "reference" else int_steps
        i = np.arange(n)
        t = a1 + i * dt
        w = np.where((i == 0) | (i == n - 1), .5, 1.) * dt
        ts.append(t)
        ws.append(w)
    return np.concatenate(ts), np.concatenate(ws)


def debye_octant(params, int_steps, Ex0=1., Ey0=0., quadrature="reference"):
    """FP64 evaluation of debye_wolf (bpm/psf/kernels/psf_debye.cl:24-113) over the octant,
    node weights as its :62-78 (pupil factor sqrt(cos t)); quadrature="physical" takes the
    exact trapezoid of quadrature_nodes and the Debye integral's sqrt(cos t) sin t.
    Returns (u, ex, ey, ez) of shape (Nz, Ny, Nx) in float64/complex128."""
    Nx, Ny, Nz = params["Nx"], params["Ny"], params["Nz"]
    x = coord_f32(Nx, params["x2"]).astype(np.float64)
    y = coord_f32(Ny, params["y2"]).astype(np.float64)
    z = coord_f32(Nz, params["z2"]).astype(np.float64)
    lam = float(params["lam"])
    k = 2. * np.pi / lam
    Y, X = np.meshgrid(y, x, indexing="ij")
    kr = (k * np.sqrt(X ** 2 + Y ** 2)).ravel()
    phi = np.arctan2(Y, X).ravel()
    kz = k * z
    t, w = quadrature_nodes(params["alphas"], int_steps, quadrature)
    co, si = np.cos(t), np.sin(t)
    with np.errstate(invalid="ignore"):
        pre = w * np.sqrt(co)
    if quadrature == "physical":
        pre = pre * si
    arg = kr[:, None] * si[None, :]
    A0 = (pre * (co + 1.))[None, :] * jv(0, arg)
    A1 = (pre * si)[None, :] * jv(1, arg)
    A2 = (pre * (co - 1.))[None, :] * jv(2, arg)
    E = np.exp(1j * kz[None, :] * co[:, None])          # (T, Z)
    I0 = A0 @ E
    I1 = A1 @ E
    I2 = A2 @ E                                           # (R, Z)
    c2 = np.cos(2 * phi)[:, None]
    s2 = np.sin(2 * phi)[:, None]
    ex = Ex0 * (I0 + I2 * c2) + Ey0 * s2 * I2
    ey = Ey0 * (I0 - I2 * c2) + Ex0 * s2 * I2
    ez = (-2j * I1) * (Ex0 * np.cos(phi) + Ey0 * np.sin(phi))[:, None]
    u = np.abs(ex) ** 2 + np.abs(ey) ** 2 + np.abs(ez) ** 2

    def vol(a):
        return np.ascontiguousarray(a.T.reshape(Nz, Ny, Nx))
    return vol(u), vol(ex), vol(ey), vol(ez)


def mirror_octant(shape, u, ex, ey, ez, real_dtype=np.float32, complex_dtype=np.complex64):
    """The reference's octant -> full volume spreading loop (_focus_fields_debye.py:116-144)."""
    Nx0, Ny0, Nz0 = shape
    Nz, Ny, Nx = u.shape
    u_all = np.empty((Nz0, Ny0, Nx0), real_dtype)
    ex_all = np.empty((Nz0, Ny0, Nx0), complex_dtype)
    ey_all = np.empty((Nz0, Ny0, Nx0), complex_dtype)
    ez_all = np.empty((Nz0, Ny0, Nx0), complex_dtype)
    sx = [slice(0, Nx), slice(Nx, Nx0)]
    sy = [slice(0, Ny), slice(Ny, Ny0)]
    sz = [slice(0, Nz), slice(Nz, Nz0)]
    for i, j, k in itertools.product([0, 1], [0, 1], [0, 1]):
        src = (slice(1 - i, Nz - 1 + i), slice(1 - j, Ny - 1 + j), slice(1 - k, Nx - 1 + k))
        flip = (slice(None, None, (-1) ** i), slice(None, None, (-1) ** j), slice(None, None, (-1) ** k))
        dst = (sz[1 - i], sy[1 - j], sx[1 - k])
        u_all[dst] = u[src][flip]
        for a, a_all in ((ex, ex_all), (ey, ey_all), (ez, ez_all)):
            v = a[src][flip]
            a_all[dst] = v if i == 0 else np.conjugate(v)
    return u_all, ex_all, ey_all, ez_all


def mirror_index(N0):
    """Index form of the same spreading along one axis (_focus_fields_debye.py:116-144):
    full index m -> octant |m - N0/2|."""
    return np.abs(np.arange(N0) - N0 // 2)


def focus_field_debye(shape, units, lam, NA, n0=1., n_integration_steps=200,
                      real_dtype=np.float32, complex_dtype=np.complex64, quadrature="reference"):
    """FP64 restatement of focus_field_debye (bpm/psf/_focus_fields_debye.py:48-146);
    returns (u, ex, ey, ez) on (Nz0, Ny0, Nx0)."""
    params = octant_params(shape, units, lam, NA, n0)
    oct_ = debye_octant(params, n_integration_steps, quadrature=quadrature)
    return mirror_octant(shape, *oct_, real_dtype=real_dtype, complex_dtype=complex_dtype)


def quadrature_nodes_f32_ends(alphas, int_steps):
    """Trapezoid rule of debye_wolf_plane/_at/_gauss (psf_debye.cl:155-167, :240-252,
    :328-343): the same INT_STEPS+1 nodes per annulus, but the half weight goes to the
    nodes whose float32 angle t = a1 + i*dt (dt = (a2-a1)/(INT_STEPS-1.f), each operation
    rounded on its own) equals a1 or a2. Node i = INT_STEPS-1 therefore gets the half
    weight only when that float32 sum lands exactly on a2. Returns FP64 nodes and weights."""
    f = np.float32
    ts, ws = [], []
    for a1, a2 in zip(alphas[0::2], alphas[1::2]):
        a1, a2 = f(a1), f(a2)
        dt32 = (a2 - a1) / f(int_steps - 1.)
        t32 = a1 + np.arange(int_steps + 1, dtype=np.float32) * dt32
        end = (t32 == a1) | (t32 == a2)
        dt = (float(a2) - float(a1)) / (int_steps - 1.)
        ts.append(float(a1) + np.arange(int_steps + 1) * dt)
        ws.append(np.where(end, .5, 1.) * dt)
    return np.concatenate(ts), np.concatenate(ws)


def _assemble(I0, I1, I2, phi, Ex0, Ey0):
    """psf_debye.cl:90-101 (and its copies in the variants)."""
    c2, s2 = np.cos(2 * phi), np.sin(2 * phi)
    ex = Ex0 * (I0 + I2 * c2) + Ey0 * s2 * I2
    ey = Ey0 * (I0 - I2 * c2) + Ex0 * s2 * I2
    ez = (-2j * I1) * (Ex0 * np.cos(phi) + Ey0 * np.sin(phi))
    return ex, ey, ez


def _integrals_points(kr, kz, t, pre):
    """I_n at arbitrary points (kr, kz), the node sums of debye_wolf_plane and debye_wolf_at
    (psf_debye.cl:117-269): (P,) arrays; pre: (T,) weights without the component factors.
    FP64."""
    co, si = np.cos(t), np.sin(t)
    arg = kr[:, None] * si[None, :]
    E = np.exp(1j * kz[:, None] * co[None, :])
    I0 = np.sum((pre * (co + 1.))[None, :] * jv(0, arg) * E, axis=1)
    I1 = np.sum((pre * si)[None, :] * jv(1, arg) * E, axis=1)
    I2 = np.sum((pre * (co - 1.))[None, :] * jv(2, arg) * E, axis=1)
    return I0, I1, I2


def focus_field_debye_gauss(shape, units, lam, NAs, sig=1. / np.sqrt(2), n_integration_steps=200):
    """FP64 restatement of _focus_fields_debye.py:focus_field_debye_gauss (:361-441) with
    debye_wolf_gauss (psf_debye.cl:273-362): octant ((N0+1)//2 per axis) on
    x in [0, dx*Nx] (Nx the octant size), lam and alphas = arcsin(NAs) without n0, pupil
    weight sqrt(cos t) sin t exp(t^2 * (-.5/alpha_max^2/sig^2)), and the slice-loop
    mirroring without conjugation. Returns (u, ex, ey, ez) on (Nz0, Ny0, Nx0)."""
    assert sig > 0
    Nx0, Ny0, Nz0 = shape
    dx, dy, dz = units
    alphas = np.arcsin(np.array(NAs)).astype(np.float32)
    Nx, Ny, Nz = (Nx0 + 1) // 2, (Ny0 + 1) // 2, (Nz0 + 1) // 2
    x = coord_f32(Nx, np.float32(dx * Nx)).astype(np.float64)
    y = coord_f32(Ny, np.float32(dy * Ny)).astype(np.float64)
    z = coord_f32(Nz, np.float32(dz * Nz)).astype(np.float64)
    k = 2. * np.pi / float(np.float32(lam))
    t, w = quadrature_nodes_f32_ends(alphas, n_integration_steps)
    amax = float(alphas[-1])
    sig32 = float(np.float32(sig))
    prefac = -.5 / amax / amax / sig32 / sig32
    co, si = np.cos(t), np.sin(t)
    with np.errstate(invalid="ignore"):
        pre = w * np.sqrt(co) * si * np.exp(t * t * prefac)
    Y, X = np.meshgrid(y, x, indexing="ij")
    kr = (k * np.sqrt(X ** 2 + Y ** 2)).ravel()
    phi = np.arctan2(Y, X).ravel()
    arg = kr[:, None] * si[None, :]
    E = np.exp(1j * (k * z)[None, :] * co[:, None])
    I0 = ((pre * (co + 1.))[None, :] * jv(0, arg)) @ E
    I1 = ((pre * si)[None, :] * jv(1, arg)) @ E
    I2 = ((pre * (co - 1.))[None, :] * jv(2, arg)) @ E
    ex, ey, ez = _assemble(I0, I1, I2, phi[:, None], 1., 0.)
    u = np.abs(ex) ** 2 + np.abs(ey) ** 2 + np.abs(ez) ** 2

    def vol(a):
        return np.ascontiguousarray(a.T.reshape(Nz, Ny, Nx))
    return mirror_octant_gauss(shape, vol(u), vol(ex), vol(ey), vol(ez))


def mirror_octant_gauss(shape, u, ex, ey, ez, real_dtype=np.float32, complex_dtype=np.complex64):
    """The gauss variant's spreading loop (_focus_fields_debye.py:426-438): octant index 0
    lands at N0-N, the mirrored copy fills 0..N-1 reversed, nothing is conjugated."""
    Nx0, Ny0, Nz0 = shape
    Nz, Ny, Nx = u.shape
    outs = [np.empty((Nz0, Ny0, Nx0), real_dtype)] + [np.empty((Nz0, Ny0, Nx0), complex_dtype)
                                                      for _ in range(3)]
    sx = [slice(0, Nx), slice(Nx0 - Nx, Nx0)]
    sy = [slice(0, Ny), slice(Ny0 - Ny, Ny0)]
    sz = [slice(0, Nz), slice(Nz0 - Nz, Nz0)]
    for i, j, k in itertools.product([0, 1], [0, 1], [0, 1]):
        flip = (slice(None, None, (-1) ** i), slice(None, None, (-1) ** j), slice(None, None, (-1) ** k))
        for a, a_all in zip((u, ex, ey, ez), outs):
            a_all[sz[1 - i], sy[1 - j], sx[1 - k]] = a[flip]
    return tuple(outs)


def mirror_index_gauss(N0):
    """Index form of mirror_octant_gauss along one axis (_focus_fields_debye.py:426-438):
    full index p -> octant index."""
    N = (N0 + 1) // 2
    p = np.arange(N0)
    return np.where(p >= N0 - N, p - (N0 - N), N - 1 - p)


def focus_field_debye_plane(shape=(128, 128), units=(.1, .1), z=0., lam=.5, NA=.6, n0=1.,
                            n_integration_steps=200):
    """FP64 restatement of _focus_fields_debye.py:focus_field_debye_plane (:149-214) with
    debye_wolf_plane (psf_debye.cl:117-183): ex only, on (Ny, Nx) over
    x in [-(Nx//2)*dx, (Nx - Nx//2)*dx] (same for y), lam/n0, alphas = arcsin(NA/n0)."""
    if np.isscalar(NA):
        NA = [0., NA]
    Nx, Ny = shape
    dx, dy = units
    alphas = np.arcsin(np.array(NA) / n0).astype(np.float32)
    assert len(alphas) % 2 == 0
    x = coord_f32(Nx, np.float32((Nx - Nx // 2) * dx), np.float32(-(Nx // 2) * dx)).astype(np.float64)
    y = coord_f32(Ny, np.float32((Ny - Ny // 2) * dy), np.float32(-(Ny // 2) * dy)).astype(np.float64)
    k = 2. * np.pi / float(np.float32(lam / n0))
    t, w = quadrature_nodes_f32_ends(alphas, n_integration_steps)
    with np.errstate(invalid="ignore"):
        pre = w * np.sqrt(np.cos(t)) * np.sin(t)
    Y, X = np.meshgrid(y, x, indexing="ij")
    kr = (k * np.sqrt(X ** 2 + Y ** 2)).ravel()
    phi = np.arctan2(Y, X).ravel()
    kz = np.full_like(kr, k * float(np.float32(z)))
    I0, I1, I2 = _integrals_points(kr, kz, t, pre)
    ex, _, _ = _assemble(I0, I1, I2, phi, 1., 0.)
    return ex.reshape(Ny, Nx).astype(np.complex64)


def focus_field_debye_at(x, y, z, lam, NA, n0=1., n_integration_steps=200):
    """FP64 restatement of _focus_fields_debye.py:focus_field_debye_at (:315-358) with
    debye_wolf_at (psf_debye.cl:187-269): fields at float32 points (x, y, z); the returned
    intensity is |ex|^2 only (psf_debye.cl:267). Returns (u, ex, ey, ez) of x's shape."""
    if np.isscalar(NA):
        NA = [0., NA]
    alphas = np.arcsin(np.array(NA) / n0).astype(np.float32)
    assert len(alphas) % 2 == 0
    x, y, z = (np.asarray(a) for a in (x, y, z))
    assert x.shape == y.shape == z.shape
    dshape = x.shape
    xf, yf, zf = (a.ravel().astype(np.float32).astype(np.float64) for a in (x, y, z))
    k = 2. * np.pi / float(np.float32(lam / n0))
    t, w = quadrature_nodes_f32_ends(alphas, n_integration_steps)
    with np.errstate(invalid="ignore"):
        pre = w * np.sqrt(np.cos(t)) * np.sin(t)
    kr = k * np.sqrt(xf ** 2 + yf ** 2)
    phi = np.arctan2(yf, xf)
    I0, I1, I2 = _integrals_points(kr, k * zf, t, pre)
    ex, ey, ez = _assemble(I0, I1, I2, phi, 1., 0.)
    u = np.abs(ex) ** 2
    return (u.reshape(dshape).astype(np.float32), ex.reshape(dshape).astype(np.complex64),
            ey.reshape(dshape).astype(np.complex64), ez.reshape(dshape).astype(np.complex64))


def psf(shape, units, lam, NA, n0=1., n_integration_steps=200, return_field=False, **kw):
    """bpm/psf/psf_functions.py:psf (:18-71)."""
    u, ex, ey, ez = focus_field_debye(shape, units, lam, NA, n0, n_integration_steps, **kw)
    return (u, ex, ey, ez) if return_field else u


def psf_u0(shape, units, zfoc=0, NA=.4, lam=.5, n0=1., n_integration_steps=200, **kw):
    """bpm/psf/psf_functions.py:psf_u0 (:104-120): ex[0] of a 4-plane PSF with dz = zfoc/2."""
    Nx, Ny = shape
    dx, dy = units
    u, ex, ey, ez = psf((Nx, Ny, 4), (dx, dy, zfoc / 2.), n0=n0, lam=lam, NA=NA,
                        n_integration_steps=n_integration_steps, return_field=True, **kw)
    return ex[0, ...]


def psf_lightsheet(shape, units, lam_illum, NA_illum, lam_detect, NA_detect, n0=1.,
                   n_integration_steps=200, **kw):
    """bpm/psf/psf_functions.py:psf_lightsheet (:75-98): detection PSF times the
    illumination PSF computed on the reversed axes and transposed back."""
    u_detect = psf(shape, units, lam=lam_detect, NA=NA_detect, n0=n0,
                   n_integration_steps=n_integration_steps, **kw)
    u_illum = psf(tuple(shape)[::-1], tuple(units)[::-1], lam=lam_illum, NA=NA_illum, n0=n0,
                  n_integration_steps=n_integration_steps, **kw)
    return u_detect * u_illum.transpose((2, 1, 0))
