"""Vectorial Debye-Wolf focus fields: the drop-in host API.

Mirrors bpm/psf/psf_functions.py (psf :18-71, psf_lightsheet :75-98, psf_u0 :104-120)
and bpm/psf/_focus_fields_debye.py:focus_field_debye (:48-146): same arguments, shapes
(arrays (Nz, Ny, Nx) for shape = (Nx, Ny, Nz)), dtypes and errors. The octant quadrature
and the spreading to the full volume both run in libbpm_gb300.so (debye_focus_field).
Pass device=True to get torch CUDA tensors instead of numpy arrays.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .bpm3d import _device, _d2h, _ptr, _stream_ptr

__all__ = ["focus_field_debye", "focus_field_debye_gauss", "focus_field_debye_plane", "focus_field_debye_at",
           "psf", "psf_u0", "psf_lightsheet"]


QUADRATURES = {"reference": 0, "physical": 1}


def _desc(shape3, units3, lam, NA, n0, n_integration_steps, ex0=1., ey0=0., quadrature="reference"):
    """debye_desc for the C ABI; returns (desc, keep-alive NA array)."""
    if quadrature not in QUADRATURES:
        raise ValueError("quadrature must be 'reference' or 'physical'")
    if np.isscalar(NA):
        NA = [0., NA]
    NA = [float(a) for a in np.asarray(NA, np.float64).ravel()]
    assert len(NA) % 2 == 0
    na = (ctypes.c_double * len(NA))(*NA)
    desc = N.DebyeDesc(int(shape3[0]), int(shape3[1]), int(shape3[2]), float(units3[0]), float(units3[1]),
                       float(units3[2]), float(lam), float(n0), ctypes.cast(na, ctypes.POINTER(ctypes.c_double)),
                       len(NA), int(n_integration_steps), float(ex0), float(ey0), QUADRATURES[quadrature])
    return desc, na


def _workspace(size_fn, run_fn, desc, what):
    """Workspace tensor for `desc`; a size of 0 means the description is invalid, and the
    entry point itself then reports why."""
    wsb = int(size_fn(ctypes.byref(desc)))
    if wsb == 0:
        N.check(run_fn(), what)
    return torch.empty(wsb, dtype=torch.uint8, device=_device()), wsb


def _debye(shape, units, lam, NA, n0, n_integration_steps, want_u, want_field, ex0=1., ey0=0.,
           quadrature="reference"):
    Nx0, Ny0, Nz0 = (int(s) for s in shape)
    if not Nx0 % 2 + Ny0 % 2 + Nz0 % 2 == 0:
        raise NotImplementedError("odd shapes not supported yet")
    desc, _na = _desc(shape, units, lam, NA, n0, n_integration_steps, ex0, ey0, quadrature)
    L = N.lib()
    ws, wsb = _workspace(L.debye_workspace_bytes,
                         lambda: L.debye_focus_field(ctypes.byref(desc), None, None, None, None, None, 0, None),
                         desc, "debye_focus_field")
    dev = _device()
    u = torch.empty((Nz0, Ny0, Nx0), dtype=torch.float32, device=dev) if want_u else None
    ex = ey = ez = None
    if want_field:
        ex = torch.empty((Nz0, Ny0, Nx0), dtype=torch.complex64, device=dev)
        ey = torch.empty_like(ex)
        ez = torch.empty_like(ex)
    rc = L.debye_focus_field(ctypes.byref(desc), _ptr(u), _ptr(ex), _ptr(ey), _ptr(ez), _ptr(ws), wsb,
                             _stream_ptr())
    N.check(rc, "debye_focus_field")
    return u, ex, ey, ez


def focus_field_debye(shape, units, lam, NA, n0=1., n_integration_steps=200, device=False,
                      quadrature="reference"):
    """Focus field of an aberration-free objective by the vectorial Debye integral
    (bpm/psf/_focus_fields_debye.py:48). Returns u, ex, ey, ez on (Nz, Ny, Nx), u being the
    intensity. NA is a number or an even-length list of annulus limits.
    quadrature="reference" (default) is the reference kernel's rule (n_integration_steps+1
    nodes, the last one past the aperture angle, pupil factor sqrt(cos t) without sin t);
    "physical" is the Debye integral's sqrt(cos t) sin t with an exact trapezoid of
    n_integration_steps nodes over each annulus (an addition: the reference kernel has no
    such option, its test script evaluates this formula)."""
    u, ex, ey, ez = _debye(shape, units, lam, NA, n0, n_integration_steps, True, True, quadrature=quadrature)
    if device:
        return u, ex, ey, ez
    return _d2h(u), _d2h(ex), _d2h(ey), _d2h(ez)


def focus_field_debye_gauss(shape, units, lam, NAs, sig=1. / np.sqrt(2), n_integration_steps=200, device=False):
    """Detection PSF of a pupil under a Gaussian envelope exp(-r^2/2/sig^2), r = 1 at the
    aperture edge (bpm/psf/_focus_fields_debye.py:361). NAs is an increasing even-length
    list of annulus limits (no n0: the angles are arcsin(NAs)). Returns u, ex, ey, ez on
    (Nz, Ny, Nx); any shape >= 3 per axis."""
    assert sig > 0
    NAs = list(np.asarray(NAs, np.float64).ravel())
    shape = tuple(int(s) for s in shape)
    desc, _na = _desc(shape, units, lam, NAs, 1., n_integration_steps)
    L = N.lib()
    ws, wsb = _workspace(L.debye_gauss_workspace_bytes,
                         lambda: L.debye_focus_field_gauss(ctypes.byref(desc), float(sig), None, None, None, None,
                                                           None, 0, None),
                         desc, "debye_focus_field_gauss")
    dev = _device()
    Nx0, Ny0, Nz0 = shape
    u = torch.empty((Nz0, Ny0, Nx0), dtype=torch.float32, device=dev)
    ex = torch.empty((Nz0, Ny0, Nx0), dtype=torch.complex64, device=dev)
    ey = torch.empty_like(ex)
    ez = torch.empty_like(ex)
    N.check(L.debye_focus_field_gauss(ctypes.byref(desc), float(sig), _ptr(u), _ptr(ex), _ptr(ey), _ptr(ez),
                                      _ptr(ws), wsb, _stream_ptr()), "debye_focus_field_gauss")
    if device:
        return u, ex, ey, ez
    return _d2h(u), _d2h(ex), _d2h(ey), _d2h(ez)


def focus_field_debye_plane(shape=(128, 128), units=(.1, .1), z=0., lam=.5, NA=.6, n0=1., ex_g=None,
                            n_integration_steps=200, device=False):
    """x component of the focus field on the plane at height z (bpm/psf/_focus_fields_debye.py:149),
    on (Ny, Nx) for shape = (Nx, Ny), x spanning [-(Nx//2)*dx, (Nx - Nx//2)*dx]. If ex_g (a
    CUDA complex64 tensor of shape (Ny, Nx)) is given it is filled and None is returned."""
    Nx, Ny = (int(s) for s in shape)
    dx, dy = units
    use_buffer = ex_g is not None
    if use_buffer:
        assert tuple(ex_g.shape)[::-1] == (Nx, Ny)
        if not (isinstance(ex_g, torch.Tensor) and ex_g.is_cuda and ex_g.dtype == torch.complex64
                and ex_g.is_contiguous()):
            raise TypeError("ex_g must be a contiguous complex64 CUDA tensor")
    desc, _na = _desc((Nx, Ny, 1), (dx, dy, 0.), lam, NA, n0, n_integration_steps)
    L = N.lib()
    ws, wsb = _workspace(L.debye_points_workspace_bytes,
                         lambda: L.debye_focus_field_plane(ctypes.byref(desc), float(z), None, None, 0, None),
                         desc, "debye_focus_field_plane")
    ex = ex_g if use_buffer else torch.empty((Ny, Nx), dtype=torch.complex64, device=_device())
    N.check(L.debye_focus_field_plane(ctypes.byref(desc), float(z), _ptr(ex), _ptr(ws), wsb, _stream_ptr()),
            "debye_focus_field_plane")
    if use_buffer:
        return None
    return ex if device else _d2h(ex)


def focus_field_debye_at(x, y, z, lam, NA, n0=1., n_integration_steps=200, device=False):
    """focus_field_debye at the points (x, y, z) (arrays of one shape; numpy or CUDA
    tensors) instead of a grid (bpm/psf/_focus_fields_debye.py:315). Returns u, ex, ey, ez
    of that shape, u being |ex|^2 as the reference kernel writes it."""
    dev = _device()

    def flat(a):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32)))
        return t.to(device=dev, dtype=torch.float32).reshape(-1).contiguous()
    shp = tuple(x.shape)
    assert shp == tuple(y.shape) == tuple(z.shape)
    xs, ys, zs = flat(x), flat(y), flat(z)
    n = xs.numel()
    desc, _na = _desc((0, 0, 0), (0., 0., 0.), lam, NA, n0, n_integration_steps)
    L = N.lib()
    ws, wsb = _workspace(L.debye_points_workspace_bytes,
                         lambda: L.debye_focus_field_at(ctypes.byref(desc), None, None, None, 0, None, None, None,
                                                        None, None, 0, None),
                         desc, "debye_focus_field_at")
    u = torch.empty(n, dtype=torch.float32, device=dev)
    ex = torch.empty(n, dtype=torch.complex64, device=dev)
    ey = torch.empty_like(ex)
    ez = torch.empty_like(ex)
    N.check(L.debye_focus_field_at(ctypes.byref(desc), _ptr(xs), _ptr(ys), _ptr(zs), n, _ptr(u), _ptr(ex), _ptr(ey),
                                   _ptr(ez), _ptr(ws), wsb, _stream_ptr()), "debye_focus_field_at")
    res = tuple(a.reshape(shp) for a in (u, ex, ey, ez))
    if device:
        return res
    return tuple(_d2h(a) for a in res)


def psf(shape, units, lam, NA, n0=1., n_integration_steps=200, return_field=False, device=False,
        quadrature="reference"):
    """3d PSF of an aberration-free optical system (bpm/psf/psf_functions.py:18): the
    intensity u, or (u, ex, ey, ez) with return_field=True. quadrature as in
    focus_field_debye."""
    u, ex, ey, ez = _debye(shape, units, lam, NA, n0, n_integration_steps, True, return_field,
                           quadrature=quadrature)
    conv = (lambda t: t) if device else _d2h
    if return_field:
        return conv(u), conv(ex), conv(ey), conv(ez)
    return conv(u)


def psf_u0(shape, units, zfoc=0, NA=.4, lam=.5, n0=1., n_integration_steps=200, device=False):
    """Initial plane u0 (Ny, Nx) of a beam focused at zfoc (bpm/psf/psf_functions.py:104):
    ex at plane 0 of a 4-plane PSF with dz = zfoc/2 (the conjugated field at z = -zfoc)."""
    Nx, Ny = shape
    dx, dy = units
    _, ex, _, _ = _debye((Nx, Ny, 4), (dx, dy, zfoc / 2.), lam, NA, n0, n_integration_steps, False, True)
    e0 = ex[0].clone()
    return e0 if device else _d2h(e0)


def psf_lightsheet(shape, units, lam_illum, NA_illum, lam_detect, NA_detect, n0=1.,
                   n_integration_steps=200, return_field=False, device=False):
    """Light-sheet PSF (bpm/psf/psf_functions.py:75): detection PSF times the illumination
    PSF computed on the reversed axes and transposed back."""
    u_detect = psf(shape, units, lam=lam_detect, NA=NA_detect, n0=n0,
                   n_integration_steps=n_integration_steps, device=True)
    u_illum = psf(tuple(shape)[::-1], tuple(units)[::-1], lam=lam_illum, NA=NA_illum, n0=n0,
                  n_integration_steps=n_integration_steps, device=True)
    res = u_detect * u_illum.permute(2, 1, 0)
    return res if device else _d2h(res.contiguous())
