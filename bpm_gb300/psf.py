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

__all__ = ["focus_field_debye", "psf", "psf_u0", "psf_lightsheet"]


def _debye(shape, units, lam, NA, n0, n_integration_steps, want_u, want_field, ex0=1., ey0=0.):
    if np.isscalar(NA):
        NA = [0., NA]
    NA = [float(a) for a in NA]
    Nx0, Ny0, Nz0 = (int(s) for s in shape)
    dx, dy, dz = (float(u) for u in units)
    if not Nx0 % 2 + Ny0 % 2 + Nz0 % 2 == 0:
        raise NotImplementedError("odd shapes not supported yet")
    assert len(NA) % 2 == 0
    na = (ctypes.c_double * len(NA))(*NA)
    desc = N.DebyeDesc(Nx0, Ny0, Nz0, dx, dy, dz, float(lam), float(n0),
                       ctypes.cast(na, ctypes.POINTER(ctypes.c_double)), len(NA),
                       int(n_integration_steps), float(ex0), float(ey0))
    L = N.lib()
    wsb = int(L.debye_workspace_bytes(ctypes.byref(desc)))
    if wsb == 0:
        rc = L.debye_focus_field(ctypes.byref(desc), None, None, None, None, None, 0, None)
        N.check(rc, "debye_focus_field")
    dev = _device()
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
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


def focus_field_debye(shape, units, lam, NA, n0=1., n_integration_steps=200, device=False):
    """Focus field of an aberration-free objective by the vectorial Debye integral
    (bpm/psf/_focus_fields_debye.py:48). Returns u, ex, ey, ez on (Nz, Ny, Nx), u being the
    intensity. NA is a number or an even-length list of annulus limits."""
    u, ex, ey, ez = _debye(shape, units, lam, NA, n0, n_integration_steps, True, True)
    if device:
        return u, ex, ey, ez
    return _d2h(u), _d2h(ex), _d2h(ey), _d2h(ez)


def psf(shape, units, lam, NA, n0=1., n_integration_steps=200, return_field=False, device=False):
    """3d PSF of an aberration-free optical system (bpm/psf/psf_functions.py:18): the
    intensity u, or (u, ex, ey, ez) with return_field=True."""
    u, ex, ey, ez = _debye(shape, units, lam, NA, n0, n_integration_steps, True, return_field)
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
