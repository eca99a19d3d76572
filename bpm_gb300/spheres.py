"""Propagation through media of coated spheres, with the dn volume generated on the device.

Mirrors bpm/bpm/bpm_3d_spheres.py: create_dn_buffer (:11-38) and bpm_3d_spheres (:42-67).
The volume is filled by bpm_spheres_fill in libbpm_gb300.so (the reference's fill_dn,
bpm/bpm/kernels/bpm_3d_spheres.cl:31-74) and stays on the device, so served requests need
no host->device upload of dn.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .bpm3d import _d2h, _device, _ptr, _stream_ptr, bpm_3d

__all__ = ["create_dn_buffer", "bpm_3d_spheres"]


def create_dn_buffer(size, units, points, dn_inner=.0, rad_inner=0, dn_outer=.1, rad_outer=.4):
    """dn volume (Nz, Ny, Nx) float32 on the device: coated spheres centred at `points`
    ([[x, y, z], ...] in microns), inner radius/index rad_inner/dn_inner, outer
    rad_outer/dn_outer (bpm/bpm/bpm_3d_spheres.py:11-38, kernel fill_dn in
    bpm_3d_spheres.cl:31-74). Returns a torch CUDA tensor (the reference returns its
    device buffer, an OCLArray)."""
    Nx, Ny, Nz = (int(s) for s in size)
    dx, dy, dz = (float(u) for u in units)
    ps = np.asarray(points, np.float64).reshape(-1, 3)
    ps = ps[np.argsort(ps[:, 2], kind="stable"), :]           # sort by z (bpm_3d_spheres.py:25)
    dev = _device()
    pts = torch.from_numpy(np.ascontiguousarray(ps.astype(np.float32))).to(dev)
    dn = torch.empty((Nz, Ny, Nx), dtype=torch.float32, device=dev)
    N.check(N.lib().bpm_spheres_fill(Nx, Ny, Nz, dx, dy, dz, _ptr(pts), int(ps.shape[0]), float(dn_inner),
                                     float(rad_inner), float(dn_outer), float(rad_outer), _ptr(dn),
                                     _stream_ptr()), "bpm_spheres_fill")
    return dn


def bpm_3d_spheres(size, units, lam=.5, u0=None, points=None, dn_inner=0.0, rad_inner=0., dn_outer=0.05,
                   rad_outer=2.5, return_scattering=False, use_fresnel_approx=False, device=False):
    """bpm_3d through coated spheres at `points` (bpm/bpm/bpm_3d_spheres.py:42-67). Results
    are numpy arrays unless device=True (or u0 is a CUDA tensor)."""
    dn_g = create_dn_buffer(size, units, points=points, dn_inner=dn_inner, rad_inner=rad_inner,
                            dn_outer=dn_outer, rad_outer=rad_outer)
    res = bpm_3d(size=size, units=units, lam=lam, u0=u0, dn=dn_g, return_scattering=return_scattering,
                 use_fresnel_approx=use_fresnel_approx)
    if device or isinstance(u0, torch.Tensor):
        return res
    if isinstance(res, tuple):
        return tuple(_d2h(r) for r in res)
    return _d2h(res)
