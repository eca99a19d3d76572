"""CPU oracle for the split-step BPM z-march. TEST INFRASTRUCTURE ONLY.

Restates, in numpy/scipy, the algorithm of the reference's functional driver
bpm/bpm/bpm_3d.py (bpm_3d :39-101, _bpm_3d :104-423, _bpm_3d_split :863-992) with the
elementwise kernels of bpm/bpm/kernels/bpm_3d_kernels.cl, and of the object path
bpm/bpmclass/bpm3d.py (:24-167) + bpm/bpmclass/_bpm3d_ocl.py (_propagate_single :66-134).

Two flavours (`precision=`):
  "fp32" -- reference-faithful: complex64 field, single-precision FFT (scipy.fft keeps
            complex64), every elementwise formula evaluated in float32 in the order the
            OpenCL kernels write it. This is the "reference-output" oracle.
  "fp64" -- complex128 field and FFT, FP64 propagator phase, dn phase and mean-index
            reductions; the evanescent mask (FP32 FFTFREQ recipe) and the absorbing
            taper values stay those of the reference so that only rounding differs.

The 2-D FFT of the reference comes from the third-party gputools package (not under
the reference tree, no version pinned in setup.py:12-14). Its convention is pinned by
the reference itself: forward unnormalised (plain_wave_dct = Nx*Ny*..., bpm_3d.py:253),
inverse normalised by 1/(Nx*Ny), sign exp(-i k x) forward. Its round-off is not pinned.

Reference quirks reproduced (see the docstring of each function): FP32-recipe evanescent
mask and propagator overwrite (bpm_3d.py:192), weighted mode reducing |u_hat|*dn over
dn slice 0 in k-space (:149-153, :302-303), plane 0 = u0 unmasked, mask of slice i+1
after step i, taper only for real/half dn. Divergences, each because the reference is
undefined there: dn=None is zeros (the reference uses an uninitialised buffer,
bpm_3d.py:214); complex dn in "weighted"/"simple" raises NotImplementedError (the
reference passes mismatched buffer types, :153, :288-293); complex dn in "ignore" uses
dn0 = 0 as intended; half dn in "weighted" reduces over the half values (the reference
reads the half buffer as float32); the Bpm3d k-grid is the intended (Ny, Nx) one
(bpmclass/bpm3d.py:93 swaps it; identical for square grids).
"""
import ctypes
import ctypes.util

import numpy as np
import scipy.fft as sfft

PI_F = np.float32(3.14159265358979)        # bpm_3d_kernels.cl:3  #define M_PI ...f
TWO_PI_F = np.float32(2.0) * PI_F          # 2.f*M_PI, bpm_3d_kernels.cl:421

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.cosf.restype = ctypes.c_float
_libm.cosf.argtypes = [ctypes.c_float]


def _workers():
    import os
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------------------
# FP32 recipes of the kernels (bit-exact where they involve no transcendental function)
# ----------------------------------------------------------------------------------------

def fftfreq_f32(N, d):
    """FFTFREQ(i,N,dx) of bpm_3d_kernels.cl:6 in float32: 1.f*i/N/dx, negative half shifted."""
    i = np.arange(N, dtype=np.int64)
    half = (N - 1) // 2 + 1
    num = np.where(i < half, i, (i - half) - N // 2).astype(np.float32)
    return (num / np.float32(N)) / np.float32(d)


def k_axes_f32(Nx, Ny, dx, dy):
    """kx = 2.f*M_PI*FFTFREQ(i,Nx,dx), ky likewise (bpm_3d_kernels.cl:421-422)."""
    return TWO_PI_F * fftfreq_f32(Nx, dx), TWO_PI_F * fftfreq_f32(Ny, dy)


def prop_tmp_f32(n, k0, kx, ky):
    """tmp = n*n*k0*k0 - kx*kx - ky*ky in float32, C evaluation order (bpm_3d_kernels.cl:425).

    Returns the (Ny, Nx) array whose sign is the evanescent mask (tmp >= 0 propagates)."""
    n = np.float32(n)
    k0 = np.float32(k0)
    nk = ((n * n) * k0) * k0
    return (nk - (kx * kx)[None, :]) - (ky * ky)[:, None]


def propagator_f32(n, k0, dx, dy, dz, Nx, Ny):
    """compute_propagator / mult_propagator factor h (bpm_3d_kernels.cl:408-432, :437-462):
    h = (tmp>=0) * (cos(-dz*h0), sin(-dz*h0)), h0 = sqrt(max(tmp,0)), all float32."""
    kx, ky = k_axes_f32(Nx, Ny, dx, dy)
    tmp = prop_tmp_f32(n, k0, kx, ky)
    mask = tmp >= np.float32(0)
    h0 = np.where(mask, np.sqrt(np.where(mask, tmp, np.float32(0))), np.float32(0)).astype(np.float32)
    ph = (-np.float32(dz)) * h0
    m = mask.astype(np.float32)
    return ((m * np.cos(ph)) + 1j * (m * np.sin(ph))).astype(np.complex64), mask


def propagator_f64(n, k0, dx, dy, dz, Nx, Ny):
    """FP64 flavour of compute_propagator (bpm/bpm/kernels/bpm_3d_kernels.cl:408-432) and of
    the host H0/H of _bpm_3d (bpm/bpm/bpm_3d.py:171-181): mask from the FP32 recipe at
    float32(n), phase exp(-i dz kz) in FP64."""
    kx32, ky32 = k_axes_f32(Nx, Ny, dx, dy)
    mask = prop_tmp_f32(np.float32(n), np.float32(k0), kx32, ky32) >= 0
    kx = 2 * np.pi * np.fft.fftfreq(Nx, dx)
    ky = 2 * np.pi * np.fft.fftfreq(Ny, dy)
    tmp = float(n) ** 2 * float(k0) ** 2 - kx[None, :] ** 2 - ky[:, None] ** 2
    kz = np.sqrt(np.maximum(tmp, 0.0))
    return np.where(mask, np.exp(-1j * float(dz) * kz), 0.0).astype(np.complex128), mask


def taper_dist(Nx, Ny):
    """dist = min(min(Nx-i-1,i), min(Ny-j-1,j)) of the mult_dn* kernels (bpm_3d_kernels.cl:32-34)."""
    i = np.arange(Nx)
    j = np.arange(Ny)
    dx_ = np.minimum(Nx - i - 1, i)
    dy_ = np.minimum(Ny - j - 1, j)
    return np.minimum(dx_[None, :], dy_[:, None])


def taper_values_f32(absorb):
    """absorb_val(dist) = 0.5f*(1-cos(M_PI*dist/absorb)) for dist < absorb, float32 with
    libm cosf (bpm_3d_kernels.cl:36). Entry d of the returned array is the value for dist=d."""
    absorb = int(absorb)
    out = np.ones(max(absorb, 0), np.float32)
    for d in range(absorb):
        arg = np.float32(PI_F * np.float32(d)) / np.float32(absorb)
        c = np.float32(_libm.cosf(float(arg)))
        out[d] = np.float32(0.5) * (np.float32(1.0) - c)
    return out


def taper_f32(Nx, Ny, absorb):
    """(Ny, Nx) float32 taper of the mult_dn* kernels (bpm_3d_kernels.cl:20-51, :104-136:
    0.5 (1 - cos(pi d / absorb)) for d < absorb); 1 where dist >= absorb."""
    dist = taper_dist(Nx, Ny)
    vals = taper_values_f32(absorb)
    t = np.ones((Ny, Nx), np.float32)
    if absorb > 0:
        sel = dist < absorb
        t[sel] = vals[dist[sel]]
    return t


def half_to_f32(dn):
    """dn stored as float16 and read back as float32, as store_dn_as_half does
    (bpm/bpm/bpm_3d.py:208-209; the *_half kernels, bpm_3d_kernels.cl:52-81, :139-171)."""
    return np.asarray(dn, dtype=np.float16).astype(np.float32)


# ----------------------------------------------------------------------------------------
# the functional driver: bpm_3d / _bpm_3d / _bpm_3d_split
# ----------------------------------------------------------------------------------------

def _fft2(a, workers):
    return sfft.fft2(a, workers=workers, overwrite_x=True)


def _ifft2(a, workers):
    return sfft.ifft2(a, workers=workers, overwrite_x=True)


def _bpm_3d(size, units, lam=.5, u0=None, dn=None, subsample=1, n0=1.,
            return_scattering=False, return_g=False, return_full=True, return_field=True,
            use_fresnel_approx=False, absorbing_width=0, scattering_plane_ind=0,
            return_last_plane=False, store_dn_as_half=False, mean_mode="weighted",
            precision="fp32", workers=None):
    """Restatement of bpm/bpm/bpm_3d.py:_bpm_3d (:104-423)."""
    if mean_mode not in ("ignore", "simple", "weighted"):
        raise NotImplementedError("mean_mode  '%s' unknown" % mean_mode)
    if subsample != 1:
        raise NotImplementedError("subsample still has to be 1")
    if return_g and not return_scattering:
        raise ValueError("return_g requires return_scattering")
    fp32 = precision == "fp32"
    ctype = np.complex64 if fp32 else np.complex128
    rtype = np.float32 if fp32 else np.float64
    w = workers or _workers()

    Nx, Ny, Nz = size
    dx, dy, dz = units
    k0 = 2. * np.pi / lam                                      # :163

    # host H0 (FP64) is only used for the scattering weights: the propagator the march
    # uses is the FP32 compute_propagator output that overwrites H (:192, quirk Q1)
    kxs = 2. * np.pi * np.fft.fftfreq(Nx, dx)
    kys = 2. * np.pi * np.fft.fftfreq(Ny, dy)
    KY, KX = np.meshgrid(kys, kxs, indexing="ij")
    with np.errstate(invalid="ignore"):
        H0 = np.sqrt(n0 ** 2 * k0 ** 2 - KX ** 2 - KY ** 2)
    if use_fresnel_approx:
        H0 = 0.j + n0 * k0 - .5 * (KX ** 2 + KY ** 2) / n0 / k0
    outside = np.isnan(H0)
    H0 = np.where(outside, 0., H0)

    if u0 is None:
        u0 = np.ones((Ny, Nx), np.complex64)
    plane = np.array(u0, dtype=np.complex64).astype(ctype)

    is_complex_dn = False
    dn_dev = None
    if dn is not None:
        dn = np.asarray(dn)
        # the reference uploads dn as complex64 / float16 / float32 (bpm_3d.py:198-211); the
        # FP64 flavour keeps the caller's values (finite differences need them unrounded)
        if dn.dtype.type in (np.complex64, np.complex128):
            is_complex_dn = True
            dn_dev = dn.astype(np.complex64).astype(ctype) if fp32 else dn.astype(ctype)
        elif store_dn_as_half:
            dn_dev = half_to_f32(dn).astype(rtype)
        else:
            dn_dev = dn.astype(np.float32).astype(rtype) if fp32 else dn.astype(rtype)
        if is_complex_dn and mean_mode != "ignore":
            raise NotImplementedError("complex dn is only defined for mean_mode='ignore'")
    dn_mean = np.mean(dn, axis=(1, 2)) if dn is not None else np.zeros(Nz, np.float32)

    unit_k = np.float32(k0 * dz) if fp32 else k0 * dz
    taper = taper_f32(Nx, Ny, absorbing_width).astype(rtype)

    if mean_mode == "ignore":
        if fp32:
            h_ignore, _ = propagator_f32(n0, k0, dx, dy, dz, Nx, Ny)
        else:
            h_ignore, _ = propagator_f64(n0, k0, dx, dy, dz, Nx, Ny)

    if return_scattering:
        cos_theta = np.real(H0) / n0 / k0
        sw = cos_theta.astype(np.float32).astype(rtype)
        gw = (cos_theta ** 2).astype(np.float32).astype(rtype)
        scat = np.zeros(Nz, np.float64)
        gfac = np.zeros(Nz, np.float64)
        plain_wave_dct = (Nx * Ny * np.exp(-1.j * k0 * n0 * (scattering_plane_ind + np.arange(Nz)) * dz)
                          ).astype(np.complex64).astype(ctype)

    if return_full:
        if return_field:
            u = np.empty((Nz, Ny, Nx), ctype)
            u[0] = plane
        else:
            u = np.empty((Nz, Ny, Nx), rtype)
            u[0] = _intens(plane, fp32)

    if dn_dev is not None and mean_mode == "weighted":
        # reduction kernels index dn without a z offset: always slice 0 (quirk Q3)
        dn_flat0 = dn_dev.reshape(-1)[:Nx * Ny].reshape(Ny, Nx)
    else:
        dn_flat0 = np.zeros((Ny, Nx), rtype)

    for i in range(Nz - 1):
        plane = _fft2(plane, w)
        if mean_mode == "simple":
            dn0 = dn_mean[i + 1]
            if fp32:
                # np.float32(n0+dn0) of bpm_3d.py:291, the sum formed in float64
                h, _ = propagator_f32(np.float32(float(n0) + float(dn0)), k0, dx, dy, dz, Nx, Ny)
            else:
                h, _ = propagator_f64(n0 + dn0, k0, dx, dy, dz, Nx, Ny)
        elif mean_mode == "weighted":
            a = np.abs(plane)
            if fp32:
                dn_sum = np.float32(np.sum(a.astype(np.float64) * dn_flat0.astype(np.float64)))
                u_sum = np.float32(np.sum(a.astype(np.float64)))
                dn0 = dn_sum / u_sum
                h, _ = propagator_f32(np.float32(n0) + dn0, k0, dx, dy, dz, Nx, Ny)
            else:
                dn0 = np.sum(a * dn_flat0) / np.sum(a)
                h, _ = propagator_f64(n0 + dn0, k0, dx, dy, dz, Nx, Ny)
        else:
            dn0 = 0.
            h = h_ignore
        plane = plane * h

        if return_scattering:
            diff = plane.copy()
            diff[0, 0] -= plain_wave_dct[i + 1]
            a2 = np.abs(diff).astype(np.float64) ** 2
            scat[i + 1] = np.sum(sw * a2)
            gfac[i + 1] = np.sum(gw * a2)

        plane = _ifft2(plane, w)

        if dn_dev is not None:
            sl = dn_dev[i + 1]
            if is_complex_dn:
                if fp32:
                    re = sl.real.astype(np.float32)
                    im = sl.imag.astype(np.float32)
                    mag = np.exp(unit_k * im).astype(np.float32)
                    ph = (-unit_k) * re
                    plane = plane * ((mag * np.cos(ph)) + 1j * (mag * np.sin(ph))).astype(np.complex64)
                else:
                    plane = plane * np.exp(-1j * unit_k * sl)
            else:
                if fp32:
                    dnd = (-unit_k) * (sl - np.float32(dn0))
                    ph = (np.cos(dnd) + 1j * np.sin(dnd)).astype(np.complex64)
                    plane = (plane * ph) * taper
                else:
                    plane = plane * np.exp(-1j * unit_k * (sl - dn0)) * taper

        if return_full:
            if return_field:
                u[i + 1] = plane
            else:
                u[i + 1] = _intens(plane, fp32)

    if return_full:
        out = u
    else:
        out = plane.copy()
        if not return_field:
            out = _intens(out, fp32)

    result = out
    if return_scattering:
        prefac = 1. / Nx / Ny * dx * dy
        p = (prefac * scat).astype(np.float32)
        if return_g:
            with np.errstate(invalid="ignore", divide="ignore"):
                g = (prefac * gfac / (prefac * scat)).astype(np.float32)
            result = (out, p, g)
        else:
            result = (out, p)
    if return_last_plane:
        if isinstance(result, tuple):
            result = result + (plane.copy(),)
        else:
            result = (result, plane.copy())
    return result


def _intens(plane, fp32):
    a = np.abs(plane)
    return (a * a).astype(np.float32 if fp32 else np.float64)


def _bpm_3d_split(size, units, lam=.5, u0=None, dn=None, n_volumes=1, n0=1., subsample=1,
                  return_scattering=False, return_full=True, return_g=False, return_field=True,
                  absorbing_width=0, use_fresnel_approx=False, store_dn_as_half=False,
                  mean_mode="weighted", precision="fp32", workers=None):
    """Restatement of bpm/bpm/bpm_3d.py:_bpm_3d_split (:863-992): z-chunks of Nz//n+1
    planes with one plane of overlap, the last plane handed on as the next u0."""
    Nx, Ny, Nz = size
    Nz2 = Nz // n_volumes + 1
    if u0 is None:
        u0 = np.ones((subsample * Ny, subsample * Nx), np.complex64)
    fp32 = precision == "fp32"
    if return_field:
        u_dtype = np.complex64 if fp32 else np.complex128
    else:
        u_dtype = np.float32 if fp32 else np.float64
    u = np.empty((Nz, Ny, Nx), u_dtype) if return_full else None
    p = np.empty(Nz, np.float32)
    g = np.empty(Nz, np.float32)
    kw = dict(units=units, lam=lam, n0=n0, subsample=subsample, return_full=return_full,
              return_field=return_field, return_g=return_g, absorbing_width=absorbing_width,
              return_scattering=return_scattering, store_dn_as_half=store_dn_as_half,
              mean_mode=mean_mode, use_fresnel_approx=use_fresnel_approx,
              precision=precision, workers=workers)
    for i in range(n_volumes):
        i1, i2 = i * Nz2, int(np.clip((i + 1) * Nz2, 0, Nz))
        if i < n_volumes - 1:
            dn_part = None if dn is None else dn[i1:i2 + 1]
            res = _bpm_3d((Nx, Ny, i2 - i1 + 1), u0=u0, dn=dn_part, return_last_plane=True,
                          scattering_plane_ind=Nz2 * i, **kw)
            if return_scattering:
                if return_g:
                    u_part, p_part, g_part, u0 = res
                    g[i1:i2] = g_part[1:]
                else:
                    u_part, p_part, u0 = res
                p[i1:i2] = p_part[1:]
            else:
                u_part, u0 = res
            if return_full:
                u[i1:i2] = u_part[:-1]
        else:
            dn_part = None if dn is None else dn[i1:i2]
            res = _bpm_3d((Nx, Ny, i2 - i1), u0=u0, dn=dn_part, scattering_plane_ind=Nz2 * i, **kw)
            if return_scattering:
                if return_g:
                    u_part, p_part, g_part = res
                    g[i1:i2] = g_part
                    g[i1] = g[i1 - 1]
                else:
                    u_part, p_part = res
                p[i1:i2] = p_part
                p[i1] = p[i1 - 1]
            else:
                u_part = res
            if return_full:
                u[i1:i2] = u_part
            else:
                u = u_part
    if return_scattering:
        return (u, p, g) if return_g else (u, p)
    return u


def bpm_3d(size, units, lam=.5, u0=None, dn=None, subsample=1, n_volumes=1, n0=1.,
           return_scattering=False, return_g=False, return_full=True, return_field=True,
           absorbing_width=0, use_fresnel_approx=False, scattering_plane_ind=0,
           store_dn_as_half=False, mean_mode="weighted", precision="fp32", workers=None):
    """Restatement of the bpm_3d dispatcher (bpm/bpm/bpm_3d.py:39-101)."""
    if n_volumes == 1:
        return _bpm_3d(size, units, lam=lam, u0=u0, dn=dn, subsample=subsample, n0=n0,
                       return_scattering=return_scattering, return_full=return_full,
                       return_field=return_field, return_g=return_g,
                       absorbing_width=absorbing_width, use_fresnel_approx=use_fresnel_approx,
                       scattering_plane_ind=scattering_plane_ind,
                       store_dn_as_half=store_dn_as_half, mean_mode=mean_mode,
                       precision=precision, workers=workers)
    return _bpm_3d_split(size, units, lam=lam, u0=u0, dn=dn, n_volumes=n_volumes,
                         subsample=subsample, n0=n0, return_scattering=return_scattering,
                         return_g=return_g, absorbing_width=absorbing_width,
                         return_full=return_full, return_field=return_field,
                         use_fresnel_approx=use_fresnel_approx,
                         store_dn_as_half=store_dn_as_half, mean_mode=mean_mode,
                         precision=precision, workers=workers)


# ----------------------------------------------------------------------------------------
# the object path: Bpm3d (bpm/bpmclass)
# ----------------------------------------------------------------------------------------

def class_propagator(size, units, lam, n0, precision="fp32"):
    """Host FP64 propagator of _Bpm3d_Base._setup (bpm/bpmclass/bpm3d.py:87-109) on the
    intended (Ny, Nx) grid; the class uploads it cast to complex64 (_bpm3d_ocl.py:46)."""
    Nx, Ny, Nz = size
    dx, dy, dz = units
    k0 = 2. * np.pi / lam
    kxs = 2. * np.pi * np.fft.fftfreq(Nx, dx)
    kys = 2. * np.pi * np.fft.fftfreq(Ny, dy)
    KY, KX = np.meshgrid(kys, kxs, indexing="ij")
    with np.errstate(invalid="ignore"):
        H0 = np.sqrt(n0 ** 2 * k0 ** 2 - KX ** 2 - KY ** 2)
    outside = np.isnan(H0)
    H = np.exp(-1.j * dz * np.where(outside, 0., H0))
    H[outside] = 0.
    return H.astype(np.complex64) if precision == "fp32" else H


def bpm3d_propagate(size, units, lam=.5, n0=1., dn=None, u0=None, return_full=True,
                    return_intensity=False, absorbing_width=0, precision="fp32", workers=None):
    """Restatement of _Bpm3d_OCL._propagate_single (bpm/bpmclass/_bpm3d_ocl.py:66-134):
    fft -> mult(H) -> ifft -> mult_dn (taper) | mult_dn_complex (no taper) -> store.
    return_intensity stores |u|^2 (the reference names a missing kernel, fill_with_energy)."""
    fp32 = precision == "fp32"
    ctype = np.complex64 if fp32 else np.complex128
    rtype = np.float32 if fp32 else np.float64
    w = workers or _workers()
    Nx, Ny, Nz = size
    dx, dy, dz = units
    k0 = 2. * np.pi / lam
    H = class_propagator(size, units, lam, n0, precision)
    if u0 is None:
        u0 = np.ones((Ny, Nx), np.complex64)
    plane = np.array(u0, dtype=np.complex64).astype(ctype)
    is_complex = dn is not None and np.iscomplexobj(dn)
    if dn is not None:
        dn = np.asarray(dn).astype(np.complex64 if is_complex else np.float32).astype(
            ctype if is_complex else rtype)
    unit_k = np.float32(k0 * dz) if fp32 else k0 * dz
    taper = taper_f32(Nx, Ny, absorbing_width).astype(rtype)
    if return_full:
        if return_intensity:
            u = np.empty((Nz, Ny, Nx), rtype)
            u[0] = _intens(plane, fp32)
        else:
            u = np.empty((Nz, Ny, Nx), ctype)
            u[0] = plane
    for i in range(Nz - 1):
        plane = _ifft2(_fft2(plane, w) * H, w)
        if dn is not None:
            sl = dn[i + 1]
            if is_complex:
                if fp32:
                    mag = np.exp(unit_k * sl.imag.astype(np.float32)).astype(np.float32)
                    ph = (-unit_k) * sl.real.astype(np.float32)
                    plane = plane * ((mag * np.cos(ph)) + 1j * (mag * np.sin(ph))).astype(np.complex64)
                else:
                    plane = plane * np.exp(-1j * unit_k * sl)
            else:
                if fp32:
                    dnd = (-unit_k) * sl
                    plane = (plane * (np.cos(dnd) + 1j * np.sin(dnd)).astype(np.complex64)) * taper
                else:
                    plane = plane * np.exp(-1j * unit_k * sl) * taper
        if return_full:
            u[i + 1] = _intens(plane, fp32) if return_intensity else plane
    return u if return_full else plane.copy()


def rel_l2(a, b):
    """||a-b||_2 / ||b||_2 in FP64 over the whole array."""
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))
