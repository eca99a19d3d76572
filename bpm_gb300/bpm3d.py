"""Split-step beam propagation: the drop-in host API.

Mirrors the reference's functional driver bpm/bpm/bpm_3d.py (bpm_3d :39-101,
_bpm_3d :104-423, _bpm_3d_split :863-992) and its object API bpm/bpmclass
(Bpm3d factory bpm3d.py:146-167, _Bpm3d_Base :24-141, _Bpm3d_OCL._propagate_single
_bpm3d_ocl.py:66-134): same names, arguments, array layouts, return values and error
types. Every z-step runs in libbpm_gb300.so (bpm_propagate); this module only moves
buffers, builds plans and shapes results.

Inputs may be numpy arrays (results come back as numpy arrays, as in the reference) or
torch CUDA tensors (results stay on the device as tensors). Additions with no reference
counterpart: `bpm_3d_batched` and `Bpm3d.propagate_batched` march many fields through one
dn volume in one launch sequence, and `BatchedMarch` replays a captured CUDA graph.
"""
import ctypes
from collections import OrderedDict

import numpy as np
import torch

from . import _native as N

__all__ = ["bpm_3d", "bpm_3d_batched", "Bpm3d", "BatchedMarch", "MixedBatch", "Plan", "get_plan"]


# ----------------------------------------------------------------------------------------
# device helpers
# ----------------------------------------------------------------------------------------

def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("bpm_gb300 needs a CUDA device (none is visible)")
    return torch.device("cuda", torch.cuda.current_device())


def _stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _is_tensor(a):
    return isinstance(a, torch.Tensor)


_PIN_MIN = 1 << 20


def _h2d(a, dtype, dev):
    """numpy/tensor -> contiguous CUDA tensor of `dtype` (pinned staging for large arrays)."""
    if _is_tensor(a):
        t = a.to(device=dev, dtype=dtype)
        return t.contiguous()
    npdt = {torch.complex64: np.complex64, torch.float32: np.float32, torch.float16: np.float16}[dtype]
    a = np.ascontiguousarray(np.asarray(a).astype(npdt, copy=False))
    src = torch.from_numpy(a)
    if a.nbytes >= _PIN_MIN:
        st = torch.empty(src.shape, dtype=dtype, pin_memory=True)
        st.copy_(src)
        return st.to(dev, non_blocking=True)
    return src.to(dev)


def _d2h(t):
    """CUDA tensor -> numpy array (through a pinned host buffer)."""
    if t.numel() * t.element_size() >= _PIN_MIN:
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return h.numpy()
    return t.cpu().numpy()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


# ----------------------------------------------------------------------------------------
# plans
# ----------------------------------------------------------------------------------------

class Plan:
    """A propagation plan: grid, propagator, twiddle, taper and scattering tables on one
    device (bpm_plan_create). It holds what the setup of _bpm_3d builds per call
    (bpm/bpm/bpm_3d.py:140-278: k-grid, propagator and evanescent mask, taper, scattering
    weights), or for prop_kind PROP_CLASS the class path's host FP64 propagator
    (bpm/bpmclass/bpm3d.py:64-115)."""

    def __init__(self, size, units, lam, n0, absorbing_width=0, mean_mode="weighted",
                 prop_kind=N.PROP_FUNCTIONAL, use_fresnel_approx=False, base=None):
        if mean_mode not in N.MEAN_MODES:
            raise NotImplementedError("mean_mode  '%s' unknown" % mean_mode)
        Nx, Ny, Nz = (int(s) for s in size)
        dx, dy, dz = (float(u) for u in units)
        self.size = (Nx, Ny, Nz)
        self.units = (dx, dy, dz)
        self.lam = float(lam)
        self.n0 = float(n0)
        self.mean_mode = mean_mode
        self.desc = N.GridDesc(Nx, Ny, Nz, dx, dy, dz, float(lam), float(n0), int(absorbing_width),
                               N.MEAN_MODES[mean_mode], int(prop_kind), int(bool(use_fresnel_approx)))
        L = N.lib()
        N.check(L.bpm_grid_check(ctypes.byref(self.desc)), "bpm_grid_check")
        self.device = _device()
        self._base = base  # a derived plan shares (and keeps alive) its base's tables
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            if base is not None:
                N.check(L.bpm_plan_derive(base.handle, Nz, ctypes.byref(h)), "bpm_plan_derive")
            else:
                N.check(L.bpm_plan_create(ctypes.byref(self.desc), ctypes.byref(h)), "bpm_plan_create")
        self.handle = h

    def workspace_bytes(self, batch, group=0, conc=0):
        return int(N.lib().bpm_workspace_bytes_conc(self.handle, int(batch), int(group), int(conc)))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                N.lib().bpm_plan_destroy(h)
            except Exception:
                pass
            self.handle = None


_plans = OrderedDict()       # (grid incl. nz) -> Plan
_bases = OrderedDict()       # (grid without nz) -> Plan that owns the device tables
_PLAN_CACHE = 64
_BASE_CACHE = 16


def get_plan(size, units, lam, n0, absorbing_width=0, mean_mode="weighted",
             prop_kind=N.PROP_FUNCTIONAL, use_fresnel_approx=False):
    """Cached plan for this grid and physics. The device tables do not depend on Nz: one
    base plan per (Nx, Ny, units, physics) builds them, and a request with another Nz gets
    a derived plan (bpm_plan_derive) that shares them, created without any device
    allocation or synchronisation."""
    Nx, Ny, Nz = (int(s) for s in size)
    dev = torch.cuda.current_device() if torch.cuda.is_available() else -1
    rest = (tuple(float(u) for u in units), float(lam), float(n0), int(absorbing_width), mean_mode,
            int(prop_kind), bool(use_fresnel_approx))
    key = (dev, (Nx, Ny, Nz)) + rest
    p = _plans.get(key)
    if p is not None:
        _plans.move_to_end(key)
        return p
    bkey = (dev, (Nx, Ny)) + rest
    base = _bases.get(bkey)
    if base is None:
        p = Plan(size, units, lam, n0, absorbing_width, mean_mode, prop_kind, use_fresnel_approx)
        _bases[bkey] = p
        while len(_bases) > _BASE_CACHE:
            _bases.popitem(last=False)
    else:
        _bases.move_to_end(bkey)
        p = Plan(size, units, lam, n0, absorbing_width, mean_mode, prop_kind, use_fresnel_approx, base=base)
    _plans[key] = p
    while len(_plans) > _PLAN_CACHE:
        _plans.popitem(last=False)
    return p


# ----------------------------------------------------------------------------------------
# one launch sequence over a batch of fields
# ----------------------------------------------------------------------------------------

def _dn_kind(dn, store_dn_as_half):
    if dn is None:
        return N.DN_NONE, None
    if _is_tensor(dn):
        if dn.is_complex():
            return N.DN_C64, torch.complex64
    elif np.iscomplexobj(dn):
        return N.DN_C64, torch.complex64
    if store_dn_as_half:
        return N.DN_F16, torch.float16
    return N.DN_F32, torch.float32


def _slice_tables(dn, n0, dev):
    """Per-slice float32(n0 + mean(dn[z])) and float32(mean(dn[z])) for mean_mode='simple'
    (bpm_3d.py:216-220, :288-293): the slice means are taken on the caller's dn, in FP64."""
    if dn is None:
        m = np.zeros(1, np.float64)
    elif _is_tensor(dn):
        m = dn.to(torch.float64).mean(dim=(1, 2)).cpu().numpy()
    else:
        m = np.asarray(np.mean(dn, axis=(1, 2)), np.float64)
    sn = np.float32(float(n0) + m)
    sd = m.astype(np.float32)
    return (torch.from_numpy(np.ascontiguousarray(sn, np.float32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(sd, np.float32)).to(dev))


def mask_pays(batch, Nx, Ny):
    """Whether a march of `batch` fields through one shared dn volume computes its phase
    masks once up front (precompute_mask) instead of per element in every row pass. The
    results are the same bits either way. It pays for several fields, and for one field on
    every grid measured, where the row pass stages one mask row instead of evaluating
    exp/sincos per element (GB300, one field, precompute included, per-element -> mask:
    Nz 128 ignore with complex dn 1024^2 4.74 -> 3.55 ms, 512^2 1.70 -> 1.23, 256^2 0.84 ->
    0.74, 128^2 0.89 -> 0.81; weighted 1024^2 6.04 -> 5.01, 512^2 (Nz 256) 5.78 -> 4.57,
    256^2 1.51 -> 1.38, 128^2 1.20 -> 1.13, 64^2 (Nz 64) 0.419 -> 0.405). Below 64x64 it
    stays per element (not measured)."""
    return batch >= 2 or Nx * Ny >= 64 * 64


def precompute_mask(plan, dn_t, dn_kind):
    """Phase masks (Nz, Ny, Nx) complex64 of a shared dn volume (bpm_mask_precompute): every
    field then reads them instead of re-evaluating exp(-i k0 dz dn) (see mask_pays). The
    mask is the factor the reference's mult_dn* kernels apply per step
    (bpm/bpm/kernels/bpm_3d_kernels.cl:20-283) without the mean-index shift, which stays
    per field."""
    Nx, Ny, Nz = plan.size
    mask = torch.empty((Nz, Ny, Nx), dtype=torch.complex64, device=dn_t.device)
    N.check(N.lib().bpm_mask_precompute(plan.handle, _ptr(dn_t), dn_kind, _ptr(mask), _stream_ptr()),
            "bpm_mask_precompute")
    return mask


def _apply_launch(req, launch):
    """Set the launch-shape fields of a request from a dict with keys conc, col_block,
    cluster, col_fuse (absent or 0: the library's rule; see bpm_request in
    include/bpm_gb300.h)."""
    if launch:
        req.conc = int(launch.get("conc", 0))
        req.col_block = int(launch.get("col_block", 0))
        req.cluster = int(launch.get("cluster", 0))
        req.col_fuse = int(launch.get("col_fuse", 0))
    return req


def _run(plan, u0_t, dn_t, dn_kind, dn_bstride, out_kind, want_last=True, scattering=False,
         return_g=False, scattering_plane_ind=0, slice_tabs=(None, None), group=0, mask=None, launch=None):
    """Launch bpm_propagate on the current stream. u0_t: (B, Ny, Nx) complex64 CUDA tensor."""
    Nx, Ny, Nz = plan.size
    B = u0_t.shape[0]
    dev = u0_t.device
    out = None
    if out_kind == N.OUT_FIELD:
        out = torch.empty((B, Nz, Ny, Nx), dtype=torch.complex64, device=dev)
    elif out_kind == N.OUT_INTENSITY:
        out = torch.empty((B, Nz, Ny, Nx), dtype=torch.float32, device=dev)
    last = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev) if want_last else None
    p = torch.empty((B, Nz), dtype=torch.float32, device=dev) if scattering else None
    g = torch.empty((B, Nz), dtype=torch.float32, device=dev) if (scattering and return_g) else None
    wsb = plan.workspace_bytes(B, group, (launch or {}).get("conc", 0))
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    req = N.Request(B, _ptr(u0_t), _ptr(dn_t), dn_kind, int(dn_bstride), _ptr(slice_tabs[0]),
                    _ptr(slice_tabs[1]), _ptr(out), out_kind, Nz * Ny * Nx, _ptr(last), _ptr(p),
                    _ptr(g), int(scattering_plane_ind), int(group), None, 0, _ptr(mask))
    _apply_launch(req, launch)
    N.check(N.lib().bpm_propagate(plan.handle, ctypes.byref(req), _ptr(ws), wsb, _stream_ptr()),
            "bpm_propagate")
    return out, last, p, g


def _check_shapes(size, u0, dn):
    Nx, Ny, Nz = size
    if u0 is not None and tuple(u0.shape[-2:]) != (Ny, Nx):
        raise ValueError("u0 has shape %s, expected (..., %d, %d)" % (tuple(u0.shape), Ny, Nx))
    if dn is not None and tuple(dn.shape) != (Nz, Ny, Nx):
        raise ValueError("dn has shape %s, expected (Nz, Ny, Nx) = %s" % (tuple(dn.shape), (Nz, Ny, Nx)))


# ----------------------------------------------------------------------------------------
# functional API (bpm/bpm/bpm_3d.py)
# ----------------------------------------------------------------------------------------

def bpm_3d(size, units, lam=.5, u0=None, dn=None, subsample=1, n_volumes=1, n0=1.,
           return_scattering=False, return_g=False, return_full=True, return_field=True,
           absorbing_width=0, use_fresnel_approx=False, scattering_plane_ind=0,
           store_dn_as_half=False, mean_mode="weighted"):
    """Simulates the propagation of a monochromatic wave of wavelength lam with initial
    field u0 along z through a medium of refractive index n0 + dn (bpm/bpm/bpm_3d.py:39).

    size = (Nx, Ny, Nz) pixels; units = (dx, dy, dz) microns; u0 (Ny, Nx) complex
    (None = plane wave); dn (Nz, Ny, Nx) real or complex; mean_mode "weighted" (default),
    "simple" or "ignore". Returns the (Nz, Ny, Nx) complex field (return_field) or |u|^2
    volume, or only the last plane (return_full=False), plus (p[, g]) when
    return_scattering. n_volumes > 1 splits z into chunks as the reference does.
    """
    if n_volumes == 1:
        return _bpm_3d(size, units, lam=lam, u0=u0, dn=dn, subsample=subsample, n0=n0,
                       return_scattering=return_scattering, return_full=return_full,
                       return_field=return_field, return_g=return_g, absorbing_width=absorbing_width,
                       use_fresnel_approx=use_fresnel_approx,
                       scattering_plane_ind=scattering_plane_ind,
                       store_dn_as_half=store_dn_as_half, mean_mode=mean_mode)
    return _bpm_3d_split(size, units, lam=lam, u0=u0, dn=dn, n_volumes=n_volumes, subsample=subsample,
                         n0=n0, return_scattering=return_scattering, return_g=return_g,
                         absorbing_width=absorbing_width, return_full=return_full,
                         return_field=return_field, use_fresnel_approx=use_fresnel_approx,
                         store_dn_as_half=store_dn_as_half, mean_mode=mean_mode)


def _validate(mean_mode, subsample, return_scattering, return_g):
    if mean_mode not in N.MEAN_MODES:
        raise NotImplementedError("mean_mode  '%s' unknown" % mean_mode)
    if subsample != 1:
        raise NotImplementedError("subsample still has to be 1")
    if return_g and not return_scattering:
        raise ValueError("return_g requires return_scattering")


def _bpm_3d(size, units, lam=.5, u0=None, dn=None, subsample=1, n0=1.,
            return_scattering=False, return_g=False, return_full=True, return_field=True,
            use_fresnel_approx=False, absorbing_width=0, scattering_plane_ind=0,
            return_last_plane=False, store_dn_as_half=False, mean_mode="weighted"):
    """One march over all of z (bpm/bpm/bpm_3d.py:_bpm_3d :104-423)."""
    _validate(mean_mode, subsample, return_scattering, return_g)
    Nx, Ny, Nz = (int(s) for s in size)
    _check_shapes((Nx, Ny, Nz), u0, dn)
    as_tensor = _is_tensor(u0) or _is_tensor(dn)
    dev = _device()
    plan = get_plan((Nx, Ny, Nz), units, lam, n0, absorbing_width, mean_mode, N.PROP_FUNCTIONAL,
                    use_fresnel_approx)
    if u0 is None:
        u0_t = torch.ones((1, Ny, Nx), dtype=torch.complex64, device=dev)
    else:
        u0_t = _h2d(u0, torch.complex64, dev).reshape(1, Ny, Nx)
    kind, tdt = _dn_kind(dn, store_dn_as_half)
    if kind == N.DN_C64 and mean_mode != "ignore":
        raise NotImplementedError("complex dn is only defined for mean_mode='ignore' "
                                  "(the reference mixes buffer types in the other modes)")
    dn_t = _h2d(dn, tdt, dev) if dn is not None else None
    tabs = _slice_tables(dn, n0, dev) if mean_mode == "simple" else (None, None)
    if mean_mode == "simple" and dn is None:
        tabs = (tabs[0].expand(Nz).contiguous(), tabs[1].expand(Nz).contiguous())
    out_kind = (N.OUT_FIELD if return_field else N.OUT_INTENSITY) if return_full else N.OUT_NONE
    mask = precompute_mask(plan, dn_t, kind) if (dn_t is not None and mask_pays(1, Nx, Ny)) else None
    out, last, p, g = _run(plan, u0_t, dn_t, kind, 0, out_kind, True, return_scattering, return_g,
                           scattering_plane_ind, tabs, mask=mask)
    conv = (lambda t: t) if as_tensor else _d2h
    if return_full:
        res = conv(out[0])
    else:
        lp = last[0]
        res = conv(lp if return_field else (lp.abs() ** 2))
    result = res
    if return_scattering:
        result = (res, conv(p[0]), conv(g[0])) if return_g else (res, conv(p[0]))
    if return_last_plane:
        lp = conv(last[0])
        result = result + (lp,) if isinstance(result, tuple) else (result, lp)
    return result


def _bpm_3d_split(size, units, lam=.5, u0=None, dn=None, n_volumes=1, n0=1., subsample=1,
                  return_scattering=False, return_full=True, return_g=False, return_field=True,
                  absorbing_width=0, use_fresnel_approx=False, store_dn_as_half=False,
                  mean_mode="weighted"):
    """z-chunked march (bpm/bpm/bpm_3d.py:_bpm_3d_split :863-992): chunks of Nz//n+1 planes
    with one plane of overlap, the last plane of a chunk handed on as the next u0. The
    per-chunk reference semantics are kept (in "weighted" mode each chunk reduces over its
    own first dn slice, so results depend on n_volumes as in the reference)."""
    Nx, Ny, Nz = (int(s) for s in size)
    Nz2 = Nz // n_volumes + 1
    as_tensor = _is_tensor(u0) or _is_tensor(dn)
    if u0 is None:
        u0 = np.ones((subsample * Ny, subsample * Nx), np.complex64)
    if return_field:
        u_dtype = np.complex64
    else:
        u_dtype = np.float32
    u = None
    if return_full:
        u = (torch.empty((Nz, Ny, Nx), dtype=torch.complex64 if return_field else torch.float32,
                         device=_device()) if as_tensor else np.empty((Nz, Ny, Nx), u_dtype))
    p = np.empty(Nz, np.float32) if not as_tensor else torch.empty(Nz, device=_device())
    g = np.empty(Nz, np.float32) if not as_tensor else torch.empty(Nz, device=_device())
    kw = dict(units=units, lam=lam, n0=n0, subsample=subsample, return_full=return_full,
              return_field=return_field, return_g=return_g, absorbing_width=absorbing_width,
              return_scattering=return_scattering, store_dn_as_half=store_dn_as_half,
              mean_mode=mean_mode, use_fresnel_approx=use_fresnel_approx)
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


def bpm_3d_batched(size, units, lam=.5, u0=None, dn=None, n0=1., return_full=True, return_field=True,
                   absorbing_width=0, use_fresnel_approx=False, store_dn_as_half=False,
                   mean_mode="weighted", group=0, out=None, launch=None):
    """Batched bpm_3d (bpm/bpm/bpm_3d.py:39, once per field): u0 of shape (B, Ny, Nx)
    marches through one shared dn (Nz, Ny, Nx),
    or through per-field dn volumes of shape (B, Nz, Ny, Nx). Each field's result equals
    bpm_3d on that field alone. Returns (B, Nz, Ny, Nx) volumes or (B, Ny, Nx) last planes.
    `out`, if given, is a host buffer of the result's shape and dtype (a numpy array or a
    CPU tensor, ideally pinned) that receives the result and is returned. `launch`: a
    launch shape (keys group, conc, col_block, cluster; autotune.tune_shape gives one) that
    never changes the result's bits except cluster at 64x64.
    No counterpart in the reference, which marches one field per call."""
    if launch and not group:
        group = int(launch.get("group", 0))
    _validate(mean_mode, 1, False, False)
    Nx, Ny, Nz = (int(s) for s in size)
    as_tensor = _is_tensor(u0) or _is_tensor(dn)
    dev = _device()
    plan = get_plan((Nx, Ny, Nz), units, lam, n0, absorbing_width, mean_mode, N.PROP_FUNCTIONAL,
                    use_fresnel_approx)
    u0_t = _h2d(u0, torch.complex64, dev)
    if u0_t.dim() == 2:
        u0_t = u0_t.reshape(1, Ny, Nx)
    B = u0_t.shape[0]
    _check_shapes((Nx, Ny, Nz), u0_t, None)
    kind, tdt = _dn_kind(dn, store_dn_as_half)
    if kind == N.DN_C64 and mean_mode != "ignore":
        raise NotImplementedError("complex dn is only defined for mean_mode='ignore'")
    dn_t, bstride = None, 0
    if dn is not None:
        dn_t = _h2d(dn, tdt, dev)
        if dn_t.dim() == 4:
            if tuple(dn_t.shape) != (B, Nz, Ny, Nx):
                raise ValueError("per-field dn must have shape (B, Nz, Ny, Nx)")
            bstride = Nz * Ny * Nx
        else:
            _check_shapes((Nx, Ny, Nz), None, dn_t)
    if mean_mode == "simple":
        if dn_t is not None and dn_t.dim() == 4:
            raise NotImplementedError("mean_mode='simple' needs one shared dn volume")
        tabs = _slice_tables(dn, n0, dev)
        if dn is None:
            tabs = (tabs[0].expand(Nz).contiguous(), tabs[1].expand(Nz).contiguous())
    else:
        tabs = (None, None)
    out_kind = (N.OUT_FIELD if return_field else N.OUT_INTENSITY) if return_full else N.OUT_NONE
    mask = precompute_mask(plan, dn_t, kind) if (dn_t is not None and bstride == 0 and mask_pays(B, Nx, Ny)) else None
    if out is not None and return_full:
        host = torch.from_numpy(out) if isinstance(out, np.ndarray) else out
        vdt = torch.complex64 if return_field else torch.float32
        if tuple(host.shape) != (B, Nz, Ny, Nx) or host.dtype != vdt:
            raise ValueError("out must have shape %s and dtype %s" % ((B, Nz, Ny, Nx), vdt))
        if host.is_contiguous() and host.is_pinned():
            _run_streamed_to_host(plan, u0_t, dn_t, kind, bstride, out_kind, tabs, group, mask, host, launch=launch)
        else:
            _run_to_host(plan, u0_t, dn_t, kind, bstride, out_kind, tabs, group, mask, host, launch=launch)
        return out
    vol, last, _, _ = _run(plan, u0_t, dn_t, kind, bstride, out_kind, True, slice_tabs=tabs, group=group,
                           mask=mask, launch=launch)
    res = vol if return_full else (last if return_field else last.abs() ** 2)
    if out is not None:
        host = torch.from_numpy(out) if isinstance(out, np.ndarray) else out
        if tuple(host.shape) != tuple(res.shape) or host.dtype != res.dtype:
            raise ValueError("out must have shape %s and dtype %s" % (tuple(res.shape), res.dtype))
        host.copy_(res, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out
    return res if as_tensor else _d2h(res)


def _run_streamed_to_host(plan, u0_t, dn_t, kind, bstride, out_kind, tabs, group, mask, host, chunk_planes=16,
                          launch=None):
    """March the whole batch into a device volume while the library's copy stream moves
    each finished run of `chunk_planes` planes into the page-locked host buffer
    (bpm_propagate_to_host), so the device->host copy runs alongside the march."""
    Nx, Ny, Nz = plan.size
    B = u0_t.shape[0]
    dev = u0_t.device
    vdt = torch.complex64 if out_kind == N.OUT_FIELD else torch.float32
    vol = torch.empty((B, Nz, Ny, Nx), dtype=vdt, device=dev)
    last = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev)
    wsb = plan.workspace_bytes(B, group, (launch or {}).get("conc", 0))
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    req = N.Request(B, _ptr(u0_t), _ptr(dn_t), kind, int(bstride), _ptr(tabs[0]), _ptr(tabs[1]), _ptr(vol),
                    out_kind, Nz * Ny * Nx, _ptr(last), None, None, 0, int(group), None, 0, _ptr(mask))
    _apply_launch(req, launch)
    N.check(N.lib().bpm_propagate_to_host(plan.handle, ctypes.byref(req), ctypes.c_void_p(host.data_ptr()),
                                          int(chunk_planes), _ptr(ws), wsb, _stream_ptr()),
            "bpm_propagate_to_host")
    torch.cuda.current_stream().synchronize()


def _run_to_host(plan, u0_t, dn_t, kind, bstride, out_kind, tabs, group, mask, host, launch=None):
    """March a batch in chunks of fields into two alternating device volumes while a copy
    stream drains the previous chunk to the host buffer, so the device->host copy of the
    output volumes overlaps the march of the next chunk."""
    Nx, Ny, Nz = plan.size
    B = u0_t.shape[0]
    dev = u0_t.device
    G = int(N.lib().bpm_group_size(plan.handle, B, int(group)))
    chunk = max(G, -(-B // 4))
    chunk = -(-chunk // G) * G
    vdt = torch.complex64 if out_kind == N.OUT_FIELD else torch.float32
    bufs = [torch.empty((min(chunk, B), Nz, Ny, Nx), dtype=vdt, device=dev) for _ in range(2 if B > chunk else 1)]
    last = torch.empty((min(chunk, B), Ny, Nx), dtype=torch.complex64, device=dev)
    wsb = plan.workspace_bytes(min(chunk, B), group, (launch or {}).get("conc", 0))
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    cs = torch.cuda.current_stream()
    copy_s = torch.cuda.Stream(device=dev)
    copied = [None, None]
    for k, b0 in enumerate(range(0, B, chunk)):
        nb = min(chunk, B - b0)
        buf = bufs[k % len(bufs)]
        if copied[k % 2] is not None:
            cs.wait_event(copied[k % 2])          # the copy out of this buffer has finished
        dn_k = dn_t[b0:b0 + nb] if (dn_t is not None and bstride) else dn_t
        req = N.Request(nb, _ptr(u0_t[b0:b0 + nb]), _ptr(dn_k), kind, int(bstride), _ptr(tabs[0]),
                        _ptr(tabs[1]), _ptr(buf), out_kind, Nz * Ny * Nx, _ptr(last), None, None, 0,
                        int(group), None, 0, _ptr(mask))
        _apply_launch(req, launch)
        N.check(N.lib().bpm_propagate(plan.handle, ctypes.byref(req), _ptr(ws), wsb, _stream_ptr()),
                "bpm_propagate")
        done = torch.cuda.Event()
        done.record(cs)
        copy_s.wait_event(done)
        with torch.cuda.stream(copy_s):
            host[b0:b0 + nb].copy_(buf[:nb], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(copy_s)
        copied[k % 2] = ev
    copy_s.synchronize()
    cs.synchronize()


class BatchedMarch:
    """A fixed batched march with resident buffers, captured once as a CUDA graph
    (bpm_exec_create) and replayed by run(). Inputs u0 (B, Ny, Nx) and dn live on the
    device; outputs are `out` (B, Nz, Ny, Nx) and `last` (B, Ny, Nx)."""

    def __init__(self, size, units, lam, n0, batch, dn=None, mean_mode="weighted", absorbing_width=0,
                 out_kind="intensity", prop_kind=N.PROP_FUNCTIONAL, group=0, store_dn_as_half=False,
                 use_graph=True, use_mask=True, launch=None):
        dev = _device()
        Nx, Ny, Nz = (int(s) for s in size)
        self.size = (Nx, Ny, Nz)
        self.batch = int(batch)
        self.plan = get_plan(self.size, units, lam, n0, absorbing_width, mean_mode, prop_kind)
        self.u0 = torch.ones((batch, Ny, Nx), dtype=torch.complex64, device=dev)
        kind, tdt = _dn_kind(dn, store_dn_as_half)
        self.dn_kind = kind
        self.dn = _h2d(dn, tdt, dev) if dn is not None else None
        self.dn_bstride = Nz * Ny * Nx if (self.dn is not None and self.dn.dim() == 4) else 0
        self.tabs = _slice_tables(dn, n0, dev) if mean_mode == "simple" else (None, None)
        ok = {"field": N.OUT_FIELD, "intensity": N.OUT_INTENSITY, "none": N.OUT_NONE}[out_kind]
        self.out_kind = ok
        self.out = None
        if ok == N.OUT_FIELD:
            self.out = torch.empty((batch, Nz, Ny, Nx), dtype=torch.complex64, device=dev)
        elif ok == N.OUT_INTENSITY:
            self.out = torch.empty((batch, Nz, Ny, Nx), dtype=torch.float32, device=dev)
        self.last = torch.empty((batch, Ny, Nx), dtype=torch.complex64, device=dev)
        # group="auto": the autotuner's launch shape (fields per launch, concurrent groups,
        # column block, cluster kernel) for this device, grid, batch and mode
        if group == "auto":
            from .autotune import tune_shape
            launch = tune_shape(self.size, units, lam, n0, batch, dn if dn is None else self.dn, mean_mode,
                                out_kind, absorbing_width)
            group = launch["group"]
        self.launch = dict(launch or {})
        self.launch["group"] = int(group)
        self.group = int(group)
        self.group_used = int(N.lib().bpm_group_size(self.plan.handle, self.batch, self.group))
        self.ws_bytes = self.plan.workspace_bytes(batch, group, self.launch.get("conc", 0))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        # the phase masks of a shared dn are computed once and reused by every run
        self.mask = (precompute_mask(self.plan, self.dn, kind)
                     if (self.dn is not None and self.dn_bstride == 0 and use_mask) else None)
        self.req = N.Request(self.batch, _ptr(self.u0), _ptr(self.dn), kind, self.dn_bstride,
                             _ptr(self.tabs[0]), _ptr(self.tabs[1]), _ptr(self.out), ok,
                             Nz * Ny * Nx, _ptr(self.last), None, None, 0, self.group, None, 0,
                             _ptr(self.mask))
        _apply_launch(self.req, self.launch)
        self.exec = None
        if use_graph:
            torch.cuda.synchronize()
            h = ctypes.c_void_p()
            N.check(N.lib().bpm_exec_create(self.plan.handle, ctypes.byref(self.req), _ptr(self.ws),
                                            self.ws_bytes, ctypes.byref(h)), "bpm_exec_create")
            self.exec = h

    def run(self, stream=None):
        s = ctypes.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        if self.exec is not None:
            N.check(N.lib().bpm_exec_launch(self.exec, s), "bpm_exec_launch")
        else:
            N.check(N.lib().bpm_propagate(self.plan.handle, ctypes.byref(self.req), _ptr(self.ws),
                                          self.ws_bytes, s), "bpm_propagate")

    def __del__(self):
        h = getattr(self, "exec", None)
        if h is not None and h.value:
            try:
                N.lib().bpm_exec_destroy(h)
            except Exception:
                pass
            self.exec = None


class MixedBatch:
    """Marches of different grids, wavelengths, refractive indices and illuminations replayed
    as one CUDA graph (one launch). Requests (objects with the fields of
    bpm_gb300.serve.BpmRequest: size, units, lam, n0, u0, dn, mean_mode, absorbing_width)
    that share a grid, physics and dn volume march together as one batched group with
    resident buffers (phase masks precomputed where mask_pays); every group runs on its own
    stream, captured as a parallel branch of the graph, so run() launches them all at once.
    Each request's |u|^2 volume (out_kind "intensity") or field volume ("field") is result(i);
    its exit field last(i). A group is bit-identical to the same requests marched alone."""

    def __init__(self, requests, out_kind="intensity", use_graph=True, tune=False):
        dev = _device()
        ok = {"field": N.OUT_FIELD, "intensity": N.OUT_INTENSITY}[out_kind]
        self.requests = list(requests)
        groups = {}
        for i, r in enumerate(self.requests):
            if r.mean_mode == "simple":
                raise NotImplementedError("MixedBatch: mean_mode 'simple' (per-request slice tables) is not batched")
            # the same dn volume: the same device memory (views of one tensor alike), or the
            # same host array object
            dn_id = ((r.dn.data_ptr(), tuple(r.dn.shape), r.dn.dtype) if _is_tensor(r.dn) else id(r.dn))
            key = (tuple(int(v) for v in r.size), tuple(float(u) for u in r.units), float(r.lam), float(r.n0),
                   r.mean_mode, int(r.absorbing_width), dn_id)
            groups.setdefault(key, []).append(i)
        self.where = [None] * len(self.requests)  # request -> (group, index in group)
        self.groups = []
        for gi, (key, idx) in enumerate(groups.items()):
            r0 = self.requests[idx[0]]
            Nx, Ny, Nz = (int(v) for v in r0.size)
            B = len(idx)
            plan = get_plan((Nx, Ny, Nz), r0.units, r0.lam, r0.n0, r0.absorbing_width, r0.mean_mode,
                            N.PROP_FUNCTIONAL)
            u0 = torch.ones((B, Ny, Nx), dtype=torch.complex64, device=dev)
            for k, i in enumerate(idx):
                if self.requests[i].u0 is not None:
                    u0[k].copy_(_h2d(self.requests[i].u0, torch.complex64, dev).reshape(Ny, Nx))
            kind, tdt = _dn_kind(r0.dn, False)
            if kind == N.DN_C64 and r0.mean_mode != "ignore":
                raise NotImplementedError("complex dn is only defined for mean_mode='ignore'")
            dn = _h2d(r0.dn, tdt, dev) if r0.dn is not None else None
            if dn is not None:
                _check_shapes((Nx, Ny, Nz), None, dn)
            mask = precompute_mask(plan, dn, kind) if (dn is not None and mask_pays(B, Nx, Ny)) else None
            shape = (B, Nz, Ny, Nx)
            out = torch.empty(shape, dtype=torch.complex64 if ok == N.OUT_FIELD else torch.float32, device=dev)
            last = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev)
            launch = {}
            if tune:
                from .autotune import tune_shape
                launch = tune_shape((Nx, Ny, Nz), r0.units, r0.lam, r0.n0, B, dn, r0.mean_mode, out_kind,
                                    r0.absorbing_width)
            wsb = plan.workspace_bytes(B, launch.get("group", 0), launch.get("conc", 0))
            ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
            req = N.Request(B, _ptr(u0), _ptr(dn), kind, 0, None, None, _ptr(out), ok, Nz * Ny * Nx, _ptr(last),
                            None, None, 0, int(launch.get("group", 0)), None, 0, _ptr(mask))
            _apply_launch(req, launch)
            self.groups.append(dict(plan=plan, u0=u0, dn=dn, mask=mask, out=out, last=last, ws=ws, wsb=wsb,
                                    req=req, stream=torch.cuda.Stream(device=dev), launch=launch))
            for k, i in enumerate(idx):
                self.where[i] = (gi, k)
        torch.cuda.synchronize()
        self.graph = None
        if use_graph:
            self._enqueue()  # first run eagerly: plans' kernels prepared outside the capture
            torch.cuda.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            cs = torch.cuda.Stream(device=dev)
            with torch.cuda.graph(self.graph, stream=cs):
                self._enqueue()

    def _enqueue(self):
        """Every group's march on its own stream, forked from and joined back to the current
        stream."""
        cur = torch.cuda.current_stream()
        for g in self.groups:
            g["stream"].wait_stream(cur)
            N.check(N.lib().bpm_propagate(g["plan"].handle, ctypes.byref(g["req"]), _ptr(g["ws"]), g["wsb"],
                                          ctypes.c_void_p(g["stream"].cuda_stream)), "bpm_propagate")
        for g in self.groups:
            cur.wait_stream(g["stream"])

    def run(self):
        """All marches once (one graph launch), ordered on the current stream."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._enqueue()

    def result(self, i):
        g, k = self.where[i]
        return self.groups[g]["out"][k]

    def last(self, i):
        g, k = self.where[i]
        return self.groups[g]["last"][k]


# ----------------------------------------------------------------------------------------
# object API (bpm/bpmclass)
# ----------------------------------------------------------------------------------------

class _Bpm3d_GB300:
    """Beam propagation object (bpm/bpmclass/bpm3d.py:_Bpm3d_Base + _bpm3d_ocl.py:_Bpm3d_OCL).

    Propagates with the host-FP64 propagator of _Bpm3d_Base._setup (no FP32 overwrite, no
    mean-index correction), the taper mask for real dn and the untapered complex mask.
    dn stays resident on the device between calls."""

    _float_type = np.float32
    _complex_type = np.complex64

    def __init__(self, size, units, lam=.5, n0=1., dn=None, use_fresnel_approx=False, n_volumes=1):
        self.n_volumes = n_volumes
        self.size = tuple(int(s) for s in size)
        self.size2d = self.size[:2]
        self.units = tuple(float(u) for u in units)
        self.lam = float(lam)
        self.n0 = float(n0)
        self.k0 = 2. * np.pi / lam
        self.dn = None
        self._dn_t = None
        self._is_complex_dn = False
        self.set_dn(dn)

    def set_dn(self, dn=None):
        """dn: (Nz, Ny, Nx) float32/complex64 array (bpm/bpmclass/bpm3d.py:122-141)."""
        if dn is None:
            self.dn = None
            self._dn_t = None
            return
        if tuple(self.size) != tuple(dn.shape)[::-1]:
            raise ValueError("size of dn  %s doesn't match internal size %s" % (tuple(dn.shape)[::-1], self.size))
        cplx = dn.is_complex() if _is_tensor(dn) else np.iscomplexobj(dn)
        self._is_complex_dn = bool(cplx)
        dt = torch.complex64 if cplx else torch.float32
        if _is_tensor(dn):
            self.dn = dn
        else:
            self.dn = np.asarray(dn).astype(self._complex_type if cplx else self._float_type, copy=False)
        self._dn_t = _h2d(dn, dt, _device())

    def _plan(self, absorbing_width):
        return get_plan(self.size, self.units, self.lam, self.n0, absorbing_width, "ignore", N.PROP_CLASS)

    def _propagate_single(self, u0=None, return_full=True, return_intensity=False, absorbing_width=0, **kwargs):
        """March one field (bpm/bpmclass/_bpm3d_ocl.py:66-134). Returns the (Nz, Ny, Nx)
        complex field, the |u|^2 volume (return_intensity), or the complex last plane
        (return_full=False)."""
        Nx, Ny, Nz = self.size
        as_tensor = _is_tensor(u0)
        dev = _device()
        u0_t = (torch.ones((1, Ny, Nx), dtype=torch.complex64, device=dev) if u0 is None
                else _h2d(u0, torch.complex64, dev).reshape(1, Ny, Nx))
        kind = N.DN_NONE if self._dn_t is None else (N.DN_C64 if self._is_complex_dn else N.DN_F32)
        ok = (N.OUT_INTENSITY if return_intensity else N.OUT_FIELD) if return_full else N.OUT_NONE
        out, last, _, _ = _run(self._plan(absorbing_width), u0_t, self._dn_t, kind, 0, ok, True)
        conv = (lambda t: t) if as_tensor else _d2h
        return conv(out[0]) if return_full else conv(last[0])

    def propagate(self, u0=None, return_full=True, return_intensity=False, absorbing_width=0, **kwargs):
        """Alias of _propagate_single."""
        return self._propagate_single(u0, return_full, return_intensity, absorbing_width, **kwargs)

    def propagate_batched(self, u0, return_full=True, return_intensity=False, absorbing_width=0, group=0):
        """March a batch u0 (B, Ny, Nx) through the resident dn in one launch sequence."""
        Nx, Ny, Nz = self.size
        as_tensor = _is_tensor(u0)
        dev = _device()
        u0_t = _h2d(u0, torch.complex64, dev)
        if u0_t.dim() == 2:
            u0_t = u0_t.reshape(1, Ny, Nx)
        kind = N.DN_NONE if self._dn_t is None else (N.DN_C64 if self._is_complex_dn else N.DN_F32)
        ok = (N.OUT_INTENSITY if return_intensity else N.OUT_FIELD) if return_full else N.OUT_NONE
        out, last, _, _ = _run(self._plan(absorbing_width), u0_t, self._dn_t, kind, 0, ok, True, group=group)
        conv = (lambda t: t) if as_tensor else _d2h
        return conv(out) if return_full else conv(last)

    def __repr__(self):
        return "Bpm3d class with size %s and units %s" % (self.size, self.units)


def Bpm3d(size, units, lam=.5, n0=1., dn=None, use_fresnel_approx=False, n_volumes=1, backend="opencl"):
    """Factory for Bpm3d objects (bpm/bpmclass/bpm3d.py:146-167). Every backend name the
    reference accepts ("opencl") and "cuda"/"gb300" select this implementation; others
    raise NotImplementedError as in the reference."""
    if backend not in ("opencl", "cuda", "gb300"):
        raise NotImplementedError
    return _Bpm3d_GB300(size=size, units=units, lam=lam, n0=n0, dn=dn,
                        use_fresnel_approx=use_fresnel_approx, n_volumes=n_volumes)


Bpm3d.__doc__ = _Bpm3d_GB300.__doc__
