"""Autotuner for the launch shape of the batched march.

A march's launch shape is five choices, none of which changes a result's bits (except the
cluster kernel at 64x64, whose FFT has another radix order; see bpm_request in
include/bpm_gb300.h):
  group      fields advanced per kernel launch: larger groups fill more of the GPU per
             launch and read a shared mask slice once for more fields, smaller ones keep
             every concurrent group's planes inside L2;
  conc       groups marching at once on their own streams (1, 2, 4, 8), so one group's
             kernels fill the SMs another group's tail wave leaves idle;
  col_block  columns per block of the non-weighted column passes (4, 8 or 16): narrower
             blocks spread a small pass over more SMs, 16-column blocks issue fewer
             instructions per column;
  cluster    the whole-march cluster kernel (the field in distributed shared memory, square
             64..256 grids) against the row/column pass kernels;
  col_fuse   the weighted mode's one fused column pass (a thread-block cluster per field)
             against its two column passes.
The tuner times a short probe march for each candidate (the same kernels on the first few
dn slices, captured as a CUDA graph, best of three trials): first the group (pick_group:
the largest group within 3 % of the fastest), then each other choice in turn, which
replaces the current one only when it is more than 3 % faster (pick_option). Results are
cached per device, grid, batch and mode in a JSON file (BPM_GB300_TUNE_CACHE, default
~/.cache/bpm_gb300/autotune.json).
"""
import json
import os

import torch

from . import _native as N

__all__ = ["tune_shape", "tune_group", "pick_group", "pick_option", "shape_candidates", "cache_path"]

_cache = None
_VERSION = 4  # cache entries of another layout are measured again


def cache_path():
    """The JSON file of measured launch shapes: BPM_GB300_TUNE_CACHE, else
    ~/.cache/bpm_gb300/autotune.json."""
    return os.environ.get("BPM_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "bpm_gb300", "autotune.json"))


def _load():
    global _cache
    if _cache is None:
        try:
            with open(cache_path()) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    try:
        os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
        tmp = cache_path() + ".tmp"
        with open(tmp, "w") as f:
            json.dump(_cache, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path())
    except OSError:
        pass


def _candidates(batch):
    c = {g for g in (1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128) if g <= batch}
    c.add(batch)
    return sorted(c)


def pick_group(times, tol=.03):
    """The largest group whose probe time is within `tol` of the fastest: near-equal
    candidates differ by noise, and a larger group launches fewer kernels and reads a shared
    mask once for more fields."""
    tmin = min(times.values())
    return max(g for g, t in times.items() if t <= (1. + tol) * tmin)


def pick_option(current, t_current, times, tol=.03):
    """The option to keep: the fastest of `times` (option -> ms) if it beats the current
    choice by more than `tol`, else the current one."""
    best = min(times, key=times.get)
    if times[best] < (1. - tol) * t_current:
        return best, times[best]
    return current, t_current


def shape_candidates(size, batch, group, mean_mode):
    """The options of each launch-shape choice after the group that apply to a march of
    `batch` fields in groups of `group` on grid `size` (0 is the library's own rule)."""
    Nx, Ny = int(size[0]), int(size[1])
    ngroups = -(-batch // max(1, group))
    out = {}
    if ngroups > 1:
        out["conc"] = [1, 2, 4, 8]
    if mean_mode != "weighted" and Ny >= 128:
        out["col_block"] = [4, 8, 16]    # the weighted passes keep 16-column blocks
    if Nx == Ny and Nx in (64, 128, 256):
        out["cluster"] = [1, 2]
    if mean_mode == "weighted" and Ny in (128, 256, 512) and Nx % 32 == 0 and Nx <= 512:
        out["col_fuse"] = [1, 2]
    return out


def _key(size, batch, mean_mode, dn_kind, out_kind, absorbing_width):
    dev = torch.cuda.get_device_properties(torch.cuda.current_device()).name
    Nx, Ny = int(size[0]), int(size[1])
    return "%s|%dx%d|b%d|%s|dn%d|%s|aw%d" % (dev, Nx, Ny, batch, mean_mode, dn_kind, out_kind, absorbing_width)


def tune_shape(size, units, lam, n0, batch, dn, mean_mode="weighted", out_kind="intensity",
               absorbing_width=0, nz_probe=12, reps=3, trials=3, force=False):
    """Launch shape {group, conc, col_block, cluster, col_fuse} that marches `batch` fields of grid
    `size` fastest on this device. dn: the (Nz, Ny, Nx) volume of the real run (its first
    slices drive the probe)."""
    from .bpm3d import BatchedMarch, _dn_kind

    Nx, Ny, Nz = (int(s) for s in size)
    kind, _ = _dn_kind(dn, False)
    key = _key(size, batch, mean_mode, kind, out_kind, absorbing_width)
    cache = _load()
    if not force and key in cache and cache[key].get("version") == _VERSION:
        return dict(cache[key]["shape"])
    nzp = max(2, min(Nz, nz_probe))
    dnp = dn[:nzp] if dn is not None else None

    def probe(shape):
        m = BatchedMarch((Nx, Ny, nzp), units, lam, n0, batch, dn=dnp, mean_mode=mean_mode,
                         absorbing_width=absorbing_width, out_kind=out_kind, group=shape["group"], launch=shape)
        m.run()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t = float("inf")
        for _ in range(trials):  # best of several short trials: robust to a stray slow one
            a.record()
            for _ in range(reps):
                m.run()
            b.record()
            torch.cuda.synchronize()
            t = min(t, a.elapsed_time(b) / reps)
        del m
        return t

    base = {"group": 0, "conc": 0, "col_block": 0, "cluster": 0, "col_fuse": 0}
    log = {"group": {g: probe(dict(base, group=g)) for g in _candidates(batch)}}
    g = pick_group(log["group"])
    shape, t_best = dict(base, group=g), log["group"][g]
    for axis, options in shape_candidates((Nx, Ny), batch, g, mean_mode).items():
        log[axis] = {v: probe(dict(shape, **{axis: v})) for v in options}
        choice, t_best = pick_option(shape[axis], t_best, log[axis])
        shape[axis] = int(choice)
    cache[key] = {"version": _VERSION, "shape": shape, "group": int(g), "nz_probe": nzp,
                  "ms_probe": {a: {str(k): v for k, v in d.items()} for a, d in log.items()}}
    _save()
    return dict(shape)


def tune_group(size, units, lam, n0, batch, dn, mean_mode="weighted", out_kind="intensity",
               absorbing_width=0, **kw):
    """Fields per launch of the tuned launch shape (tune_shape)."""
    return int(tune_shape(size, units, lam, n0, batch, dn, mean_mode, out_kind, absorbing_width, **kw)["group"])
