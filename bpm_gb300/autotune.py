"""Autotuner for the launch shape of the batched march.

The march advances `group` fields per kernel launch and up to four groups at the same
time on separate streams (see bpm_workspace_bytes in include/bpm_gb300.h). The best group
depends on the grid, the batch, the mean mode and the device: larger groups fill more of
the GPU per launch, smaller ones keep every concurrent group's planes inside L2. The tuner
times a short probe march (the same kernels on the first few dn slices, captured as a CUDA
graph) for each candidate group, best of three trials, and keeps the largest group within
3 % of the fastest (pick_group); results are cached per device and shape in a JSON file
(BPM_GB300_TUNE_CACHE, default ~/.cache/bpm_gb300/autotune.json).
"""
import json
import os

import torch

from . import _native as N

__all__ = ["tune_group", "pick_group", "cache_path"]

_cache = None


def cache_path():
    """The JSON file of measured group sizes: BPM_GB300_TUNE_CACHE, else
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


def tune_group(size, units, lam, n0, batch, dn, mean_mode="weighted", out_kind="intensity",
               absorbing_width=0, nz_probe=12, reps=3, trials=3, force=False):
    """Fields per launch that march `batch` fields of grid `size` fastest on this device.
    dn: the (Nz, Ny, Nx) volume of the real run (its first slices drive the probe)."""
    from .bpm3d import BatchedMarch, _dn_kind

    Nx, Ny, Nz = (int(s) for s in size)
    kind, _ = _dn_kind(dn, False)
    dev = torch.cuda.get_device_properties(torch.cuda.current_device()).name
    key = "%s|%dx%d|b%d|%s|dn%d|%s|aw%d" % (dev, Nx, Ny, batch, mean_mode, kind, out_kind, absorbing_width)
    cache = _load()
    if not force and key in cache:
        return int(cache[key]["group"])
    nzp = max(2, min(Nz, nz_probe))
    dnp = dn[:nzp] if dn is not None else None
    times = {}
    for g in _candidates(batch):
        m = BatchedMarch((Nx, Ny, nzp), units, lam, n0, batch, dn=dnp, mean_mode=mean_mode,
                         absorbing_width=absorbing_width, out_kind=out_kind, group=g)
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
        times[g] = t
        del m
    best = pick_group(times)
    cache[key] = {"group": int(best), "ms_probe": times, "nz_probe": nzp}
    _save()
    return int(best)
