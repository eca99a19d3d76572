"""March cases for the tests that run them in child processes (cross-process determinism;
the cluster kernel against the pass kernels, chosen by BPM_GB300_CLUSTER; the 1024-point
warp-FFT kernels against the tile kernels, chosen by BPM_GB300_WARP1024).

    python tests/_march_cases.py OUT.npz [cluster|w1024]
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def cases():
    rng = np.random.default_rng(21)
    out = []
    for (nx, ny, nz), mode, dtype, half, B in [((512, 256, 10), "weighted", np.float32, False, 3),
                                               ((256, 512, 8), "simple", np.float32, True, 2),
                                               ((128, 128, 12), "ignore", np.complex64, False, 3),
                                               ((512, 512, 6), "weighted", np.float32, False, 5),
                                               ((256, 128, 7), "weighted", np.float32, True, 2)]:
        dn = (.03 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
        if dtype == np.complex64:
            dn = (dn - 1j * np.abs(.002 * rng.standard_normal((nz, ny, nx)))).astype(np.complex64)
        x = np.arange(nx) * .1
        u0 = np.exp(2j * np.pi * rng.uniform(-.3, .3, (B, 1, 1)) * x[None, None, :]).repeat(ny, 1)
        out.append(dict(size=(nx, ny, nz), mode=mode, dn=dn, half=half, u0=u0.astype(np.complex64)))
    return out


def cluster_cases():
    """Square grids the whole-march cluster kernel serves (64, 128, 256), every mean mode
    and dn kind, batched (shared and per-field dn) and single."""
    rng = np.random.default_rng(5)
    out = []
    for n, nz, mode, kind, B in [(64, 7, "weighted", "f32", 3), (128, 12, "simple", "f16", 2),
                                 (128, 9, "ignore", "c64", 3), (256, 6, "weighted", "f32", 2),
                                 (256, 5, "ignore", "none", 1), (64, 1, "weighted", "f32", 2),
                                 (128, 8, "weighted", "per-field", 3)]:
        dn = None
        if kind != "none":
            dn = (.03 * rng.standard_normal((nz, n, n))).astype(np.float32)
            if kind == "c64":
                dn = (dn - 1j * np.abs(.002 * rng.standard_normal((nz, n, n)))).astype(np.complex64)
            if kind == "per-field":
                dn = (.03 * rng.standard_normal((B, nz, n, n))).astype(np.float32)
        x = np.arange(n) * .1
        u0 = np.exp(2j * np.pi * rng.uniform(-.3, .3, (B, 1, 1)) * x[None, None, :]).repeat(n, 1)
        out.append(dict(size=(n, n, nz), mode=mode, dn=dn, half=kind == "f16", u0=u0.astype(np.complex64)))
    return out


def run_cluster(path):
    import bpm_gb300 as bpm
    res = {}
    for i, c in enumerate(cluster_cases()):
        res["f%d" % i] = bpm.bpm_3d_batched(c["size"], (.1, .1, .1), u0=c["u0"], dn=c["dn"], mean_mode=c["mode"],
                                            store_dn_as_half=c["half"], return_field=True)
        res["l%d" % i] = bpm.bpm_3d_batched(c["size"], (.1, .1, .1), u0=c["u0"], dn=c["dn"], mean_mode=c["mode"],
                                            store_dn_as_half=c["half"], return_full=False, absorbing_width=4)
        if c["dn"] is None or c["dn"].ndim == 3:
            res["i%d" % i] = bpm.bpm_3d(c["size"], (.1, .1, .1), u0=c["u0"][0], dn=c["dn"], mean_mode=c["mode"],
                                        store_dn_as_half=c["half"], return_field=False, absorbing_width=3)
    np.savez(path, **res)


def w1024_cases():
    """1024-point rows or columns (and both), every dn kind: the warp-FFT kernels
    (BPM_GB300_WARP1024=1) against the shared-memory tile kernels (=0)."""
    rng = np.random.default_rng(9)
    out = []
    for (nx, ny, nz), mode, kind, B in [((1024, 128, 6), "weighted", "f32", 3), ((128, 1024, 6), "ignore", "c64", 1),
                                        ((1024, 1024, 4), "simple", "f16", 1), ((256, 1024, 5), "weighted", "f32", 2)]:
        dn = (.03 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
        if kind == "c64":
            dn = (dn - 1j * np.abs(.002 * rng.standard_normal((nz, ny, nx)))).astype(np.complex64)
        x = np.arange(nx) * .1
        u0 = np.exp(2j * np.pi * rng.uniform(-.3, .3, (B, 1, 1)) * x[None, None, :]).repeat(ny, 1)
        out.append(dict(size=(nx, ny, nz), mode=mode, dn=dn, half=kind == "f16", u0=u0.astype(np.complex64)))
    return out


def run_w1024(path):
    import bpm_gb300 as bpm
    res = {}
    for i, c in enumerate(w1024_cases()):
        res["f%d" % i] = bpm.bpm_3d_batched(c["size"], (.1, .1, .1), u0=c["u0"], dn=c["dn"], mean_mode=c["mode"],
                                            store_dn_as_half=c["half"], return_field=True, absorbing_width=4)
    np.savez(path, **res)


def run(path):
    import bpm_gb300 as bpm
    res = {}
    for i, c in enumerate(cases()):
        res["f%d" % i] = bpm.bpm_3d_batched(c["size"], (.1, .1, .1), u0=c["u0"], dn=c["dn"], mean_mode=c["mode"],
                                            store_dn_as_half=c["half"], return_field=True, group=2)
        res["i%d" % i] = bpm.bpm_3d(c["size"], (.1, .1, .1), u0=c["u0"][0], dn=c["dn"], mean_mode=c["mode"],
                                    store_dn_as_half=c["half"], return_field=False, absorbing_width=5)
    np.savez(path, **res)


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "cluster":
        run_cluster(sys.argv[1])
    elif len(sys.argv) > 2 and sys.argv[2] == "w1024":
        run_w1024(sys.argv[1])
    else:
        run(sys.argv[1])
