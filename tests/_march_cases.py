"""March cases shared by the kernel-path comparison test: run in-process (pipelined
kernels) and in a child process with BPM_GB300_KERNELS=warp (single-wave warp kernels).

    python tests/_march_cases.py OUT.npz
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
                                               ((512, 512, 6), "weighted", np.float32, False, 5)]:
        dn = (.03 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
        if dtype == np.complex64:
            dn = (dn - 1j * np.abs(.002 * rng.standard_normal((nz, ny, nx)))).astype(np.complex64)
        x = np.arange(nx) * .1
        u0 = np.exp(2j * np.pi * rng.uniform(-.3, .3, (B, 1, 1)) * x[None, None, :]).repeat(ny, 1)
        out.append(dict(size=(nx, ny, nz), mode=mode, dn=dn, half=half, u0=u0.astype(np.complex64)))
    return out


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
    run(sys.argv[1])
