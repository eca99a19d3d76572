"""Debye-Wolf focus fields for the test that runs them in child processes, one with the
quadrature on the tensor cores (the default) and one with BPM_GB300_DEBYE=fma (FP32 FMA
kernels), which the library reads once per process.

    python tests/_psf_cases.py OUT.npz
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

CASES = [
    ("psf_64", dict(shape=(64, 64, 64), units=(.1, .1, .1), lam=.5, NA=1.1, n0=1.33, steps=200)),
    ("psf_96x64x32", dict(shape=(96, 64, 32), units=(.05, .08, .1), lam=.488, NA=.8, n0=1.0, steps=100)),
    ("psf_annuli", dict(shape=(128, 128, 64), units=(.1, .1, .1), lam=.5, NA=[.2, .4, .6, .8], n0=1.33, steps=64)),
    ("psf_256", dict(shape=(256, 256, 256), units=(.1, .1, .1), lam=.5, NA=1.1, n0=1.33, steps=512)),
    ("psf_200x160x96", dict(shape=(200, 160, 96), units=(.1, .1, .1), lam=.6, NA=1.3, n0=1.52, steps=300)),
]
GAUSS = [("gauss_63x48x40", dict(shape=(63, 48, 40), units=(.1, .1, .1), lam=.5, NA=[0, .9], sig=.7, steps=80)),
         ("gauss_96", dict(shape=(96, 96, 96), units=(.1, .1, .1), lam=.5, NA=[.1, .95], sig=1., steps=150))]


def run(path):
    import bpm_gb300 as bpm
    res = {}
    for name, c in CASES:
        u, ex, ey, ez = bpm.psf(c["shape"], c["units"], c["lam"], c["NA"], c["n0"], c["steps"], return_field=True)
        res[name + "_u"], res[name + "_ex"], res[name + "_ey"], res[name + "_ez"] = u, ex, ey, ez
    for name, c in GAUSS:
        u, ex, ey, ez = bpm.focus_field_debye_gauss(c["shape"], c["units"], c["lam"], c["NA"], sig=c["sig"],
                                                    n_integration_steps=c["steps"])
        res[name + "_u"], res[name + "_ex"], res[name + "_ey"], res[name + "_ez"] = u, ex, ey, ez
    from bpm_gb300 import _native as N
    res["device_status"] = np.array([N.lib().bpm_device_status(1)])
    np.savez(path, **res)


if __name__ == "__main__":
    run(sys.argv[1])
