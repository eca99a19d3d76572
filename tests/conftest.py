import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbpm_gb300.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = a.astype(dt)
    b = b.astype(dt)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def golden_case(g, name):
    a = g[name + "_args"]
    Nx, Ny, Nz = (int(v) for v in a[:3])
    return dict(size=(Nx, Ny, Nz), units=tuple(float(v) for v in a[3:6]), lam=float(a[6]),
                n0=float(a[7]), absorbing_width=int(a[8]), return_field=bool(a[9]),
                store_dn_as_half=bool(a[10]), mean_mode=str(g[name + "_mode"]),
                u0=g[name + "_u0"], dn=g[name + "_dn"], out=g[name + "_out"])


def golden_psf_case(g, name):
    a = g[name + "_args"]
    NA = g[name + "_NA"]
    NA = float(NA[0]) if len(NA) == 1 else [float(v) for v in NA]
    return dict(shape=tuple(int(v) for v in a[:3]), units=tuple(float(v) for v in a[3:6]),
                lam=float(a[6]), n0=float(a[7]), steps=int(a[8]), NA=NA,
                u=g[name + "_u"], ex=g[name + "_ex"], ey=g[name + "_ey"], ez=g[name + "_ez"])


BPM_GOLDEN = ["bpm_sphere_weighted", "bpm_sphere_simple", "bpm_sphere_ignore",
              "bpm_tilt_taper_weighted", "bpm_tilt_taper_ignore_half"]
PSF_GOLDEN = ["psf_16_NA08", "psf_24x20x12_NA11", "psf_annulus", "psf_u0_like"]
