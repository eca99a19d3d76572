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


def debye_point_fp64(x, y, z, k, NA, n_int):
    """The vectorial Debye integral at one point, x-polarised, by the trapezoid rule on
    n_int equispaced angles over [0, arcsin NA] with the pupil factor sqrt(cos t) sin t:
    the independent formula of the reference's tests/test_psf_vectorial.py:15-42, in FP64."""
    from scipy.special import jv
    a = np.arcsin(NA)
    t = np.linspace(0., a, n_int)
    w = np.full(n_int, a / (n_int - 1.))
    w[0] *= .5
    w[-1] *= .5
    kr, kz, phi = k * np.hypot(x, y), k * z, np.arctan2(y, x)
    pupil = w * np.sqrt(np.cos(t)) * np.sin(t) * np.exp(1j * kz * np.cos(t))
    I0 = np.sum(pupil * (np.cos(t) + 1.) * jv(0, kr * np.sin(t)))
    I1 = np.sum(pupil * np.sin(t) * jv(1, kr * np.sin(t)))
    I2 = np.sum(pupil * (np.cos(t) - 1.) * jv(2, kr * np.sin(t)))
    return I0 + I2 * np.cos(2 * phi), I2 * np.sin(2 * phi), -2j * I1 * np.cos(phi)
