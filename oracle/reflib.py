"""ctypes bindings to oracle/_ref/libref_cl.so. TEST INFRASTRUCTURE ONLY.

libref_cl.so is the reference's own kernel source (bpm/bpm/kernels/bpm_3d_kernels.cl,
bpm/psf/kernels/psf_debye.cl + bessel.cl) compiled as host C++ through oracle/ref_shim.
It exists only where the reference checkout was available at build time (oracle/Makefile);
`load()` returns None elsewhere and callers skip.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libref_cl.so")

_lib = None


class CFloat(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


def load():
    """Return the loaded library or None when it was not built here."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        return None
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError:
        return None
    P = ctypes.c_void_p
    F = ctypes.c_float
    I = ctypes.c_int
    lib.ref_debye_wolf.argtypes = [P, P, P, P, F, F, F, F, F, F, F, F, F, P, I, I, I, I, I]
    lib.ref_debye_wolf_plane.argtypes = [P, F, F, F, F, F, F, F, F, P, I, I, I, I]
    lib.ref_debye_wolf_at.argtypes = [P, P, P, P, P, P, P, F, F, F, P, I, ctypes.c_long, I]
    lib.ref_debye_wolf_gauss.argtypes = [P, P, P, P, F, F, F, F, F, F, F, F, F, F, P, I, I, I, I, I]
    lib.ref_bessel_jn.argtypes = [I, P, P, ctypes.c_long]
    lib.ref_compute_propagator.argtypes = [P, F, F, F, F, F, I, I]
    lib.ref_mult_propagator.argtypes = [P, F, F, F, F, F, I, I]
    lib.ref_mult_propagator_buff.argtypes = [P, P, P, F, F, F, F, F, I, I]
    lib.ref_mult.argtypes = [P, P, I]
    lib.ref_mult_dn.argtypes = [P, P, F, I, I, I, I]
    lib.ref_mult_dn_half.argtypes = [P, P, F, I, I, I, I]
    lib.ref_mult_dn_complex.argtypes = [P, P, F, I, I, I, I]
    lib.ref_mult_dn_mean.argtypes = [P, P, F, F, I, I, I, I]
    lib.ref_mult_dn_mean_half.argtypes = [P, P, F, F, I, I, I, I]
    lib.ref_mult_dn_mean_complex.argtypes = [P, P, F, CFloat, I, I, I, I]
    lib.ref_mult_dn_mean_buff.argtypes = [P, P, P, P, F, I, I, I, I]
    lib.ref_mult_dn_mean_half_buff.argtypes = [P, P, P, P, F, I, I, I, I]
    lib.ref_copy_intens.argtypes = [P, P, I, I]
    lib.ref_fill_dn.argtypes = [P, P, I, F, F, F, F, F, F, F, I, I, I]
    _lib = lib
    return lib


def ptr(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def f32(x):
    return ctypes.c_float(float(np.float32(x)))
