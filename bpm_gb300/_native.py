"""ctypes bindings to libbpm_gb300.so (the C ABI declared in include/bpm_gb300.h).

The library is built in-tree by bpm_gb300/build.py. There is no fallback: if the
library is missing or cannot be loaded, every entry point raises.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbpm_gb300.so")

c_int = ctypes.c_int
c_double = ctypes.c_double
c_ll = ctypes.c_longlong
c_vp = ctypes.c_void_p
c_size = ctypes.c_size_t

BPM_OK = 0
BPM_ERR_ARG = -1
BPM_ERR_SHAPE = -2
BPM_ERR_OOM = -3
BPM_ERR_CUDA = -4
BPM_ERR_TIMEOUT = -5
BPM_ERR_UNSUPPORTED = -6

MEAN_MODES = {"ignore": 0, "simple": 1, "weighted": 2}
PROP_FUNCTIONAL = 0
PROP_CLASS = 1
DN_NONE, DN_F32, DN_F16, DN_C64 = 0, 1, 2, 3
OUT_NONE, OUT_FIELD, OUT_INTENSITY = 0, 1, 2
PASS_FIRST_ROW, PASS_COLUMN, PASS_COLUMN_REDUCE, PASS_COLUMN_PROPAGATE, PASS_ROW, PASS_COLUMN_FUSED = 0, 1, 2, 3, 4, 5


class GridDesc(ctypes.Structure):
    """bpm_grid_desc of include/bpm_gb300.h: grid, units and physics of a plan."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("dx", c_double), ("dy", c_double), ("dz", c_double),
                ("lam", c_double), ("n0", c_double),
                ("absorbing_width", c_int), ("mean_mode", c_int), ("prop_kind", c_int),
                ("use_fresnel_approx", c_int)]


class Request(ctypes.Structure):
    """bpm_request of include/bpm_gb300.h: the device buffers and options of one march."""
    _fields_ = [("batch", c_int), ("u0", c_vp), ("dn", c_vp), ("dn_dtype", c_int),
                ("dn_batch_stride", c_ll), ("slice_n", c_vp), ("slice_dn0", c_vp),
                ("out", c_vp), ("out_kind", c_int), ("out_batch_stride", c_ll),
                ("last_plane", c_vp), ("scatter_p", c_vp), ("scatter_g", c_vp),
                ("scattering_plane_ind", c_int), ("group", c_int),
                ("ckpt", c_vp), ("ckpt_every", c_int), ("mask", c_vp),
                ("conc", c_int), ("col_block", c_int), ("cluster", c_int), ("col_fuse", c_int),
                ("grad_sum", c_int)]


class DebyeDesc(ctypes.Structure):
    """debye_desc of include/bpm_gb300.h: grid, units, optics and polarisation of a
    Debye-Wolf field."""
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("dx", c_double), ("dy", c_double), ("dz", c_double),
                ("lam", c_double), ("n0", c_double),
                ("na", ctypes.POINTER(c_double)), ("n_na", c_int),
                ("n_integration_steps", c_int), ("ex0", c_double), ("ey0", c_double), ("quadrature", c_int)]


# every symbol include/bpm_gb300.h declares, with its ctypes signature
SIGNATURES = {
    "bpm_version": (c_int, []),
    "bpm_last_error": (ctypes.c_char_p, []),
    "bpm_launch_count": (ctypes.c_ulonglong, []),
    "bpm_grid_check": (c_int, [ctypes.POINTER(GridDesc)]),
    "bpm_plan_create": (c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(c_vp)]),
    "bpm_plan_derive": (c_int, [c_vp, c_int, ctypes.POINTER(c_vp)]),
    "bpm_plan_destroy": (c_int, [c_vp]),
    "bpm_group_size": (c_int, [c_vp, c_int, c_int]),
    "bpm_workspace_bytes": (c_size, [c_vp, c_int, c_int]),
    "bpm_workspace_bytes_conc": (c_size, [c_vp, c_int, c_int, c_int]),
    "bpm_propagate": (c_int, [c_vp, ctypes.POINTER(Request), c_vp, c_size, c_vp]),
    "bpm_mask_precompute": (c_int, [c_vp, c_vp, c_int, c_vp, c_vp]),
    "bpm_propagate_noalloc": (c_int, [c_vp, ctypes.POINTER(Request), c_vp]),
    "bpm_propagate_to_host": (c_int, [c_vp, ctypes.POINTER(Request), c_vp, c_int, c_vp, c_size, c_vp]),
    "bpm_launch_pass": (c_int, [c_vp, ctypes.POINTER(Request), c_vp, c_size, c_int, c_int, c_vp]),
    "bpm_backward_workspace_bytes": (c_size, [c_vp, c_int, c_int, c_int]),
    "bpm_backward": (c_int, [c_vp, ctypes.POINTER(Request), c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
    "bpm_exec_create": (c_int, [c_vp, ctypes.POINTER(Request), c_vp, c_size, ctypes.POINTER(c_vp)]),
    "bpm_exec_launch": (c_int, [c_vp, c_vp]),
    "bpm_exec_destroy": (c_int, [c_vp]),
    "bpm_spheres_fill": (c_int, [c_int, c_int, c_int, c_double, c_double, c_double, c_vp, c_int,
                                 c_double, c_double, c_double, c_double, c_vp, c_vp]),
    "bpm_host_ptr_mapped": (c_int, [c_vp]),
    "bpm_device_status": (c_int, [c_int]),
    "debye_tc_timeout_selftest": (c_int, [c_double]),
    "debye_workspace_bytes": (c_size, [ctypes.POINTER(DebyeDesc)]),
    "debye_focus_field": (c_int, [ctypes.POINTER(DebyeDesc), c_vp, c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
    "debye_gauss_workspace_bytes": (c_size, [ctypes.POINTER(DebyeDesc)]),
    "debye_focus_field_gauss": (c_int, [ctypes.POINTER(DebyeDesc), c_double, c_vp, c_vp, c_vp, c_vp, c_vp, c_size,
                                        c_vp]),
    "debye_points_workspace_bytes": (c_size, [ctypes.POINTER(DebyeDesc)]),
    "debye_focus_field_plane": (c_int, [ctypes.POINTER(DebyeDesc), c_double, c_vp, c_vp, c_size, c_vp]),
    "debye_focus_field_at": (c_int, [ctypes.POINTER(DebyeDesc), c_vp, c_vp, c_vp, ctypes.c_longlong, c_vp, c_vp, c_vp,
                                     c_vp, c_vp, c_size, c_vp]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load libbpm_gb300.so (once). Raises RuntimeError when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("bpm_gb300 CUDA library not built (%s missing): run "
                               "`python -m bpm_gb300.build`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    """Text of the calling thread's last library error (bpm_last_error)."""
    return lib().bpm_last_error().decode(errors="replace")


def check(rc, what=""):
    """Map a bpm_status to the exception the reference raises in the same situation."""
    if rc == BPM_OK:
        return
    msg = "%s: %s" % (what, last_error()) if what else last_error()
    if rc == BPM_ERR_ARG:
        raise ValueError(msg)
    if rc in (BPM_ERR_SHAPE, BPM_ERR_UNSUPPORTED):
        raise NotImplementedError(msg)
    if rc == BPM_ERR_OOM:
        raise MemoryError(msg)
    raise RuntimeError("bpm_gb300 error %d: %s" % (rc, msg))


def launch_count():
    """Kernels this process has launched through the library (bpm_launch_count)."""
    return int(lib().bpm_launch_count())
