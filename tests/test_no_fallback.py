"""The product path has no CPU fallback: without a CUDA device every public entry point
raises before computing anything, and without the built library every C-ABI call raises.
These run on the CPU-only machine (skipped where a GPU is visible)."""
import numpy as np
import pytest
import torch

import bpm_gb300 as bpm
from bpm_gb300 import _native as N

no_gpu = pytest.mark.skipif(torch.cuda.is_available(), reason="a CUDA device is visible")


def _calls():
    u0 = np.ones((32, 64), np.complex64)
    dn = np.zeros((8, 32, 64), np.float32)
    from bpm_gb300.serve import BpmRequest
    return {
        "bpm_3d": lambda: bpm.bpm_3d((64, 32, 8), (.1, .1, .1), u0=u0, dn=dn),
        "bpm_3d_batched": lambda: bpm.bpm_3d_batched((64, 32, 8), (.1, .1, .1), u0=np.stack([u0, u0]), dn=dn),
        "bpm_3d n_volumes": lambda: bpm.bpm_3d((64, 32, 8), (.1, .1, .1), u0=u0, dn=dn, n_volumes=2),
        "Bpm3d": lambda: bpm.Bpm3d((64, 32, 8), (.1, .1, .1), dn=dn).propagate(u0),
        "BatchedMarch": lambda: bpm.BatchedMarch((64, 32, 8), (.1, .1, .1), .5, 1., 2, dn=dn),
        "MixedBatch": lambda: bpm.MixedBatch([BpmRequest((64, 32, 8), (.1, .1, .1), u0=u0, dn=dn)]),
        "psf": lambda: bpm.psf((16, 16, 16), (.1, .1, .1), .5, .8),
        "psf_u0": lambda: bpm.psf_u0((32, 32), (.1, .1), zfoc=1.),
        "focus_field_debye": lambda: bpm.focus_field_debye((16, 16, 16), (.1, .1, .1), .5, .8),
        "focus_field_debye_gauss": lambda: bpm.focus_field_debye_gauss((16, 16, 16), (.1, .1, .1), .5, [0, .8]),
        "focus_field_debye_plane": lambda: bpm.focus_field_debye_plane((16, 16), (.1, .1)),
        "focus_field_debye_at": lambda: bpm.focus_field_debye_at(np.zeros(4, np.float32), np.zeros(4, np.float32),
                                                                 np.zeros(4, np.float32), .5, .8),
        "psf_lightsheet": lambda: bpm.psf_lightsheet((16, 16, 16), (.1, .1, .1), .5, .2, .5, .8),
        "bpm_3d_spheres": lambda: bpm.bpm_3d_spheres((64, 32, 8), (.1, .1, .1), points=[(3., 1.5, .4)]),
    }


@no_gpu
@pytest.mark.parametrize("name", sorted(_calls()))
def test_entry_point_raises_without_a_gpu(name):
    with pytest.raises(RuntimeError, match="bpm_gb300 needs a CUDA device"):
        _calls()[name]()


def test_missing_library_raises(monkeypatch, tmp_path):
    monkeypatch.setattr(N, "LIB_PATH", str(tmp_path / "libbpm_gb300.so"))
    monkeypatch.setattr(N, "_lib", None)
    with pytest.raises(RuntimeError, match="not built"):
        N.lib()
    with pytest.raises(RuntimeError, match="not built"):
        N.last_error()
