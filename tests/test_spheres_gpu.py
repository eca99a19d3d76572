"""On-device coated-sphere dn volumes (bpm_spheres_fill) against the reference kernel's
output (golden, bit-exact) and bpm_3d_spheres against bpm_3d on the oracle's volume."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300.spheres
    return bpm_gb300


@pytest.mark.parametrize("name", ["spheres_a", "spheres_b"])
def test_fill_bit_exact(bpm, golden, name):
    a = golden[name + "_args"]
    size = tuple(int(v) for v in a[:3])
    r = a[6:10]
    dn = bpm.spheres.create_dn_buffer(size, tuple(a[3:6]), golden[name + "_pts"], r[0], r[1], r[2], r[3])
    assert bool(np.array_equal(dn.cpu().numpy(), golden[name + "_out"]))


def test_bpm_3d_spheres(bpm):
    from oracle import spheres_ref, bpm_ref
    size, units = (64, 64, 32), (.1, .1, .1)
    pts = [[3.2, 3.2, 1.6], [1.0, 5.0, 2.5], [5.5, 1.5, 0.8]]
    u = bpm.spheres.bpm_3d_spheres(size, units, lam=.5, points=pts, dn_inner=.02, rad_inner=.3, dn_outer=.05,
                                   rad_outer=.8)
    assert isinstance(u, np.ndarray) and u.shape == (32, 64, 64)
    dn = spheres_ref.create_dn_buffer(size, units, pts, .02, .3, .05, .8)
    o = bpm_ref.bpm_3d(size, units, lam=.5, dn=dn, precision="fp64")
    assert rel_l2(u, o) < 1e-4
