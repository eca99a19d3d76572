"""Launch shapes of the march (fields per launch, concurrent groups, column-block width,
cluster kernel or pass kernels, one fused or two weighted column passes; bpm_request in
include/bpm_gb300.h) never change a result:
every candidate the autotuner may pick gives the same bits as the library's default shape
(the cluster kernel at 64x64, whose FFT has another radix order, to FP32 rounding), and the
tuner's choice is valid, cached and applied by BatchedMarch(group="auto")."""
import itertools

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    return bpm_gb300


def inputs(size, batch, seed, cplx=False):
    Nx, Ny, Nz = size
    rng = np.random.default_rng(seed)
    dn = (.03 * rng.standard_normal((Nz, Ny, Nx))).astype(np.float32)
    if cplx:
        dn = (dn - 1j * np.abs(.002 * rng.standard_normal((Nz, Ny, Nx)))).astype(np.complex64)
    x = .1 * np.arange(Nx)
    u0 = np.exp(2j * np.pi * rng.uniform(-.3, .3, (batch, 1, 1)) * x[None, None, :]).repeat(Ny, 1)
    return u0.astype(np.complex64), dn


@pytest.mark.parametrize("size,batch,mode,cplx", [
    ((256, 256, 9), 10, "weighted", False),
    ((512, 256, 7), 9, "ignore", True),
    ((128, 128, 10), 5, "simple", False),
    ((64, 64, 8), 3, "weighted", False),
])
def test_every_launch_shape_gives_the_same_result(bpm, size, batch, mode, cplx):
    u0, dn = inputs(size, batch, 3, cplx)
    kw = dict(lam=.5, n0=1.33, dn=dn, mean_mode=mode, absorbing_width=3, return_field=True)
    ref = bpm.bpm_3d_batched(size, (.1, .1, .1), u0=u0, **kw)
    n = 0
    for group, conc, col_block, cluster, fuse in itertools.product((1, 3, 0), (1, 2, 8), (4, 8, 16), (1, 2), (1, 2)):
        launch = {"group": group, "conc": conc, "col_block": col_block, "cluster": cluster, "col_fuse": fuse}
        got = bpm.bpm_3d_batched(size, (.1, .1, .1), u0=u0, launch=launch, **kw)
        if size[0] == 64 and cluster == 2:
            # the default at 64x64 is the cluster kernel (warp FFT); the pass kernels run the
            # tile FFT there: the same to FP32 rounding
            assert rel_l2(got, ref) < 2e-6, launch
        else:
            assert np.array_equal(got, ref), launch
        n += 1
    assert n == 108


def test_tuned_shape_is_applied(bpm, tmp_path, monkeypatch):
    import torch
    from bpm_gb300 import autotune
    monkeypatch.setenv("BPM_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_cache", None)
    size, batch = (256, 256, 16), 12
    u0, dn = inputs(size, batch, 5)
    dn_t = torch.from_numpy(dn).cuda()
    shape = autotune.tune_shape(size, (.1, .1, .1), .5, 1.33, batch, dn_t, "weighted", "intensity")
    assert set(shape) == {"group", "conc", "col_block", "cluster", "col_fuse"}
    assert 1 <= shape["group"] <= batch and shape["conc"] in (0, 1, 2, 4, 8)
    assert shape["col_block"] in (0, 4, 8, 16) and shape["cluster"] in (0, 1, 2) and shape["col_fuse"] in (0, 1, 2)
    assert (tmp_path / "tune.json").exists()
    assert autotune.tune_shape(size, (.1, .1, .1), .5, 1.33, batch, dn_t, "weighted", "intensity") == shape
    m = bpm.BatchedMarch(size, (.1, .1, .1), .5, 1.33, batch, dn=dn_t, group="auto")
    assert m.launch == shape
    m.u0.copy_(torch.from_numpy(u0))
    m.run()
    torch.cuda.synchronize()
    want = bpm.bpm_3d_batched(size, (.1, .1, .1), lam=.5, n0=1.33, u0=u0, dn=dn, return_field=False)
    assert np.array_equal(m.out.cpu().numpy(), want)
