"""Parity of the CUDA Debye-Wolf focus field with the reference (golden vectors from the
reference's own kernel) and with the FP64 oracle. Tolerance: relative L2 <= 1e-4."""
import numpy as np
import pytest

from conftest import PSF_GOLDEN, golden_psf_case, rel_l2
from oracle import debye_ref

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    return bpm_gb300


@pytest.mark.parametrize("name", PSF_GOLDEN)
def test_golden_reference_kernel(bpm, golden, name):
    c = golden_psf_case(golden, name)
    u, ex, ey, ez = bpm.psf(c["shape"], c["units"], c["lam"], c["NA"], c["n0"], c["steps"], return_field=True)
    assert u.shape == c["u"].shape and u.dtype == np.float32 and ex.dtype == np.complex64
    for a, k in zip((u, ex, ey, ez), ("u", "ex", "ey", "ez")):
        assert rel_l2(a, c[k]) < TOL, k


@pytest.mark.parametrize("shape,units,lam,NA,n0,steps", [
    ((64, 64, 64), (.1, .1, .1), .5, 1.1, 1.33, 200),
    ((96, 64, 32), (.05, .08, .1), .488, .8, 1.0, 100),
    ((128, 128, 64), (.1, .1, .1), .5, [.2, .4, .6, .8], 1.33, 64),
    ((2, 2, 2), (.1, .1, .1), .5, .5, 1.0, 20),
])
def test_oracle_parity(bpm, shape, units, lam, NA, n0, steps):
    u, ex, ey, ez = bpm.focus_field_debye(shape, units, lam, NA, n0, steps)
    o = debye_ref.focus_field_debye(shape, units, lam, NA, n0, steps,
                                    real_dtype=np.float64, complex_dtype=np.complex128)
    for a, b, k in zip((u, ex, ey, ez), o, ("u", "ex", "ey", "ez")):
        assert rel_l2(a, b) < TOL, k


def test_config2_psf_256(bpm):
    """256^3 vectorial PSF, NA 1.1, n0 1.33, lam 0.5, x-polarised, 512 steps: the intensity
    agrees with the FP64 oracle on a set of full-resolution slices."""
    shape = (256, 256, 256)
    u, ex, ey, ez = bpm.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 512, return_field=True)
    params = debye_ref.octant_params(shape, (.1, .1, .1), .5, 1.1, 1.33)
    octant = debye_ref.debye_octant(params, 512)
    c = 128
    # full index c + k (k >= 1 along z, >= 0 along x, y) holds octant sample k, unconjugated
    for a, b, k in zip((u, ex, ey, ez), octant, ("u", "ex", "ey", "ez")):
        assert rel_l2(a[c + 1:, c:, c:], b[1:c, :c, :c]) < TOL, k
    assert np.all(np.isfinite(u))
    u_only = bpm.psf(shape, (.1, .1, .1), .5, 1.1, 1.33, 512)
    assert np.array_equal(u_only, u)


def test_psf_u0_matches_oracle(bpm):
    a = bpm.psf_u0((256, 256), (.1, .1), zfoc=12.8, NA=.4, lam=.5, n0=1.33)
    b = debye_ref.psf_u0((256, 256), (.1, .1), zfoc=12.8, NA=.4, lam=.5, n0=1.33)
    assert a.shape == (256, 256) and a.dtype == np.complex64
    assert rel_l2(a, b) < TOL


def test_psf_lightsheet_matches_oracle(bpm):
    a = bpm.psf_lightsheet((32, 32, 32), (.1, .1, .1), .5, .2, .5, .8, n0=1.33, n_integration_steps=50)
    b = debye_ref.psf_lightsheet((32, 32, 32), (.1, .1, .1), .5, .2, .5, .8, n0=1.33, n_integration_steps=50)
    assert rel_l2(a, b) < TOL


def test_psf_errors(bpm):
    with pytest.raises(NotImplementedError):
        bpm.psf((16, 16, 15), (.1, .1, .1), .5, .8)
    with pytest.raises(AssertionError):
        bpm.psf((16, 16, 16), (.1, .1, .1), .5, [.1, .2, .3])
