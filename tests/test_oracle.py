"""The CPU oracle against the golden vectors made from the reference's own kernels.

Pins oracle/bpm_ref.py and oracle/debye_ref.py (tests/golden/make_golden.py documents how
the vectors were produced: reference OpenCL kernel sources compiled as host C++)."""
import numpy as np
import pytest

from conftest import BPM_GOLDEN, PSF_GOLDEN, golden_case, golden_psf_case, rel_l2
from oracle import bpm_ref, debye_ref, reflib


def test_masks_bit_exact(golden):
    keys = [k for k in golden.files if k.startswith("mask_") and not k.endswith("_args")]
    assert keys
    for key in keys:
        Nx, Ny = map(int, key[5:].split("x"))
        dx, dy, lam, n0, dz = golden[key + "_args"]
        _, m = bpm_ref.propagator_f32(n0, 2 * np.pi / lam, dx, dy, dz, Nx, Ny)
        assert np.array_equal(m, golden[key]), key


@pytest.mark.parametrize("absorb", [0, 1, 5, 12])
def test_taper_bit_exact(golden, absorb):
    assert np.array_equal(bpm_ref.taper_f32(40, 36, absorb), golden["taper_%d" % absorb])


@pytest.mark.parametrize("name", BPM_GOLDEN)
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bpm_oracle_vs_reference_kernels(golden, name, precision):
    c = golden_case(golden, name)
    o = bpm_ref.bpm_3d(c["size"], c["units"], lam=c["lam"], n0=c["n0"], u0=c["u0"], dn=c["dn"],
                       mean_mode=c["mean_mode"], absorbing_width=c["absorbing_width"],
                       return_field=c["return_field"], store_dn_as_half=c["store_dn_as_half"],
                       precision=precision)
    assert rel_l2(o, c["out"]) < 5e-6


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_class_oracle_vs_reference_kernels(golden, precision):
    dnc = golden["class_complex_dn"]
    o = bpm_ref.bpm3d_propagate((32, 32, 10), (.1, .1, .1), .5, 1.33, dn=dnc, precision=precision)
    assert rel_l2(o, golden["class_complex_out"]) < 5e-6
    o = bpm_ref.bpm3d_propagate((32, 32, 10), (.1, .1, .1), .5, 1.33, dn=dnc.real.astype(np.float32),
                                absorbing_width=4, precision=precision)
    assert rel_l2(o, golden["class_real_out"]) < 5e-6


@pytest.mark.parametrize("name", PSF_GOLDEN)
def test_debye_oracle_vs_reference_kernel(golden, name):
    c = golden_psf_case(golden, name)
    u, ex, ey, ez = debye_ref.psf(c["shape"], c["units"], c["lam"], c["NA"], c["n0"], c["steps"],
                                  return_field=True)
    for a, k in zip((u, ex, ey, ez), ("u", "ex", "ey", "ez")):
        assert rel_l2(a, c[k]) < 5e-6, k


def test_bessel_reference_approximation(golden):
    from scipy.special import jv
    x = golden["bessel_x"].astype(np.float64)
    for n in range(3):
        assert np.max(np.abs(jv(n, x) - golden["bessel_j%d" % n])) < 5e-7


@pytest.mark.parametrize("N0", [2, 4, 16, 30])
def test_mirror_index_form_equals_slice_loop(N0):
    """The |m - N0/2| index map (used by the GPU assembly) equals the reference's loop."""
    rng = np.random.default_rng(N0)
    shape = (N0, N0 + 2, 4)
    No = [s // 2 + 1 for s in shape]
    u = rng.normal(size=(No[2], No[1], No[0])).astype(np.float32)
    ex = (rng.normal(size=u.shape) + 1j * rng.normal(size=u.shape)).astype(np.complex64)
    u_all, ex_all, _, _ = debye_ref.mirror_octant(shape, u, ex, ex, ex)
    ix = debye_ref.mirror_index(shape[0])
    iy = debye_ref.mirror_index(shape[1])
    iz = debye_ref.mirror_index(shape[2])
    U = u[iz][:, iy][:, :, ix]
    E = ex[iz][:, iy][:, :, ix]
    E = np.where((np.arange(shape[2]) <= shape[2] // 2)[:, None, None], np.conj(E), E)
    assert np.array_equal(U, u_all)
    assert np.array_equal(E, ex_all)


def test_split_oracle_consistency():
    """test_field_intens.py:29-43: |field|^2 == intensity mode, through the z-split."""
    Nx = Ny = 32
    Nz = 20
    z, y, x = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    dn = (.05 * (((x - 16) ** 2 + (y - 16) ** 2 + (z - 10) ** 2) < 36)).astype(np.float32)
    u1 = bpm_ref.bpm_3d((Nx, Ny, Nz), (.1, .1, .1), dn=dn, n_volumes=2, return_field=True)
    u2 = bpm_ref.bpm_3d((Nx, Ny, Nz), (.1, .1, .1), dn=dn, n_volumes=2, return_field=False)
    assert np.allclose(np.abs(u1) ** 2, u2)


def test_reflib_optional():
    """Where the reference checkout was present at build time the shim library loads."""
    lib = reflib.load()
    if lib is None:
        pytest.skip("oracle/_ref/libref_cl.so not built here")
    assert hasattr(lib, "ref_debye_wolf")
