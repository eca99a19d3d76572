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


@pytest.mark.parametrize("name", ["spheres_a", "spheres_b"])
def test_spheres_oracle_bit_exact(golden, name):
    """bpm_3d_spheres.cl:fill_dn (reference kernel) against the numpy restatement."""
    from oracle import spheres_ref
    a = golden[name + "_args"]
    size = tuple(int(v) for v in a[:3])
    r = a[6:10]
    dn = spheres_ref.create_dn_buffer(size, tuple(a[3:6]), golden[name + "_pts"], r[0], r[1], r[2], r[3])
    assert np.array_equal(dn, golden[name + "_out"])


@pytest.mark.parametrize("name", ["gauss_a", "gauss_b"])
def test_debye_gauss_oracle_vs_reference_kernel(golden, name):
    """debye_wolf_gauss (reference kernel) + the gauss spreading loop against the restatement;
    gauss_b has odd shapes and two annuli."""
    a = golden[name + "_args"]
    shape = tuple(int(v) for v in a[:3])
    o = debye_ref.focus_field_debye_gauss(shape, tuple(a[3:6]), a[6], list(golden[name + "_NA"]), a[7], int(a[8]))
    for v, k in zip(o, ("u", "ex", "ey", "ez")):
        assert v.shape == shape[::-1]
        assert rel_l2(v, golden["%s_%s" % (name, k)]) < 5e-6, k


@pytest.mark.parametrize("name", ["plane_a", "plane_b"])
def test_debye_plane_oracle_vs_reference_kernel(golden, name):
    Nx, Ny, dx, dy, z, lam, NA, n0, steps = golden[name + "_args"]
    o = debye_ref.focus_field_debye_plane((int(Nx), int(Ny)), (dx, dy), z, lam, NA, n0, int(steps))
    assert o.shape == (int(Ny), int(Nx))
    assert rel_l2(o, golden[name + "_ex"]) < 5e-6


def test_debye_at_oracle_vs_reference_kernel(golden):
    p = golden["at_a_pts"]
    lam, n0, steps = golden["at_a_args"]
    o = debye_ref.focus_field_debye_at(p[0], p[1], p[2], lam, list(golden["at_a_NA"]), n0, int(steps))
    for v, k in zip(o, ("u", "ex", "ey", "ez")):
        assert rel_l2(v, golden["at_a_" + k]) < 5e-6, k


def test_sine_rule_end_weights():
    """psf_debye.cl:155: the half weight follows the float32 test t == a2, so node
    INT_STEPS-1 gets it only when a1 + (INT_STEPS-1)*dt rounds exactly onto a2."""
    hits = []
    for NA in (.3, .5, .8, 1.0):
        a = np.arcsin(np.array([0., NA])).astype(np.float32)
        t, w = debye_ref.quadrature_nodes_f32_ends(a, 200)
        dt = w[1]
        assert w[0] == .5 * dt and w[-1] == dt
        f = np.float32
        t32 = f(a[0]) + f(199) * ((a[1] - a[0]) / f(199.))
        hits.append(w[-2] == .5 * dt)
        assert hits[-1] == (t32 == a[1])
    assert any(hits) and not all(hits)


@pytest.mark.parametrize("N0", [5, 6, 9, 16])
def test_gauss_mirror_index_form_equals_slice_loop(N0):
    rng = np.random.default_rng(N0)
    shape = (N0, N0 + 1, 3)
    No = [(s + 1) // 2 for s in shape]
    u = rng.normal(size=(No[2], No[1], No[0])).astype(np.float32)
    e = (rng.normal(size=u.shape) + 1j * rng.normal(size=u.shape)).astype(np.complex64)
    U, E, _, _ = debye_ref.mirror_octant_gauss(shape, u, e, e, e)
    ix, iy, iz = (debye_ref.mirror_index_gauss(s) for s in shape)
    assert np.array_equal(U, u[iz][:, iy][:, :, ix])
    assert np.array_equal(E, e[iz][:, iy][:, :, ix])
