"""Parity at the sizes and depths that are benchmarked: every z-step of the full march,
against the FP64 oracle (oracle/bpm_ref.py, the reference's per-step loop
bpm/bpm/bpm_3d.py:283-381 restated in float64), relative L2 <= 1e-4 on the |u|^2 volume
and on the exit field.

(a) the batched workload of the benchmark: plane waves with tilts area-uniform in NA 0.8
    through one shared seeded Gaussian-random 512x512x256 dn (correlation 5 px, sigma
    0.02, clipped to +-0.06), weighted mean mode, marched 8 fields per launch through the
    captured CUDA graph (the kernels the benchmark times); two of the fields are checked
    over all 255 steps;
(b) the single large request: 256^3, 50 seeded spheres with complex dn (Re U[0.01, 0.05],
    Im U[0, 1e-3], radius U[3, 15] px), the Gaussian focus psf_u0(NA 0.4, zfoc 12.8 um)
    as input, mean mode "ignore" (the one complex dn is defined for);
(c) the largest grid of the serving trace: one 1024x1024x256 field through complex
    random spheres, mean mode "ignore"; and a 1024x1024x128 weighted march.
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import bpm_ref

pytestmark = pytest.mark.gpu

TOL = 1e-4
UNITS = (.1, .1, .1)
LAM, N0 = .5, 1.33


@pytest.fixture(scope="module")
def bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    return bpm_gb300


def gaussian_random_dn(nx, ny, nz, seed, corr=5., sigma=.02, clip=.06):
    """Gaussian-filtered white noise (correlation length `corr` px), scaled to std
    `sigma` and clipped, float32 (the benchmark's dn recipe, generated on the host)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nz, ny, nx))
    fz = np.fft.fftfreq(nz)[:, None, None]
    fy = np.fft.fftfreq(ny)[None, :, None]
    fx = np.fft.fftfreq(nx)[None, None, :]
    f = np.fft.ifftn(np.fft.fftn(w) * np.exp(-2 * np.pi ** 2 * corr ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))).real
    f *= sigma / f.std()
    return np.clip(f, -clip, clip).astype(np.float32)


def tilted_waves(batch, nx, ny, seed, na=.8):
    """Plane waves exp(-i (kx x + ky y)) with (kx, ky) = k0 (NA_x, NA_y) drawn
    area-uniformly in the disk of radius `na`."""
    rng = np.random.default_rng(seed)
    r = na * np.sqrt(rng.uniform(0, 1, batch))
    th = 2 * np.pi * rng.uniform(0, 1, batch)
    k0 = 2 * np.pi / LAM
    kx, ky = k0 * r * np.cos(th), k0 * r * np.sin(th)
    x = UNITS[0] * np.arange(nx)
    y = UNITS[1] * np.arange(ny)
    return np.exp(-1j * (kx[:, None, None] * x[None, None, :] + ky[:, None, None] * y[None, :, None])
                  ).astype(np.complex64)


def complex_spheres(side, nz, seed, n=50, rmin=3., rmax=15.):
    """n spheres with centres uniform in the volume, radius U[rmin, rmax] px,
    Re dn U[0.01, 0.05], Im dn U[0, 1e-3] (later spheres overwrite earlier ones)."""
    rng = np.random.default_rng(seed)
    dn = np.zeros((nz, side, side), np.complex64)
    for _ in range(n):
        c = rng.uniform(0, 1, 3) * (side, side, nz)
        r = rng.uniform(rmin, rmax)
        v = complex(rng.uniform(.01, .05), rng.uniform(0, 1e-3))
        # the sphere's bounding box only
        lo = [max(0, int(np.floor(c[k] - r))) for k in range(3)]
        hi = [min(s, int(np.ceil(c[k] + r)) + 1) for k, s in enumerate((side, side, nz))]
        z = np.arange(lo[2], hi[2])[:, None, None]
        y = np.arange(lo[1], hi[1])[None, :, None]
        x = np.arange(lo[0], hi[0])[None, None, :]
        box = dn[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        box[((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) <= r * r] = v
    return dn


def oracle_fp64(size, u0, dn, mode):
    """FP64 |u|^2 volume and exit field of one field."""
    vol, last = bpm_ref._bpm_3d(size, UNITS, lam=LAM, n0=N0, u0=u0, dn=dn, mean_mode=mode, return_field=False,
                                return_last_plane=True, precision="fp64")
    return vol, last


def rel_l2_planes(a, b):
    """rel_l2 over a volume, accumulated plane by plane (bounded host memory)."""
    num = den = 0.
    for z in range(b.shape[0]):
        d = a[z].astype(np.float64) - b[z]
        num += float(np.vdot(d, d).real)
        den += float(np.vdot(b[z], b[z]).real)
    return (num / den) ** .5


def test_batched_512_weighted_full_depth(bpm):
    """(a): 8 fields per launch through the captured graph, fields 0 and 5 checked over
    all 255 steps."""
    import torch
    nx = ny = 512
    nz = 256
    dn = gaussian_random_dn(nx, ny, nz, seed=11)
    u0 = tilted_waves(8, nx, ny, seed=12)
    march = bpm.BatchedMarch((nx, ny, nz), UNITS, LAM, N0, 8, dn=torch.from_numpy(dn).cuda(), mean_mode="weighted",
                             out_kind="intensity", group=8)
    march.u0.copy_(torch.from_numpy(u0))
    march.run()
    torch.cuda.synchronize()
    for b in (0, 5):
        vol, last = oracle_fp64((nx, ny, nz), u0[b], dn, "weighted")
        e_vol = rel_l2_planes(march.out[b].cpu().numpy(), vol)
        e_last = rel_l2(march.last[b].cpu().numpy(), last)
        print("batched 512^2 x 256 weighted, field %d: |u|^2 volume %.3e, exit field %.3e" % (b, e_vol, e_last))
        assert e_vol < TOL
        assert e_last < TOL


def test_config2_bpm_full_size(bpm):
    """(b): 256^3, 50 complex-dn spheres, Gaussian focus input, through bpm_3d."""
    side = nz = 256
    dn = complex_spheres(side, nz, seed=2)
    u0 = bpm.psf_u0((side, side), (.1, .1), zfoc=12.8, NA=.4, lam=LAM, n0=N0)
    u0 = np.asarray(u0, np.complex64)
    vol_g = bpm.bpm_3d((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dn, mean_mode="ignore",
                       return_field=False)
    last_g = bpm.bpm_3d((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dn, mean_mode="ignore",
                        return_full=False)
    vol, last = oracle_fp64((side, side, nz), u0, dn, "ignore")
    e_vol, e_last = rel_l2_planes(vol_g, vol), rel_l2(last_g, last)
    print("config 2 BPM 256^3 complex spheres: |u|^2 volume %.3e, exit field %.3e" % (e_vol, e_last))
    assert e_vol < TOL
    assert e_last < TOL


@pytest.mark.parametrize("nz,mode", [(256, "ignore"), (128, "weighted")])
def test_1024_full_depth(bpm, nz, mode):
    """(c): one 1024x1024 field, complex random spheres (ignore) or real ones (weighted)."""
    side = 1024
    dn = complex_spheres(side, nz, seed=3, n=120)
    if mode == "weighted":
        dn = np.ascontiguousarray(dn.real)
    u0 = tilted_waves(1, side, side, seed=4, na=.5)[0]
    vol_g = bpm.bpm_3d((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dn, mean_mode=mode, return_field=False)
    last_g = bpm.bpm_3d((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dn, mean_mode=mode, return_full=False)
    vol, last = oracle_fp64((side, side, nz), u0, dn, mode)
    e_vol, e_last = rel_l2_planes(vol_g, vol), rel_l2(last_g, last)
    print("1024^2 x %d %s: |u|^2 volume %.3e, exit field %.3e" % (nz, mode, e_vol, e_last))
    assert e_vol < TOL
    assert e_last < TOL
