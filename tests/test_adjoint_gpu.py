"""The hand-written adjoint (bpm_backward behind torch autograd) against FP64 central finite
differences of the CPU oracle and against FP64 torch autograd through a torch.fft
restatement of the same march (the reference gradient; the reference itself has none).
Loss: L = sum (|u_out|^2 - I_target)^2 over the exit planes of several illumination angles."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import bpm_ref, torch_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_bpm():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    from bpm_gb300.adjoint import propagate_exit
    return torch, bpm_gb300, propagate_exit


def spheres(Nx, Ny, Nz, n, seed, lo=.01, hi=.04, rmin=3, rmax=8):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    dn = np.zeros((Nz, Ny, Nx), np.float64)
    for _ in range(n):
        c = rng.uniform(.2, .8, 3) * (Nx, Ny, Nz)
        r = rng.uniform(rmin, rmax)
        dn[(x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= r * r] = rng.uniform(lo, hi)
    return dn


def tilted_waves(B, Nx, Ny, dx, lam, na_max, seed):
    rng = np.random.default_rng(seed)
    r = na_max * np.sqrt(rng.uniform(0, 1, B))
    th = 2 * np.pi * rng.uniform(0, 1, B)
    k0 = 2 * np.pi / lam
    x = dx * np.arange(Nx)
    y = dx * np.arange(Ny)
    return np.exp(-1j * (k0 * r * np.cos(th))[:, None, None] * x[None, None, :]
                  - 1j * (k0 * r * np.sin(th))[:, None, None] * y[None, :, None]).astype(np.complex64)


def torch_march64(torch, dn, u0, size, units, lam, n0, absorbing_width=0):
    """FP64 torch restatement of the ignore-mode march (FP32-recipe mask, FP64 phase)."""
    return torch_ref.march_exit_fp64(torch, dn, u0, size, units, lam, n0, absorbing_width)


def test_gradient_vs_fp64_finite_differences(torch_bpm):
    """64x64x32 sub-grid, central differences in FP64 with eps = 1e-6 on the oracle."""
    torch, bpm, propagate_exit = torch_bpm
    Nx = Ny = 64
    Nz = 32
    size, units, lam, n0 = (Nx, Ny, Nz), (.1, .1, .1), .5, 1.33
    B = 3
    u0 = tilted_waves(B, Nx, Ny, .1, lam, .6, 1)
    dn_true = spheres(Nx, Ny, Nz, 4, 2)
    dn = .5 * dn_true
    I_t = np.stack([np.abs(bpm_ref.bpm_3d(size, units, lam=lam, n0=n0, u0=u0[b], dn=dn_true, mean_mode="ignore",
                                          return_full=False, precision="fp64")) ** 2 for b in range(B)])

    def loss64(d):
        L = 0.
        for b in range(B):
            u = bpm_ref.bpm_3d(size, units, lam=lam, n0=n0, u0=u0[b], dn=d, mean_mode="ignore",
                               return_full=False, precision="fp64")
            L += np.sum((np.abs(u) ** 2 - I_t[b]) ** 2)
        return L

    dn_t = torch.tensor(dn, dtype=torch.float32, device="cuda", requires_grad=True)
    out = propagate_exit(dn_t, torch.as_tensor(u0, device="cuda"), size, units, lam, n0, ckpt_every=8)
    L = ((out.abs() ** 2 - torch.as_tensor(I_t, device="cuda")) ** 2).sum()
    L.backward()
    grad = dn_t.grad.cpu().numpy()
    assert np.all(grad[0] == 0)
    rng = np.random.default_rng(3)
    # voxels where the gradient is large (inside the beam paths), plus random ones
    flat = np.argsort(np.abs(grad).ravel())[::-1][:4].tolist() + rng.integers(Nx * Ny, Nz * Nx * Ny, 4).tolist()
    eps = 1e-6
    scale = np.abs(grad).max()
    for f in flat:
        idx = np.unravel_index(f, grad.shape)
        dp = dn.copy()
        dm = dn.copy()
        dp[idx] += eps
        dm[idx] -= eps
        fd = (loss64(dp) - loss64(dm)) / (2 * eps)
        assert abs(grad[idx] - fd) <= 2e-3 * abs(fd) + 1e-4 * scale, (idx, grad[idx], fd)


@pytest.mark.parametrize("size", [(64, 32, 24), (256, 128, 10), (128, 512, 6), (1024, 64, 5)])
def test_gradient_vs_torch_fp64_autograd(torch_bpm, size):
    """Forward exit field, d(loss)/d(dn) and d(loss)/d(u0) against FP64 torch autograd of
    the restated march: tile kernels (64, 32), warp row / column-split kernels (128 .. 512),
    1024-point rows; with and without the absorbing taper."""
    torch, bpm, propagate_exit = torch_bpm
    units, lam, n0 = (.1, .1, .1), .5, 1.33
    Nx, Ny, Nz = size
    u0 = tilted_waves(4, Nx, Ny, .1, lam, .6, 5)
    dn = spheres(Nx, Ny, Nz, 3, 6)
    I_t = np.random.default_rng(0).uniform(.5, 1.5, (4, Ny, Nx))
    for aw in (0, 4):
        dn64 = torch.tensor(dn, dtype=torch.float64, device="cuda", requires_grad=True)
        u064 = torch.tensor(u0.astype(np.complex128), device="cuda", requires_grad=True)
        ref = torch_march64(torch, dn64, u064, size, units, lam, n0, aw)
        ((ref.abs() ** 2 - torch.as_tensor(I_t, device="cuda")) ** 2).sum().backward()
        dn32 = torch.tensor(dn, dtype=torch.float32, device="cuda", requires_grad=True)
        u032 = torch.tensor(u0, device="cuda", requires_grad=True)
        out = propagate_exit(dn32, u032, size, units, lam, n0, absorbing_width=aw, ckpt_every=5)
        assert rel_l2(out.detach().cpu().numpy(), ref.detach().cpu().numpy()) < 1e-4
        ((out.abs() ** 2 - torch.as_tensor(I_t, device="cuda")) ** 2).sum().backward()
        assert rel_l2(dn32.grad.cpu().numpy(), dn64.grad.cpu().numpy()) < 1e-3
        assert rel_l2(u032.grad.cpu().numpy(), u064.grad.cpu().numpy()) < 1e-3


def test_checkpoint_spacing_does_not_change_the_gradient(torch_bpm):
    torch, bpm, propagate_exit = torch_bpm
    size = (32, 32, 20)
    u0 = torch.as_tensor(tilted_waves(2, 32, 32, .1, .5, .5, 7), device="cuda")
    dn = torch.tensor(spheres(32, 32, 20, 2, 8), dtype=torch.float32, device="cuda")
    grads = []
    for k in (1, 3, 19, 40):
        d = dn.clone().requires_grad_(True)
        out = propagate_exit(d, u0, size, (.1, .1, .1), .5, 1.33, ckpt_every=k)
        (out.abs() ** 4).sum().backward()
        grads.append(d.grad)
    for g in grads[1:]:
        assert torch.equal(g, grads[0])


def test_config4_inversion_gradient(torch_bpm):
    """256x256x128 grid, 16 illumination angles within NA 0.6, checkpoints every 16
    slices; I_target from a ground-truth dn of 20 spheres (dn 0.01-0.04). The gradient at
    an inversion iterate dn = 0.5 dn_true (the march through the spheres scatters, so every
    mask derivative sees a scattered field) against FP64 torch autograd of the restated
    march, relative L2 <= 1e-4."""
    torch, bpm, propagate_exit = torch_bpm
    size, units, lam, n0 = (256, 256, 128), (.1, .1, .1), .5, 1.33
    Nx, Ny, Nz = size
    u0 = torch.as_tensor(tilted_waves(16, Nx, Ny, .1, lam, .6, 11), device="cuda")
    dn_true = torch.tensor(spheres(Nx, Ny, Nz, 20, 12, rmin=3, rmax=15), dtype=torch.float32, device="cuda")
    with torch.no_grad():
        I_t = propagate_exit(dn_true, u0, size, units, lam, n0).abs() ** 2
    dn = (.5 * dn_true).requires_grad_(True)
    out = propagate_exit(dn, u0, size, units, lam, n0, ckpt_every=16)
    L = ((out.abs() ** 2 - I_t) ** 2).sum()
    L.backward()
    dn64 = (.5 * dn_true).double().requires_grad_(True)
    ref = torch_march64(torch, dn64, u0.to(torch.complex128), size, units, lam, n0)
    ((ref.abs() ** 2 - I_t.double()) ** 2).sum().backward()
    err = rel_l2(dn.grad.cpu().numpy(), dn64.grad.cpu().numpy())
    print("config 4 gradient at 0.5 dn_true: rel-L2 %.3e against FP64 autograd" % err)
    assert err < 1e-4, err


@pytest.mark.parametrize("group", [0, 5, 12])
def test_summed_gradient_matches_per_field_sum(torch_bpm, group):
    """Fields sharing one dn: the library sums the dn gradient over them (bpm_request.grad_sum,
    row_adj_shared_kernel, per-block partials added in block order when a group spans more
    than 8 fields). Same result as the per-field gradients summed (a per-field dn volume per
    field), to FP32 rounding, and bit-identical from run to run; groups of 5 (three
    sequential groups added in order) and of 12 (two row blocks per row)."""
    torch, bpm, propagate_exit = torch_bpm
    size, units, lam, n0 = (256, 128, 12), (.1, .1, .1), .5, 1.33
    Nx, Ny, Nz = size
    B = 12
    u0 = torch.as_tensor(tilted_waves(B, Nx, Ny, .1, lam, .6, 21), device="cuda")
    dn0 = torch.tensor(spheres(Nx, Ny, Nz, 3, 22), dtype=torch.float32, device="cuda")
    I_t = torch.as_tensor(np.random.default_rng(1).uniform(.5, 1.5, (B, Ny, Nx)), device="cuda")

    def grad_of(dn):
        d = dn.clone().requires_grad_(True)
        out = propagate_exit(d, u0, size, units, lam, n0, ckpt_every=4, group=group)
        ((out.abs() ** 2 - I_t) ** 2).sum().backward()
        return d.grad

    g1, g2 = grad_of(dn0), grad_of(dn0)
    assert torch.equal(g1, g2)
    per_field = grad_of(dn0.expand(B, Nz, Ny, Nx).contiguous()).double().sum(dim=0)
    assert torch.all(g1[0] == 0)
    assert rel_l2(g1.double().cpu().numpy(), per_field.cpu().numpy()) < 1e-6
