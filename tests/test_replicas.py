"""Multi-rank host logic on CPU (gloo, world size 2): the field shards partition a batch,
max-over-ranks timing, and the sharded gradient (each rank differentiates the march for its
own illumination angles, then one all-reduce) equals the single-process gradient. The
march here is an FP64 torch restatement of the ignore-mode split step, so no GPU is used."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from bpm_gb300.replicas import shard


@pytest.mark.parametrize("batch,world", [(10, 2), (7, 3), (1, 1), (64, 8), (3, 4)])
def test_shards_partition_the_batch(batch, world):
    seen = []
    sizes = []
    for r in range(world):
        b0, b1 = shard(batch, r, world)
        seen += list(range(b0, b1))
        sizes.append(b1 - b0)
    assert seen == list(range(batch))
    assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(batch, world, world)


def march64(dn, u0, dz, k0, H):
    u = u0
    for i in range(dn.shape[0] - 1):
        u = torch.fft.ifft2(torch.fft.fft2(u) * H)
        u = u * torch.exp(-1j * (k0 * dz) * dn[i + 1])
    return u


def problem():
    from oracle import bpm_ref
    Nx = Ny = 16
    Nz = 6
    k0 = 2 * np.pi / .5
    H, _ = bpm_ref.propagator_f64(1.33, k0, .1, .1, .1, Nx, Ny)
    rng = np.random.default_rng(0)
    dn = rng.uniform(0, .03, (Nz, Ny, Nx))
    tilts = rng.uniform(-1, 1, (5, 2))
    x = .1 * np.arange(Nx)
    u0 = np.exp(1j * (tilts[:, 0, None, None] * x[None, None, :] + tilts[:, 1, None, None] * x[None, :, None]))
    target = rng.uniform(.5, 1.5, (5, Ny, Nx))
    return dn, u0, target, H, k0


def grad_for(idx, dn, u0, target, H, k0):
    d = torch.tensor(dn, requires_grad=True)
    u = march64(d, torch.tensor(u0[idx]), .1, k0, torch.tensor(H))
    ((u.abs() ** 2 - torch.tensor(target[idx])) ** 2).sum().backward()
    return d.grad


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    from bpm_gb300.replicas import max_over_ranks, sum_over_ranks, shard as sh
    dn, u0, target, H, k0 = problem()
    b0, b1 = sh(u0.shape[0], rank, world)
    g = grad_for(slice(b0, b1), dn, u0, target, H, k0)
    sum_over_ranks(g)
    t = max_over_ranks(float(rank + 1))
    if rank == 0:
        q.put((g.numpy(), t))
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_sharded_gradient_equals_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    g_sharded, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    dn, u0, target, H, k0 = problem()
    g_full = grad_for(slice(0, u0.shape[0]), dn, u0, target, H, k0).numpy()
    assert t == 2.0
    assert np.allclose(g_sharded, g_full, rtol=1e-10, atol=1e-14)


def test_torch_restatement_matches_the_oracle():
    """The FP64 torch march differentiated above is the oracle's ignore-mode march (the
    reference's mult_propagator + mult_dn step, no taper): same last plane to rounding."""
    from oracle import bpm_ref
    dn, u0, _, H, k0 = problem()
    Nz, Ny, Nx = dn.shape
    dn32 = dn.astype(np.float32)
    for b in range(u0.shape[0]):
        f0 = u0[b].astype(np.complex64)
        got = march64(torch.tensor(dn32.astype(np.float64)), torch.tensor(f0.astype(np.complex128)), .1, k0,
                      torch.tensor(H)).numpy()
        want = bpm_ref.bpm_3d((Nx, Ny, Nz), (.1, .1, .1), lam=.5, n0=1.33, u0=f0, dn=dn32, mean_mode="ignore",
                              return_full=False, precision="fp64")
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-6, b
