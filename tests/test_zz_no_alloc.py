"""bpm_propagate_noalloc, the march for callers that may not allocate device memory (a host
with a fixed device budget, a plugin whose host owns all allocations, a loop where a
synchronising cudaMalloc would stall other streams): through the C ABI, its results equal
bpm_propagate's with a caller workspace bit for bit (the march's result does not depend
on how its fields are grouped), on two calls in a row (the shared scratch keeps the
previous call's contents), the second call leaves the device's free memory unchanged, and
grids too large for its fixed scratch are refused.

This file is named to be collected last, so a run that stops at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bpm_gb300 import _native as N
    from bpm_gb300.bpm3d import Plan, _slice_tables
    return torch, N, Plan, _slice_tables


def inputs(torch, size, batch, seed):
    Nx, Ny, Nz = size
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.arange(Nx, device="cuda", dtype=torch.float32) * .1
    tilt = torch.rand((batch, 1, 1), device="cuda", generator=g) * 2 - 1
    u0 = torch.exp(1j * 2 * np.pi * .4 * tilt * x[None, None, :]).to(torch.complex64).expand(batch, Ny, Nx).contiguous()
    dn = (torch.rand((Nz, Ny, Nx), device="cuda", generator=g) * .04).contiguous()
    return u0, dn


def run(torch, N, plan, u0, dn, out_kind, noalloc, tabs=(None, None), group=0, free_bytes=None):
    """One march through the C ABI; returns (status, output volume, exit planes). With
    `free_bytes` (a list), the device's free memory just before and just after the call is
    appended to it."""
    Nx, Ny, Nz = plan.size
    B = u0.shape[0]

    def p(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None
    dt = torch.complex64 if out_kind == N.OUT_FIELD else torch.float32
    out = torch.full((B, Nz, Ny, Nx), float("nan"), dtype=dt, device="cuda")
    last = torch.full((B, Ny, Nx), float("nan"), dtype=torch.complex64, device="cuda")
    req = N.Request(B, p(u0), p(dn), N.DN_F32, 0, p(tabs[0]), p(tabs[1]), p(out), out_kind, Nz * Ny * Nx,
                    p(last), None, None, 0, group)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = N.lib()
    if noalloc:
        torch.cuda.synchronize()
        if free_bytes is not None:
            free_bytes.append(torch.cuda.mem_get_info()[0])
        rc = L.bpm_propagate_noalloc(plan.handle, ctypes.byref(req), stream)
        torch.cuda.synchronize()
        if free_bytes is not None:
            free_bytes.append(torch.cuda.mem_get_info()[0])
    else:
        wsb = plan.workspace_bytes(B, 0)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        rc = L.bpm_propagate(plan.handle, ctypes.byref(req), ctypes.c_void_p(ws.data_ptr()), wsb, stream)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy(), last.cpu().numpy()


@pytest.mark.parametrize("size,batch,group,mode,out_kind", [
    ((256, 128, 12), 5, 0, "weighted", "intensity"),   # all fields in one group
    ((512, 512, 8), 4, 0, "ignore", "field"),          # the scratch holds 3 fields: two groups
    ((64, 128, 20), 3, 0, "simple", "intensity"),
    ((256, 256, 10), 16, 4, "weighted", "intensity"),  # 3 groups of 4 march at once in the array
    ((1024, 512, 5), 2, 0, "ignore", "field"),         # above 512x512: 4 MiB of plane per field
])
def test_noalloc_matches_workspace_march_twice(env, size, batch, group, mode, out_kind):
    torch, N, Plan, slice_tables = env
    plan = Plan(size, (.1, .1, .1), .5, 1.33, absorbing_width=3, mean_mode=mode)
    u0, dn = inputs(torch, size, batch, 0)
    ok = N.OUT_FIELD if out_kind == "field" else N.OUT_INTENSITY
    tabs = slice_tables(dn, 1.33, torch.device("cuda")) if mode == "simple" else (None, None)
    ref = run(torch, N, plan, u0, dn, ok, False, tabs)
    assert ref[0] == 0
    free = []
    for k in range(2):
        rc, out, last = run(torch, N, plan, u0, dn, ok, True, tabs, group=group, free_bytes=free if k else None)
        assert rc == 0, N.last_error()
        assert np.all(np.isfinite(out)) and np.all(np.isfinite(last))
        assert np.array_equal(out, ref[1])
        assert np.array_equal(last, ref[2])
    # the second call allocated nothing on the device
    assert free[0] == free[1], free


def test_noalloc_refuses_grids_beyond_its_scratch(env):
    torch, N, Plan, _ = env
    plan = Plan((1024, 1024, 4), (.1, .1, .1), .5, 1.33, mean_mode="ignore")
    u0, dn = inputs(torch, (1024, 1024, 4), 1, 1)
    rc, _, _ = run(torch, N, plan, u0, dn, N.OUT_INTENSITY, True)
    assert rc == N.BPM_ERR_OOM
    msg = N.last_error()
    assert "scratch" in msg and str(8 << 20) in msg
