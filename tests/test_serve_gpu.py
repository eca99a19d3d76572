"""The continuous-batching server: every result equals the same request run alone, the
HBM budget is respected, late arrivals join running work, and errors reach the caller."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bpm_gb300
    from bpm_gb300.serve import BpmRequest, PsfRequest, Server
    return torch, bpm_gb300, BpmRequest, PsfRequest, Server


def make_requests(BpmRequest, PsfRequest, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        if rng.uniform() < .7:
            side = int(rng.choice([32, 64, 128]))
            nz = int(rng.integers(8, 24))
            z, y, x = np.meshgrid(np.arange(nz), np.arange(side), np.arange(side), indexing="ij")
            c = rng.uniform(0, 1, 3) * (side, side, nz)
            dn = (rng.uniform(.01, .05) * ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 < (side / 5) ** 2)
                  ).astype(np.float32)
            kx = rng.uniform(-2, 2)
            u0 = np.exp(1j * kx * .1 * np.arange(side))[None, :].repeat(side, 0).astype(np.complex64)
            mode = ["weighted", "ignore"][i % 2]
            reqs.append(BpmRequest((side, side, nz), (.1, .1, .1), lam=.5, n0=1.33, u0=u0, dn=dn, mean_mode=mode,
                                   return_field=bool(i % 3 == 0), host=True))
        else:
            s = int(rng.choice([16, 32, 48]))
            reqs.append(PsfRequest((s, s, s), (.1, .1, .1), lam=float(rng.uniform(.4, .7)),
                                   NA=float(rng.uniform(.3, .9)), n0=1.33, n_integration_steps=50, host=True))
    return reqs


def alone(bpm, r):
    if hasattr(r, "shape"):
        return bpm.psf(r.shape, r.units, r.lam, r.NA, r.n0, r.n_integration_steps, return_field=r.return_field)
    return bpm.bpm_3d(r.size, r.units, lam=r.lam, n0=r.n0, u0=r.u0, dn=r.dn, mean_mode=r.mean_mode,
                      return_field=r.return_field, return_full=r.return_full)


def test_results_same_alone_and_in_the_mix(env):
    torch, bpm, BpmRequest, PsfRequest, Server = env
    reqs = make_requests(BpmRequest, PsfRequest, 40, 0)
    srv = Server(max_inflight=4, max_batch=8)
    futs = []
    rng = np.random.default_rng(1)
    for r in reqs:
        futs.append(srv.submit(r))
        time.sleep(float(rng.exponential(.002)))      # Poisson arrivals while others run
    res = [f.result(timeout=120) for f in futs]
    srv.close()
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for r, got in zip(reqs, res):
        want = alone(bpm, r)
        assert got.shape == want.shape and got.dtype == want.dtype
        assert np.array_equal(got, want), r


def test_budget_admission_and_merging(env):
    torch, bpm, BpmRequest, PsfRequest, Server = env
    side, nz = 64, 16
    dn = np.zeros((nz, side, side), np.float32)
    dn[5:10, 20:40, 20:40] = .03
    reqs = [BpmRequest((side, side, nz), (.1, .1, .1), n0=1.33, dn=dn,
                       u0=np.exp(1j * .05 * k * np.arange(side))[None].repeat(side, 0).astype(np.complex64))
            for k in range(12)]
    fp = reqs[0].footprint()
    srv = Server(hbm_budget=int(3.5 * fp), max_inflight=8, max_batch=8)
    futs = [srv.submit(r) for r in reqs]
    out = [f.result(timeout=60) for f in futs]
    srv.close()
    assert srv.peak_used <= srv.budget
    st = srv.stats()
    # requests with the same grid and physics were merged into batched launches
    assert st["merged_launches"] >= 1 and st["launches"] < len(reqs), st
    for r, o in zip(reqs, out):
        want = bpm.bpm_3d(r.size, r.units, lam=r.lam, n0=r.n0, u0=r.u0, dn=r.dn, return_field=False)
        assert np.array_equal(o.cpu().numpy(), want)


def test_launches_overlap_on_the_device(env):
    """Requests that cannot merge (four Nz) submitted together run as four launches on their
    own streams: more than one is in flight at once, and their device intervals (CUDA
    events on each launch's stream) overlap; each result equals the request alone."""
    torch, bpm, BpmRequest, PsfRequest, Server = env
    side = 512
    reqs = []
    for k, nz in enumerate((96, 112, 128, 144)):
        u0 = np.exp(1j * .03 * (k + 1) * np.arange(side))[None].repeat(side, 0).astype(np.complex64)
        reqs.append(BpmRequest((side, side, nz), (.1, .1, .1), n0=1.33, u0=u0, mean_mode="ignore",
                               return_field=False, return_full=False))
    for _ in range(2):   # the first pass builds the plans and fills the allocator's cache
        srv = Server(max_inflight=4, max_batch=8)
        futs = [srv.submit(r) for r in reqs]
        out = [f.result(timeout=60) for f in futs]
        srv.close()
    st = srv.stats()
    assert st["launches"] == 4 and st["merged_launches"] == 0, st
    assert st["max_inflight_seen"] >= 2, st
    assert st["overlapped_launches"] >= 2, (st, srv.spans)
    for r, o in zip(reqs, out):
        want = bpm.bpm_3d(r.size, r.units, lam=r.lam, n0=r.n0, u0=r.u0, mean_mode="ignore", return_field=False,
                          return_full=False)
        assert np.array_equal(o.cpu().numpy(), want)


def test_cancelled_requests_are_dropped(env):
    """Futures cancelled while their requests wait are dropped by the scheduler; the other
    requests complete with the same results as alone, and the server keeps serving."""
    torch, bpm, BpmRequest, PsfRequest, Server = env
    side, nz = 64, 12
    reqs = [BpmRequest((side, side, nz), (.1, .1, .1), n0=1.33, mean_mode="ignore",
                       u0=np.exp(1j * .04 * k * np.arange(side))[None].repeat(side, 0).astype(np.complex64))
            for k in range(16)]
    # a budget of one request at a time keeps the later ones waiting long enough to cancel
    srv = Server(hbm_budget=int(1.5 * reqs[0].footprint()), max_inflight=1, max_batch=1)
    futs = [srv.submit(r) for r in reqs]
    cancelled = [f.cancel() for f in futs[8:]]
    done = [f.result(timeout=60) for f in futs[:8]]
    for f, c in zip(futs[8:], cancelled):
        if c:
            assert f.cancelled()
        else:   # admitted before the cancel arrived: it runs to the end
            f.result(timeout=60)
    assert any(cancelled)
    late = srv.submit(reqs[0]).result(timeout=60)
    srv.close()
    assert srv.error is None
    for r, o in zip(reqs[:8], done):
        want = bpm.bpm_3d(r.size, r.units, lam=r.lam, n0=r.n0, u0=r.u0, mean_mode="ignore", return_field=False)
        assert np.array_equal(o.cpu().numpy(), want)
    assert np.array_equal(late.cpu().numpy(), done[0].cpu().numpy())


def test_oversized_request_is_refused(env):
    torch, bpm, BpmRequest, PsfRequest, Server = env
    srv = Server(hbm_budget=1 << 20)
    f = srv.submit(BpmRequest((256, 256, 64), (.1, .1, .1)))
    with pytest.raises(MemoryError):
        f.result(timeout=5)
    srv.close()


def test_bad_request_reports_error(env):
    torch, bpm, BpmRequest, PsfRequest, Server = env
    srv = Server()
    f = srv.submit(BpmRequest((100, 64, 8), (.1, .1, .1)))   # not a power-of-two grid
    with pytest.raises(NotImplementedError):
        f.result(timeout=30)
    srv.close()
