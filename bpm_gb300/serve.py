"""Continuous-batching server for propagation and PSF requests on one GPU.

Requests (`BpmRequest`, `PsfRequest`) arrive at any time through `Server.submit`, which
returns a future. A scheduler thread
  * admits requests in arrival order while their HBM footprint (inputs, outputs and
    workspace, estimated before launch) fits the budget and an execution slot is free;
  * merges admitted BPM requests that share a grid and physics (size, units, lam, n0,
    mean mode, taper, dn dtype) into one batched launch, so a late arrival joins the
    next launch instead of waiting for a whole queue to drain. Fields whose dn is the
    same resident CUDA volume march it in place (no copy; for several fields its phase
    masks are computed once); other dn volumes are gathered into one per-field buffer
    (bpm_propagate with dn_batch_stride);
  * runs every launch on its own CUDA stream from a pool, so requests of different grid
    sizes and PSFs overlap on the device, and retires launches as their CUDA events
    complete, returning memory and slots to admission.
Inputs are uploaded once and stay resident until the request retires; results stay on
the device (torch tensors) unless the request asks for host arrays. Latency is measured
from `submit` to the completion of the request's work on the device.

The reference has no serving path; results are identical to bpm_3d / psf on the same
request alone (a batched launch computes every field exactly as a single-field one).
"""
import ctypes
import itertools
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from .bpm3d import _dn_kind, _ptr, get_plan, mask_pays, precompute_mask
from .psf import _debye, _desc

__all__ = ["BpmRequest", "PsfRequest", "Server"]


@dataclass
class BpmRequest:
    """One bpm_3d call: size=(Nx, Ny, Nz), units, lam, n0, u0 (Ny, Nx) or None, dn
    (Nz, Ny, Nx) or None, mean_mode ("ignore" or "weighted"; "simple" is not merged),
    absorbing_width, return_field, return_full, host (return numpy). A contiguous CUDA
    dn tensor is read in place until the request completes: do not modify it meanwhile."""
    size: tuple
    units: tuple
    lam: float = .5
    n0: float = 1.
    u0: object = None
    dn: object = None
    mean_mode: str = "weighted"
    absorbing_width: int = 0
    return_field: bool = False
    return_full: bool = True
    host: bool = False

    def key(self):
        kind, _ = _dn_kind(self.dn, False)
        return ("bpm", tuple(int(s) for s in self.size), tuple(float(u) for u in self.units), float(self.lam),
                float(self.n0), self.mean_mode, int(self.absorbing_width), kind, bool(self.return_field),
                bool(self.return_full))

    def voxel_updates(self):
        Nx, Ny, Nz = self.size
        return Nx * Ny * (Nz - 1)

    def footprint(self):
        Nx, Ny, Nz = self.size
        plane = Nx * Ny
        b = plane * 8 * 3                                    # u0, last plane, workspace plane
        if self.dn is not None:
            cplx = self.dn.is_complex() if torch.is_tensor(self.dn) else np.iscomplexobj(self.dn)
            b += Nz * plane * (8 if cplx else 4)
            b += Nz * plane * 8  # phase masks, if the launch precomputes them (an upper bound)
        if self.return_full:
            b += Nz * plane * (8 if self.return_field else 4)
        return b


@dataclass
class PsfRequest:
    """One psf call: shape=(Nx, Ny, Nz), units, lam, NA, n0, n_integration_steps,
    return_field, host."""
    shape: tuple
    units: tuple
    lam: float = .5
    NA: object = .8
    n0: float = 1.
    n_integration_steps: int = 200
    return_field: bool = False
    host: bool = False

    def key(self):
        return ("psf", id(self))

    def voxel_updates(self):
        return 0

    def footprint(self):
        # computed once: the scheduler asks at submission and again at admission
        fp = self.__dict__.get("_footprint")
        if fp is None:
            fp = self.__dict__["_footprint"] = self._footprint()
        return fp

    def _footprint(self):
        Nx, Ny, Nz = self.shape
        n_na = 2 if np.isscalar(self.NA) else len(self.NA)
        T = n_na // 2 * (self.n_integration_steps + 1)
        M = (Nx // 2 + 1) * (Ny // 2 + 1)
        # an upper estimate of the tables (Bessel rows, phases, integrals), used when the
        # library rejects the description (the launch then reports the error)
        ws = 4 * 3 * T * M + 8 * 3 * (Nz // 2 + 1) * M + 8 * T * (Nz // 2 + 1)
        try:
            # the library's exact figure (node, radius and angle tables and row padding)
            desc, _na = _desc(self.shape, self.units, self.lam, self.NA, self.n0, self.n_integration_steps)
            exact = int(N.lib().debye_workspace_bytes(ctypes.byref(desc)))
            if exact > 0:
                ws = exact
        except (AssertionError, TypeError, ValueError):
            pass
        return ws + Nx * Ny * Nz * (28 if self.return_field else 4)


@dataclass
class _Entry:
    req: object
    fut: Future
    t_submit: float
    seq: int


@dataclass
class _Launch:
    entries: list
    stream: torch.cuda.Stream
    start: torch.cuda.Event
    done: torch.cuda.Event
    footprint: int
    keep: list = field(default_factory=list)
    results: list = field(default_factory=list)


class Server:
    """Continuous-batching scheduler. hbm_budget: bytes the in-flight work may hold;
    max_inflight: concurrent launches (CUDA streams); max_batch: fields per BPM launch."""

    def __init__(self, hbm_budget=None, max_inflight=8, max_batch=32, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(free * .7)
        self.budget = int(hbm_budget)
        self.max_inflight = int(max_inflight)
        self.max_batch = int(max_batch)
        self._inbox = queue.Queue()
        self._pending = []
        self._inflight = []
        self._used = 0
        self._seq = itertools.count()
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.max_inflight)]
        self._free_streams = list(self._streams)
        self._stop = threading.Event()
        self.latencies = []
        self.completed = 0
        self.voxel_updates = 0
        self.peak_used = 0
        # what the scheduler did: launches, launches that merged several requests, the most
        # launches in flight at once, and each retired launch's device interval (ms after
        # the server started), measured by CUDA events on the launch's stream
        self.launches = 0
        self.merged_launches = 0
        self.max_inflight_seen = 0
        self.spans = []
        self._t0 = torch.cuda.Event(enable_timing=True)
        self._t0.record(torch.cuda.current_stream(self.device))
        self.error = None
        self._thread = threading.Thread(target=self._loop, name="bpm-serve", daemon=True)
        self._thread.start()

    # ---------------------------------------------------------------------------------
    def submit(self, req):
        fut = Future()
        if req.footprint() > self.budget:
            fut.set_exception(MemoryError("request footprint %d B exceeds the HBM budget %d B"
                                          % (req.footprint(), self.budget)))
            return fut
        self._inbox.put(_Entry(req, fut, time.perf_counter(), next(self._seq)))
        return fut

    def close(self, wait=True):
        self._stop.set()
        if wait:
            self._thread.join()

    def stats(self):
        lat = np.array(self.latencies) * 1e3
        return {"completed": self.completed,
                "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                "mean_ms": float(lat.mean()) if len(lat) else None,
                "voxel_updates": int(self.voxel_updates), "peak_hbm_bytes": int(self.peak_used),
                "budget_bytes": self.budget, "launches": self.launches,
                "merged_launches": self.merged_launches, "max_inflight_seen": self.max_inflight_seen,
                "overlapped_launches": overlapped(self.spans)}

    # ---------------------------------------------------------------------------------
    def _loop(self):
        torch.cuda.set_device(self.device)
        try:
            while True:
                self._drain_inbox(block=not (self._pending or self._inflight))
                self._retire()
                self._admit()
                if self._stop.is_set() and not self._pending and not self._inflight and self._inbox.empty():
                    break
                if self._inflight and not self._pending:
                    time.sleep(0.0002)
        except Exception as e:  # pragma: no cover - surfaced through the futures
            self.error = e
            for en in self._pending:
                if not en.fut.done():
                    en.fut.set_exception(e)
            for la in self._inflight:
                for en in la.entries:
                    if not en.fut.done():
                        en.fut.set_exception(e)

    def _drain_inbox(self, block):
        try:
            if block:
                en = self._inbox.get(timeout=0.005)
                self._pending.append(en)
            while True:
                self._pending.append(self._inbox.get_nowait())
        except queue.Empty:
            pass

    def _retire(self):
        still = []
        for la in self._inflight:
            if la.done.query():
                t = time.perf_counter()
                for en, res in zip(la.entries, la.results):
                    self.latencies.append(t - en.t_submit)
                    self.completed += 1
                    self.voxel_updates += en.req.voxel_updates()
                    if en.req.host:
                        res = _to_host(res)
                    en.fut.set_result(res)
                self.spans.append((self._t0.elapsed_time(la.start), self._t0.elapsed_time(la.done)))
                self._used -= la.footprint
                self._free_streams.append(la.stream)
                la.keep.clear()
            else:
                still.append(la)
        self._inflight = still

    def _drop_cancelled(self):
        """Requests whose future the caller cancelled while they waited are dropped; a
        request admitted to a launch is running and can no longer be cancelled
        (Future.set_running_or_notify_cancel)."""
        self._pending = [en for en in self._pending if not en.fut.cancelled()]

    def _admit(self):
        self._drop_cancelled()
        while self._pending and self._free_streams:
            head = self._pending[0]
            if self._used + head.req.footprint() > self.budget:
                return  # in arrival order: wait for memory to free up
            group = [head]
            if isinstance(head.req, BpmRequest) and head.req.mean_mode != "simple":
                k = head.req.key()
                fp = head.req.footprint()
                for en in self._pending[1:]:
                    if len(group) >= self.max_batch:
                        break
                    if isinstance(en.req, BpmRequest) and en.req.key() == k and \
                            self._used + fp + en.req.footprint() <= self.budget:
                        group.append(en)
                        fp += en.req.footprint()
            for en in group:
                self._pending.remove(en)
            # claim the futures; one cancelled since _drop_cancelled leaves the group
            group = [en for en in group if en.fut.set_running_or_notify_cancel()]
            if group:
                self._launch(group)

    def _launch(self, group):
        stream = self._free_streams.pop()
        fp = sum(en.req.footprint() for en in group)
        la = _Launch(group, stream, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True), fp)
        try:
            with torch.cuda.stream(stream):
                la.start.record(stream)
                if isinstance(group[0].req, BpmRequest):
                    la.results = self._run_bpm([en.req for en in group], la, stream)
                else:
                    r = group[0].req
                    u, ex, ey, ez = _debye(r.shape, r.units, r.lam, r.NA, r.n0, r.n_integration_steps, True,
                                           r.return_field)
                    la.results = [(u, ex, ey, ez) if r.return_field else u]
                la.done.record(stream)
        except Exception as e:
            # a request the library rejects (bad shape, arguments) fails alone
            self._free_streams.append(stream)
            for en in group:
                en.fut.set_exception(e)
            return
        self._used += fp
        self.peak_used = max(self.peak_used, self._used)
        self._inflight.append(la)
        self.launches += 1
        self.merged_launches += len(group) > 1
        self.max_inflight_seen = max(self.max_inflight_seen, len(self._inflight))

    def _run_bpm(self, reqs, la, stream):
        r0 = reqs[0]
        Nx, Ny, Nz = (int(s) for s in r0.size)
        B = len(reqs)
        dev = self.device
        plan = get_plan(r0.size, r0.units, r0.lam, r0.n0, r0.absorbing_width, r0.mean_mode, N.PROP_FUNCTIONAL)
        u0 = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev)
        for i, r in enumerate(reqs):
            if r.u0 is None:
                u0[i].fill_(1.)
            else:
                u0[i].copy_(torch.as_tensor(r.u0).to(torch.complex64), non_blocking=True)
        kind, tdt = _dn_kind(r0.dn, False)
        dn, dn_stride, mask = None, 0, None
        if kind != N.DN_NONE:
            vols = [r.dn for r in reqs]
            if all(_device_volume(v, tdt, (Nz, Ny, Nx), dev) for v in vols) and \
                    all(v.data_ptr() == vols[0].data_ptr() for v in vols):
                # every field reads the same resident volume: march it in place, no copy; its
                # phase masks are computed once where that pays (several fields, large grids)
                dn = vols[0]
                if mask_pays(B, Nx, Ny):
                    mask = precompute_mask(plan, dn, kind)
            else:
                dn = torch.empty((B, Nz, Ny, Nx), dtype=tdt, device=dev)
                for i, r in enumerate(reqs):
                    dn[i].copy_(torch.as_tensor(r.dn).to(tdt), non_blocking=True)
                dn_stride = Nz * Ny * Nx
        ok = (N.OUT_FIELD if r0.return_field else N.OUT_INTENSITY) if r0.return_full else N.OUT_NONE
        out = None
        if ok == N.OUT_FIELD:
            out = torch.empty((B, Nz, Ny, Nx), dtype=torch.complex64, device=dev)
        elif ok == N.OUT_INTENSITY:
            out = torch.empty((B, Nz, Ny, Nx), dtype=torch.float32, device=dev)
        last = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev)
        wsb = plan.workspace_bytes(B, 0)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        req = N.Request(B, _ptr(u0), _ptr(dn), kind, dn_stride, None, None,
                        _ptr(out), ok, Nz * Ny * Nx, _ptr(last), None, None, 0, 0, None, 0, _ptr(mask))
        if Nx == Ny == 128 and self._inflight:
            # 128^2 fields march fastest on the pass kernels when they have the GPU to
            # themselves (the library's choice); beside other launches they take the
            # whole-march cluster kernel, which holds 8 SMs per field for the march instead
            # of interleaving full-GPU passes with theirs (the same bits either way; GB300:
            # the serving trace's p50 2.70 -> 2.57 ms, 48 mixed requests submitted at once
            # 17.5 -> 17.1 ms)
            req.cluster = 1
        N.check(N.lib().bpm_propagate(plan.handle, ctypes.byref(req), _ptr(ws), wsb,
                                      ctypes.c_void_p(stream.cuda_stream)), "bpm_propagate")
        la.keep += [u0, dn, ws, mask]
        if r0.return_full:
            return [out[i] for i in range(B)]
        return [last[i] if r0.return_field else (last[i].abs() ** 2) for i in range(B)]


def overlapped(spans):
    """How many of the device intervals (start, end) overlap at least one other."""
    order = sorted(range(len(spans)), key=lambda i: spans[i][0])
    hit = [False] * len(spans)
    end, who = float("-inf"), -1
    for i in order:
        s, e = spans[i]
        if s < end:
            hit[i] = hit[who] = True
        if e > end:
            end, who = e, i
    return sum(hit)


def _device_volume(v, dtype, shape, dev):
    """v can be marched in place: a contiguous, 16-byte aligned CUDA tensor of the request's
    dn dtype and (Nz, Ny, Nx) shape on the server's device."""
    return (torch.is_tensor(v) and v.is_cuda and v.device == dev and v.dtype == dtype and v.is_contiguous()
            and tuple(v.shape) == tuple(shape) and v.data_ptr() % 16 == 0)


def _to_host(res):
    if isinstance(res, tuple):
        return tuple(t.cpu().numpy() for t in res)
    return res.cpu().numpy()
