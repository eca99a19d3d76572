"""Benchmark of the batched split-step BPM march on GB300.

Workload (one step = one pass of the hot path over one batch): 64 illumination plane
waves, tilts drawn area-uniformly inside NA 0.8, marched through one shared 512x512x256
dn volume (seeded Gaussian random field, correlation length 5 px, sigma 0.02, clipped to
+-0.06), dx = dz = 0.1 um, lambda 0.5 um, n0 1.33, mean_mode "weighted" (bpm_3d's
default), complex64 field, |u|^2 volume output (64 x 256 x 512 x 512 float32). Inputs are
synthetic and seeded. Metric: voxel-updates/s, one voxel-update = one (x, y) point of one
field advanced one z-step (Nx*Ny*(Nz-1) per field).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is device throughput with inputs resident in HBM (captured
CUDA graph, timed with CUDA events); `e2e` is the same through the public API
bpm_gb300.bpm_3d_batched with host buffers (pinned), H2D of u0 and dn and D2H of the
volume inside each timed step, reported for the median step (the mean and every step are
in the record); `plain` is the single-request path (one field per call).
--impl reference times the CPU restatement of the reference's algorithm (numpy/scipy,
FP32, all host cores) on a bounded sample of the same workload (median step).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = 512
NZ = 256
BATCH = 64
UNITS = (.1, .1, .1)
LAM = .5
N0 = 1.33
MODE = "weighted"
SEED = 0
# both arms (this library and the CPU restatement of the reference) report this metric on
# this workload
METRIC = "BPM voxel-updates/s, batched (64 fields, 512x512x256, |u|^2 volume)"
WORKLOAD = "batched_64x512x512x256_weighted"


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def make_u0(batch, nx, ny, seed):
    rng = np.random.default_rng(seed)
    r = .8 * np.sqrt(rng.uniform(0, 1, batch))
    th = 2 * np.pi * rng.uniform(0, 1, batch)
    k0 = 2 * np.pi / LAM
    kx, ky = k0 * r * np.cos(th), k0 * r * np.sin(th)
    x = UNITS[0] * np.arange(nx)
    y = UNITS[1] * np.arange(ny)
    return np.exp(-1j * (kx[:, None, None] * x[None, None, :] + ky[:, None, None] * y[None, :, None])
                  ).astype(np.complex64)


def make_dn_device(nx, ny, nz, seed, corr=5., sigma=.02, clip=.06):
    """Gaussian-filtered white noise, generated on the device (input synthesis only)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    w = torch.randn((nz, ny, nx), device="cuda", generator=g)
    fz = torch.fft.fftfreq(nz, device="cuda")[:, None, None]
    fy = torch.fft.fftfreq(ny, device="cuda")[None, :, None]
    fx = torch.fft.fftfreq(nx, device="cuda")[None, None, :]
    k = torch.exp(-2 * np.pi ** 2 * corr ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    f = torch.fft.ifftn(torch.fft.fftn(w) * k).real
    f = f * (sigma / f.std())
    return f.clamp_(-clip, clip).float().contiguous()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return self
        # nvidia-smi takes a few hundred ms to start: wait for its first sample so that the
        # samples cover the timed region from its start
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 5:
            time.sleep(.01)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800., "fallback"


def fp32_peak_tflops(sm_mhz):
    """FP32 CUDA-core peak: 152 SMs x 128 FMA lanes x 2 flop x clock (no measured figure
    exists for the FP32 pipe; this is the nominal formula at the sampled median clock)."""
    mhz = sm_mhz or 2070.
    return 152 * 128 * 2 * mhz * 1e6 / 1e12


def bench_ours(args, rank, world, local_rank):
    import torch
    import bpm_gb300
    from bpm_gb300 import _native as N
    from bpm_gb300.bpm3d import _ptr

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    units_per_step = BATCH * NX * NY * (NZ - 1)

    dn = make_dn_device(NX, NY, NZ, SEED)
    u0 = torch.from_numpy(make_u0(BATCH, NX, NY, SEED + 1)).to(dev)
    # fields per launch: the autotuner's choice (a short untimed probe march) unless --group
    march = bpm_gb300.BatchedMarch((NX, NY, NZ), UNITS, LAM, N0, BATCH, dn=dn, mean_mode=MODE,
                                   out_kind="intensity", group=args.group or "auto")
    march.u0.copy_(u0)
    launch = dict(march.launch)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        march.run()
    barrier()
    l0 = bpm_gb300.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            march.run()
        ev1.record(stream)
        barrier()
    launches = bpm_gb300.launch_count() - l0
    t_ms = ev0.elapsed_time(ev1) / args.steps
    # field 0 of the last timed step, its input and the dn volume, for the FP64 parity check
    check = None
    if rank == 0 and not args.no_cpu_baseline:
        check = {"u0": u0[0].cpu().numpy(), "dn": dn.cpu().numpy(), "vol": march.out[0].cpu().numpy(),
                 "last": march.last[0].cpu().numpy()}
    if world > 1:
        t = torch.tensor([t_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
    value = world * units_per_step / (t_ms * 1e-3)
    clocks = clk.summary()

    # per-kernel times of one group (CUDA events around single passes)
    req, ws, wsb = march.req, march.ws, march.ws_bytes
    L = N.lib()
    grp = march.group_used

    def time_pass(kind, z, reps=20):
        for _ in range(3):
            N.check(L.bpm_launch_pass(march.plan.handle, ctypes.byref(req), _ptr(ws), wsb, kind, z,
                                      ctypes.c_void_p(stream.cuda_stream)))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for r in range(reps):
            N.check(L.bpm_launch_pass(march.plan.handle, ctypes.byref(req), _ptr(ws), wsb, kind,
                                      z + (r % 8 if z + 9 < NZ else 0), ctypes.c_void_p(stream.cuda_stream)))
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    zmid = max(1, min(100, NZ - 2))
    t_row = time_pass(N.PASS_ROW, zmid)
    t_cr = time_pass(N.PASS_COLUMN_REDUCE, zmid)
    t_cp = time_pass(N.PASS_COLUMN_PROPAGATE, zmid)
    groups = -(-BATCH // grp)
    t_step_sum = groups * (NZ - 1) * (t_row + t_cr + t_cp)
    hbm_peak, peak_kind = peaks()
    vox = grp * NX * NY
    # algorithmic bytes of one row pass over a group: the dn slice once, the |u|^2 plane per
    # field, and the field in/out once per request spread over the nz-1 steps
    row_bytes = NX * NY * 4 + vox * 4 + vox * 16. / (NZ - 1)
    row_gbs = row_bytes / (t_row * 1e-3) / 1e9
    log2n = int(np.log2(NX))
    row_flops = vox * (2 * 5 * log2n + 12)           # inverse + forward row FFT, mask, |u|^2
    col_flops = vox * (2 * 5 * int(np.log2(NY)) + 8)  # forward + inverse column FFT, propagator
    fp32_peak = fp32_peak_tflops(clocks.get("sm_mhz"))
    traffic = profile_traffic(grp)

    # plain: one field per request through the same library, no graph
    plain = bpm_gb300.BatchedMarch((NX, NY, NZ), UNITS, LAM, N0, 1, dn=dn, mean_mode=MODE,
                                   out_kind="intensity", use_graph=False)
    plain.u0.copy_(u0[:1])
    for _ in range(2):
        plain.run()
    torch.cuda.synchronize()
    n_plain = max(2, min(8, args.steps))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(n_plain):
        plain.run()
    b.record(stream)
    torch.cuda.synchronize()
    t_plain = a.elapsed_time(b) / n_plain
    plain_value = NX * NY * (NZ - 1) / (t_plain * 1e-3)
    same = bool(torch.equal(plain.last[0], march.last[0]))
    del plain

    # e2e through the public API with pinned host buffers
    u0_h = torch.from_numpy(make_u0(BATCH, NX, NY, SEED + 1)).pin_memory()
    dn_h = torch.empty(dn.shape, dtype=torch.float32, pin_memory=True)
    dn_h.copy_(dn)
    out_h = torch.empty((BATCH, NZ, NY, NX), dtype=torch.float32, pin_memory=True)
    del march
    torch.cuda.empty_cache()
    # each step is one public-API call: H2D of u0 and dn from pinned memory, the march, and
    # the D2H of the |u|^2 volume into pinned memory (the call returns once it has landed)
    # at least 15 steps, so that the median is likely a step the shared host link did not slow
    e2e_steps = min(max(15, args.steps), 25)
    for _ in range(1):
        bpm_gb300.bpm_3d_batched((NX, NY, NZ), UNITS, lam=LAM, u0=u0_h, dn=dn_h, n0=N0, return_field=False,
                                 mean_mode=MODE, out=out_h, launch=launch)
    barrier()
    step_ms, step_gpu_ms = [], []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bpm_gb300.bpm_3d_batched((NX, NY, NZ), UNITS, lam=LAM, u0=u0_h, dn=dn_h, n0=N0, return_field=False,
                                 mean_mode=MODE, out=out_h, launch=launch)
        e1.record()
        step_ms.append((time.perf_counter() - ts) * 1e3)
        e1.synchronize()
        step_gpu_ms.append(e0.elapsed_time(e1))
    barrier()
    t_mean = (time.perf_counter() - t0) / e2e_steps
    # the median step, as the reference arm reports its median step: the host link of this
    # box is shared, and some steps run several times slower while other traffic holds it
    # (every step's time and the mean are in the record)
    t_e2e = statistics.median(step_ms) * 1e-3
    if world > 1:
        t = torch.tensor([t_e2e, t_mean], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_e2e, t_mean = float(t[0].item()), float(t[1].item())
    e2e = {"value": world * units_per_step / t_e2e, "unit": "voxel-updates/s",
           "h2d_bytes_per_step": int(u0_h.numel() * 8 + dn_h.numel() * 4),
           "d2h_bytes_per_step": int(out_h.numel() * 4), "ms_per_step": t_e2e * 1e3,
           "statistic": "median of the steps (wall clock around each public call)",
           "mean_value": world * units_per_step / t_mean, "mean_ms_per_step": t_mean * 1e3,
           "best_ms_per_step": min(step_ms),
           "steps": e2e_steps, "step_ms": [round(v, 2) for v in step_ms],
           "step_gpu_ms": [round(v, 2) for v in step_gpu_ms],
           "api": "bpm_gb300.bpm_3d_batched (pinned host u0/dn/out)"}

    res = {
        "metric": METRIC,
        "value": value, "unit": "voxel-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "nz": NZ,
                   "batch_per_gpu": BATCH, "units_um": UNITS, "lam_um": LAM, "n0": N0,
                   "mean_mode": MODE, "output": "intensity volume", "group": grp, "launch_shape": launch,
                   "dn": "gaussian random field corr 5 px sigma 0.02 clip 0.06 (shared)",
                   "u0": "64 plane waves, tilts area-uniform in NA 0.8",
                   "l2": "inputs larger than L2 (dn 256 MiB, output 16 GiB per step)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "graph": "one CUDA graph per step"},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "plain": {"value": plain_value, "unit": "voxel-updates/s", "ms_per_request": t_plain,
                  "config": "one field per request, 512x512x256, no graph", "same_result_as_batched": same},
        "batched_over_plain": value / world / plain_value,
        "kernels_ms": {"row_pass": t_row, "col_fwd_reduce": t_cr, "col_inv": t_cp,
                       "per_launch_group_fields": grp, "sum_over_step_ms": t_step_sum},
        "roofline": {"bound": "hbm", "kernel": "row_shared_kernel<512, 1>", "achieved": row_gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": row_gbs / hbm_peak,
                     "traffic": traffic, "traffic_cold": profile_traffic(grp, "dram_bytes_per_launch_cold"),
                     "traffic_note": "ncu DRAM bytes per launch: warm cache (L2 kept, as in the march) and with "
                                     "L2 flushed before the launch",
                     "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": row_bytes,
                     "fp32": {"row_pass_tflops": row_flops / (t_row * 1e-3) / 1e12,
                              "col_pass_tflops": col_flops / ((t_cr + t_cp) * 1e-3) / 1e12,
                              "peak_tflops_nominal": fp32_peak,
                              "row_frac": row_flops / (t_row * 1e-3) / 1e12 / fp32_peak,
                              "note": "FFT flops counted as 5 N log2 N per 1-D transform"}},
        "clocks": clocks,
    }
    return res, check


def psf_timing(reps=20, cpu=False):
    """Config 2's vectorial Debye-Wolf PSF: 256^3, NA 1.1, n0 1.33, lambda 0.5, x-polarised,
    512 quadrature steps (513 nodes), all four output volumes on the device (and, beside
    it, the reference's default psf() call, which returns the intensity u alone). The
    quadrature is 12 flops per octant voxel per node in FP32 terms (the tensor-core product
    executes it as three TF32 products)."""
    import torch
    import bpm_gb300
    shape, units = (256, 256, 256), (.1, .1, .1)
    args = (shape, units, .5, 1.1, 1.33, 512)

    def timed(return_field):
        for _ in range(3):
            bpm_gb300.psf(*args, return_field=return_field, device=True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            bpm_gb300.psf(*args, return_field=return_field, device=True)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    t = timed(True)
    t_u = timed(False)
    octant = 129 ** 3
    flops = octant * 513 * 12
    out_bytes = 256 ** 3 * 28
    res = {"workload": "vectorial PSF 256^3, NA 1.1, n0 1.33, 513 nodes, u+ex+ey+ez",
           "ms": t, "voxels_per_s": 256 ** 3 / (t * 1e-3),
           "quadrature_tflops": flops / (t * 1e-3) / 1e12, "quadrature_flops": flops,
           "output_gbs": out_bytes / (t * 1e-3) / 1e9,
           "u_only_ms": t_u}
    if cpu:
        res["cpu_baseline"] = psf_cpu_sample(shape, units)
    return res


def psf_cpu_sample(shape, units, rows=16):
    """The oracle's FP64 restatement of debye_wolf (numpy/scipy, factorised like the GPU
    pipeline: node x radius Bessel tables times node x plane phases) on the first `rows` of
    the octant's y rows, scaled to the full octant; output voxels/s of the full volume
    (the mirroring into it excluded)."""
    from oracle import debye_ref
    prm = debye_ref.octant_params(shape, units, .5, 1.1, 1.33)
    ny = prm["Ny"]
    sub = dict(prm, Ny=rows, y2=np.float32(float(prm["y2"]) * (rows - 1) / (ny - 1)))
    t0 = time.perf_counter()
    debye_ref.debye_octant(sub, 512)
    t = (time.perf_counter() - t0) * ny / rows
    nvox = shape[0] * shape[1] * shape[2]
    return {"value": nvox / t, "unit": "voxels/s", "cores": host_cores(), "kind": "port",
            "sample": "octant rows 0..%d of %d (%d x %d x %d octant points, 513 nodes), %.1f s scaled to %.1f s" % (
                rows - 1, ny, prm["Nx"], rows, prm["Nz"], t * rows / ny, t)}


def single_request_timing(reps=5):
    """The single-request configurations through the public API (device-resident inputs,
    and host numpy in / numpy out):
    config 1, 128x128x128, dx=dz=0.1, lambda 0.5, n0 1.33, unit plane wave, one centred
    sphere of radius 20 px and dn 0.05, weighted mean mode, |u|^2 volume + exit field;
    config 2 (BPM part), 256^3, 50 seeded spheres with radius U[3,15] px and complex dn
    (Re U[0.01,0.05], Im U[0,1e-3]), input a Gaussian focus of NA 0.4 at mid-depth
    (psf_u0), mean mode 'ignore' (the one complex dn is defined for)."""
    import torch
    import bpm_gb300
    out = {}
    n = 128
    dn1 = config1_dn(n)
    dn2 = sphere_pool(256, 256, SEED + 2).contiguous()
    u02 = bpm_gb300.psf_u0((256, 256), (.1, .1), zfoc=12.8, NA=.4, lam=.5, n0=1.33, device=True)
    cases = [("config1_128cube_plain", (n, n, n), torch.from_numpy(dn1).cuda(), None, "weighted", dn1),
             ("config2_256cube_bpm", (256, 256, 256), dn2, u02, "ignore", None)]
    for name, size, dn_d, u0_d, mode, dn_h in cases:
        def call():
            return bpm_gb300.bpm_3d(size, UNITS, lam=LAM, n0=N0, u0=u0_d, dn=dn_d, mean_mode=mode,
                                    return_field=False)
        call()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            call()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / reps
        vu = size[0] * size[1] * (size[2] - 1)
        rec = {"ms": t, "voxel_updates_per_s": vu / (t * 1e-3), "api": "bpm_gb300.bpm_3d, CUDA tensors in/out"}
        if dn_h is not None:
            # host numpy in, numpy out (the reference's own calling convention)
            bpm_gb300.bpm_3d(size, UNITS, lam=LAM, n0=N0, dn=dn_h, mean_mode=mode, return_field=False)
            t0 = time.perf_counter()
            for _ in range(reps):
                bpm_gb300.bpm_3d(size, UNITS, lam=LAM, n0=N0, dn=dn_h, mean_mode=mode, return_field=False)
            th = (time.perf_counter() - t0) / reps
            rec["e2e_numpy"] = {"ms": th * 1e3, "voxel_updates_per_s": vu / th}
        out[name] = rec
    return out


def adjoint_timing():
    """Config 4: d(loss)/d(dn) on 256x256x128 for 16 angles within NA 0.6, checkpoints
    every 16 slices: forward march + hand-written adjoint (recompute + backward)."""
    import torch
    from bpm_gb300.adjoint import propagate_exit
    size, units = (256, 256, 128), (.1, .1, .1)
    u0 = torch.from_numpy(make_u0(16, 256, 256, SEED + 7)).cuda()
    g = torch.Generator(device="cuda").manual_seed(3)
    dn = (torch.rand((128, 256, 256), device="cuda", generator=g) * .04).requires_grad_(True)
    target = torch.rand((16, 256, 256), device="cuda", generator=g)

    def one():
        dn.grad = None
        out = propagate_exit(dn, u0, size, units, LAM, N0, ckpt_every=16)
        ((out.abs() ** 2 - target) ** 2).sum().backward()
    one()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(3):
        one()
    b.record()
    torch.cuda.synchronize()
    t = a.elapsed_time(b) / 3
    vu = 16 * 256 * 256 * 127
    case = {"dn": dn.detach(), "u0": u0, "target": target, "grad": dn.grad.detach().clone(), "size": size,
            "units": units}
    return {"workload": "config 4: 256x256x128, 16 angles, ckpt 16, forward + adjoint", "ms": t,
            "forward_voxel_updates_per_s_equiv": vu / (t * 1e-3)}, case


def sphere_pool(side, nz, seed, n=50):
    """Complex random-sphere dn on the device: 50 spheres, radius U[3,15] px,
    Re dn U[0.01,0.05], Im dn U[0,1e-3] (input synthesis only)."""
    import torch
    rng = np.random.default_rng(seed)
    dn = torch.zeros((nz, side, side), dtype=torch.complex64, device="cuda")
    z = torch.arange(nz, device="cuda", dtype=torch.float32)[:, None, None]
    y = torch.arange(side, device="cuda", dtype=torch.float32)[None, :, None]
    x = torch.arange(side, device="cuda", dtype=torch.float32)[None, None, :]
    for _ in range(n):
        c = rng.uniform(0, 1, 3) * (side, side, nz)
        r = rng.uniform(3, 15)
        v = complex(rng.uniform(.01, .05), rng.uniform(0, 1e-3))
        m = ((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) <= r * r
        dn[m] = v
    return dn


def serve_trace(n=2000, rate=200., seed=0):
    """Config-5 trace: Poisson arrivals; 70% BPM requests (side in {128,256,512,1024}, Nz
    U[64,512], complex random-sphere dn, plane or Gaussian input of NA U[0.2,0.8],
    |u|^2 volume kept on the device), 30% vectorial PSFs (NA U[0.3,1.3], n0 in
    {1.33,1.52}, lambda U[0.4,0.7], cube side U{128..256} even). Complex dn is defined for
    mean_mode "ignore" only, which the BPM requests use."""
    import torch
    from bpm_gb300.serve import BpmRequest, PsfRequest, Server
    rng = np.random.default_rng(seed)
    pools = {s: sphere_pool(s, 512, seed + s) for s in (128, 256, 512, 1024)}
    t_arr = np.cumsum(rng.exponential(1. / rate, n))
    reqs = []
    for i in range(n):
        if rng.uniform() < .7:
            side = int(rng.choice([128, 256, 512, 1024]))
            nz = int(rng.integers(64, 513))
            na = rng.uniform(.2, .8)
            x = (np.arange(side) - side / 2) * .1
            if rng.uniform() < .5:
                u0 = None
            else:
                w0 = LAM / np.pi / np.arcsin(na)
                g = np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / w0 ** 2).astype(np.complex64)
                u0 = torch.from_numpy(g).cuda()
            reqs.append(BpmRequest((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=pools[side][:nz],
                                   mean_mode="ignore", return_field=False, return_full=True))
        else:
            s = 2 * int(rng.integers(64, 129))
            reqs.append(PsfRequest((s, s, s), UNITS, lam=float(rng.uniform(.4, .7)), NA=float(rng.uniform(.3, 1.3)),
                                   n0=float(rng.choice([1.33, 1.52])), n_integration_steps=200))
    torch.cuda.synchronize()
    srv = Server(max_inflight=8, max_batch=16)
    done = []
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        dt = t0 + t_arr[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        f = srv.submit(r)
        f.add_done_callback(lambda fu: done.append(fu.exception() is None))
    srv.close(wait=True)
    wall = time.perf_counter() - t0
    st = srv.stats()
    bpm_n = sum(isinstance(r, BpmRequest) for r in reqs)
    del pools, reqs
    torch.cuda.empty_cache()
    return {"requests": n, "rate_per_s": rate, "bpm_requests": bpm_n, "psf_requests": n - bpm_n,
            "ok": int(sum(done)), "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
            "wall_s": wall, "voxel_updates_per_s": st["voxel_updates"] / wall, "requests_per_s": n / wall,
            "peak_hbm_gb": st["peak_hbm_bytes"] / 1e9, "budget_gb": st["budget_bytes"] / 1e9,
            "workload": "config-5 trace, seeded Poisson arrivals, all requests latency-measured"}


def mixed_batch_timing(n=48, seed=5):
    """Config 3's second batch, the uneven-size path: n plane-wave requests over grids 128^2,
    256^2 and 512^2 with Nz in {64, 128, 256} (weighted mean mode, one shared resident dn
    volume per grid, |u|^2 volume kept on the device), submitted at once to the serving
    loop, which merges same-grid requests into batched launches and overlaps the grids on
    separate streams, and replayed as one CUDA graph (MixedBatch); against the same
    requests one after the other through bpm_3d."""
    import torch
    import bpm_gb300
    from bpm_gb300.serve import BpmRequest, Server
    rng = np.random.default_rng(seed)
    dns = {side: make_dn_device(side, side, 256, seed + side) for side in (128, 256, 512)}
    reqs = []
    for i in range(n):
        side = (128, 256, 512)[i % 3]
        nz = int(rng.choice([64, 128, 256]))
        u0 = torch.from_numpy(make_u0(1, side, side, seed + i)[0]).cuda()
        reqs.append((side, nz, u0))
    vu = sum(side * side * (nz - 1) for side, nz, _ in reqs)

    def alone(side, nz, u0):
        return bpm_gb300.bpm_3d((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dns[side][:nz],
                                return_field=False)

    for key in sorted({(side, nz) for side, nz, _ in reqs}):   # plans and kernels, untimed
        alone(key[0], key[1], next(u for sd, z, u in reqs if (sd, z) == key))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = [alone(*r) for r in reqs]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0

    def served():
        srv = Server(max_inflight=8, max_batch=16)
        t1 = time.perf_counter()
        futs = [srv.submit(BpmRequest((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dns[side][:nz],
                                      return_field=False)) for side, nz, u0 in reqs]
        out = [f.result() for f in futs]
        torch.cuda.synchronize()
        t = time.perf_counter() - t1
        srv.close(wait=True)
        return out, t, srv.stats()

    served()                                                    # warm-up of the serving path
    out, t_mix, st = served()
    same = all(bool(torch.equal(out[i], ref[i])) for i in range(0, n, 7))
    # the same requests replayed as one CUDA graph (MixedBatch): groups of a grid and Nz march
    # together, every group a parallel branch
    mb = bpm_gb300.MixedBatch([BpmRequest((side, side, nz), UNITS, lam=LAM, n0=N0, u0=u0, dn=dns[side][:nz])
                               for side, nz, u0 in reqs], tune=True)
    mb.run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(3):
        mb.run()
    b.record()
    torch.cuda.synchronize()
    t_graph = a.elapsed_time(b) / 3 * 1e-3
    same = same and all(bool(torch.equal(mb.result(i), ref[i])) for i in range(0, n, 5))
    n_groups = len(mb.groups)
    shapes = ["%dx%dx%d b%d: %s" % (g["u0"].shape[2], g["u0"].shape[1], g["out"].shape[1], g["u0"].shape[0],
                                    g["launch"]) for g in mb.groups]
    del mb
    del dns, reqs, ref, out
    torch.cuda.empty_cache()
    return {"requests": n, "grids": "128^2, 256^2, 512^2; Nz in {64, 128, 256}; weighted; shared dn per grid",
            "voxel_updates": vu, "mixed_ms": t_mix * 1e3, "mixed_voxel_updates_per_s": vu / t_mix,
            "sequential_ms": t_seq * 1e3, "sequential_voxel_updates_per_s": vu / t_seq,
            "speedup": t_seq / t_mix, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "one_graph_ms": t_graph * 1e3, "one_graph_voxel_updates_per_s": vu / t_graph,
            "one_graph_groups": n_groups, "one_graph_speedup": t_seq / t_graph,
            "one_graph_launch_shapes": shapes,
            "same_result_as_alone": same,
            "api": "bpm_gb300.serve.Server (all submitted at once) and bpm_gb300.MixedBatch (one CUDA graph) "
                   "vs bpm_gb300.bpm_3d per request"}


def config1_dn(n=128):
    """Config 1's dn: one centred sphere of radius 20 px and dn 0.05 in an n^3 grid."""
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return (.05 * (((x - n / 2) ** 2 + (y - n / 2) ** 2 + (z - n / 2) ** 2) <= 20 ** 2)).astype(np.float32)


def profile_kernels():
    """One small invocation of every kernel family not in the batched march, for per-kernel
    ncu captures: tile kernels (1024^2, 64x32), narrow single-field kernels (256^2), the
    adjoint, the scattering column pass, the mask precompute, the coated-sphere fill, the
    Debye-Wolf plane / free-point / Gaussian-pupil variants (the last through the tensor-core
    quadrature), an intensity-only PSF (the scatter assembly) and the fused weighted column
    pass."""
    import torch
    import bpm_gb300
    from bpm_gb300.adjoint import propagate_exit
    rng = np.random.default_rng(SEED)
    for (nx, ny, nz) in ((1024, 1024, 6), (64, 32, 6), (256, 256, 6)):
        dn = torch.from_numpy((.02 * rng.standard_normal((nz, ny, nx)) - 1e-4j).astype(np.complex64)).cuda()
        bpm_gb300.bpm_3d((nx, ny, nz), UNITS, lam=LAM, n0=N0, dn=dn, mean_mode="ignore", return_field=False)
    dn = torch.from_numpy((.02 * rng.standard_normal((6, 256, 256))).astype(np.float32)).cuda()
    bpm_gb300.bpm_3d((256, 256, 6), UNITS, lam=LAM, n0=N0, dn=dn, return_scattering=True)
    bpm_gb300.bpm_3d_batched((256, 128, 6), UNITS, lam=LAM, n0=N0, u0=make_u0(2, 256, 128, 1), dn=dn[:, :128].contiguous(),
                             return_field=False)
    dng = dn.clone().requires_grad_(True)
    # 10 fields: two row blocks per row in the summed-gradient adjoint, so the partial sum runs too
    out = propagate_exit(dng, torch.from_numpy(make_u0(10, 256, 256, 2)).cuda(), (256, 256, 6), UNITS, LAM, N0,
                         ckpt_every=2)
    (out.abs() ** 2).sum().backward()
    bpm_gb300.bpm_3d_spheres((256, 256, 64), UNITS, points=[[12.8, 12.8, 3.2], [6.4, 19.2, 2.]], dn_outer=.05,
                             rad_outer=2.)
    bpm_gb300.focus_field_debye_plane((256, 256), (.1, .1), z=1., lam=LAM, NA=.8)
    pts = np.linspace(-2, 2, 4096).astype(np.float32)
    bpm_gb300.focus_field_debye_at(pts, pts[::-1].copy(), .5 * pts, LAM, 1.1, n0=N0)
    bpm_gb300.focus_field_debye_gauss((128, 128, 128), (.1, .1, .1), LAM, [0, .9])
    # the intensity alone: the scatter form of the assembly
    bpm_gb300.psf((128, 128, 128), (.1, .1, .1), LAM, 1.1, N0, 512)
    # the weighted column passes fused into one cluster launch per step (opt-in launch shape)
    dnw = torch.from_numpy((.02 * rng.standard_normal((6, 256, 256))).astype(np.float32)).cuda()
    bpm_gb300.bpm_3d_batched((256, 256, 6), UNITS, lam=LAM, n0=N0, u0=make_u0(4, 256, 256, 3), dn=dnw,
                             return_field=False, launch={"col_fuse": 1})
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": True, "case": "kernels", "launches": bpm_gb300.launch_count()}))


def profile_run(args):
    """The device march alone (same buffers as the timed region), for ncu captures;
    --profile-case config1: one 128^3 weighted request through bpm_3d per step instead."""
    import torch
    import bpm_gb300
    torch.cuda.set_device(0)
    if args.profile_case == "kernels":
        profile_kernels()
        return
    if args.profile_case == "config1":
        dn1 = torch.from_numpy(config1_dn()).cuda()
        for _ in range(args.warmup + args.steps):
            u = bpm_gb300.bpm_3d((128, 128, 128), UNITS, lam=LAM, n0=N0, dn=dn1, mean_mode="weighted",
                                 return_field=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": True, "case": "config1", "sum": float(u.sum()),
                          "launches": bpm_gb300.launch_count()}))
        return
    dn = make_dn_device(NX, NY, NZ, SEED)
    march = bpm_gb300.BatchedMarch((NX, NY, NZ), UNITS, LAM, N0, BATCH, dn=dn, mean_mode=MODE,
                                   out_kind="intensity", group=args.group)
    march.u0.copy_(torch.from_numpy(make_u0(BATCH, NX, NY, SEED + 1)).cuda())
    for _ in range(args.warmup + args.steps):
        march.run()
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": True, "batch": BATCH, "nz": NZ, "launches": bpm_gb300.launch_count()}))



def profile_traffic(fields, key="dram_bytes_per_launch"):
    """DRAM bytes of one row-pass launch over `fields` fields: the committed ncu capture's
    per-field figure (dram__bytes_read.sum + dram__bytes_write.sum, captured on a smaller
    batch of the same 512x512 kernel; `key` dram_bytes_per_launch: warm cache, as in the
    timed march; dram_bytes_per_launch_cold: L2 flushed before the launch) scaled by the
    fields the bench's launch processes."""
    p = os.path.join(ROOT, "profiles", "row_pass_512_traffic.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d[key]) / float(d["fields_per_launch"]) * fields
        except (KeyError, ValueError, ZeroDivisionError, TypeError):
            return None
    return None


def cpu_sample(fields=1, steps=48):
    """The CPU restatement of the reference's march (oracle, FP32, scipy.fft with all host
    cores) on a bounded sample of the workload: `fields` fields x `steps` z-steps."""
    from oracle import bpm_ref
    rng = np.random.default_rng(SEED)
    dn = (np.clip(rng.normal(0, .02, (steps + 1, NY, NX)), -.06, .06)).astype(np.float32)
    u0 = make_u0(fields, NX, NY, SEED + 1)
    t0 = time.perf_counter()
    for f in range(fields):
        bpm_ref.bpm_3d((NX, NY, steps + 1), UNITS, lam=LAM, n0=N0, u0=u0[f], dn=dn, mean_mode=MODE,
                       return_field=False, precision="fp32", workers=host_cores())
    t = time.perf_counter() - t0
    units = fields * NX * NY * steps
    return units / t, t, "%d field(s) x %dx%d x %d z-steps, mean_mode=%s, |u|^2 volume" % (
        fields, NX, NY, steps, MODE)


def parity_vs_fp64(check):
    """Relative L2 of the timed march's field 0 (|u|^2 volume over all 256 planes, and the
    exit field) against the oracle's FP64 march of the same input through the same dn."""
    from oracle import bpm_ref
    t0 = time.perf_counter()
    vol, last = bpm_ref._bpm_3d((NX, NY, NZ), UNITS, lam=LAM, n0=N0, u0=check["u0"], dn=check["dn"],
                                mean_mode=MODE, return_field=False, return_last_plane=True, precision="fp64",
                                workers=host_cores())
    num = den = 0.
    for z in range(NZ):
        d = check["vol"][z].astype(np.float64) - vol[z]
        num += float(np.vdot(d, d).real)
        den += float(np.vdot(vol[z], vol[z]).real)
    dl = check["last"].astype(np.complex128) - last
    return {"field": 0, "rel_l2_intensity_volume": (num / den) ** .5,
            "rel_l2_exit_field": float(np.linalg.norm(dl) / np.linalg.norm(last)),
            "against": "oracle FP64 march (numpy/scipy) of the same u0 and dn, all %d planes" % NZ,
            "oracle_s": time.perf_counter() - t0}


def adjoint_grad_check(case):
    """Relative L2 of the timed adjoint's d(loss)/d(dn) against FP64 torch autograd through
    the oracle's restatement of the ignore-mode march (same dn, illuminations, target)."""
    import torch
    from oracle import torch_ref
    dn64 = case["dn"].double().requires_grad_(True)
    ref = torch_ref.march_exit_fp64(torch, dn64, case["u0"].to(torch.complex128), case["size"], case["units"],
                                    LAM, N0)
    ((ref.abs() ** 2 - case["target"].double()) ** 2).sum().backward()
    g, r = case["grad"].double(), dn64.grad
    e = float(torch.linalg.vector_norm(g - r) / torch.linalg.vector_norm(r))
    del dn64, ref
    torch.cuda.empty_cache()
    return e


def bench_reference(args, rank):
    if rank != 0:
        return None
    vals = []
    for _ in range(args.warmup):
        cpu_sample(1, 8)
    for _ in range(args.steps):
        v, t, sample = cpu_sample(1, 64)
        vals.append((v, t))
    v = statistics.median(x[0] for x in vals)
    t_ms = statistics.median(x[1] for x in vals) * 1e3
    cores = host_cores()
    return {"impl": "reference",
            "metric": METRIC,
            "value": v, "unit": "voxel-updates/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": v, "unit": "voxel-updates/s", "cores": cores, "kind": "port",
                             "sample": sample + " per step (reference algorithm restated in numpy/scipy "
                                                "FP32; the reference's OpenCL path cannot run here)"},
            "e2e": {"value": v, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def launch_ranks(n, argv):
    """Re-run this script as n ranks on this node (torch.distributed.run, one process per
    GPU, rendezvous on 127.0.0.1); rank 0 prints the JSON line. Returns the launcher's exit
    status."""
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=%d" % n,
           "--master-addr=127.0.0.1", "--master-port=%d" % port, os.path.abspath(__file__), *argv]
    return subprocess.call(cmd)


def rank_census():
    """Number of ranks in the initialised process group that reach this point (a sum of
    ones over every rank)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.distributed.get_backend() == "nccl" \
        else torch.device("cpu")
    t = torch.ones(1, device=dev)
    torch.distributed.all_reduce(t)
    return int(t.item())


def print_rank_census(world, rank):
    """--check-launch: every rank joins a CPU (gloo) process group and rank 0 prints how
    many ranks reached the benchmark's entry, with no GPU work."""
    import torch
    n = 1
    if world > 1:
        torch.distributed.init_process_group("gloo")
        n = rank_census()
    if rank == 0:
        print(json.dumps({"check_launch": True, "ranks": n, "world_size": world}))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--group", type=int, default=0, help="fields per pass (0 = library default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving trace")
    ap.add_argument("--batch", type=int, default=BATCH, help="fields per GPU (smaller for profiling)")
    ap.add_argument("--nz", type=int, default=NZ, help="z planes (smaller for profiling)")
    ap.add_argument("--profile", action="store_true",
                    help="only the device march (warm-up + steps), for ncu launch lists")
    ap.add_argument("--profile-case", default="batched", choices=["batched", "config1", "kernels"],
                    help="with --profile: the batched march, one 128^3 weighted request per step, or one "
                         "small call of every other kernel family")
    ap.add_argument("--check-launch", action="store_true",
                    help="only start the ranks and report how many joined (no GPU work)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    globals()["BATCH"] = args.batch
    globals()["NZ"] = args.nz
    if args.profile:
        profile_run(args)
        return

    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # --gpus N without an external launcher: start the N ranks here
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))

    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local_rank = env_int("LOCAL_RANK", 0)

    if args.check_launch:
        print_rank_census(world, rank)
        return

    if args.impl == "reference":
        res = bench_reference(args, rank)
        if res is not None:
            print(json.dumps(res))
        return

    if world > 1:
        import torch
        if torch.cuda.device_count() < world:
            raise SystemExit("bench.py: %d ranks but %d visible GPUs" % (world, torch.cuda.device_count()))
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
        # n_gpus counts the ranks that joined the job, not the requested number
        world = rank_census()
    res, check = bench_ours(args, rank, world, local_rank)
    if rank == 0:
        if not args.no_serve:
            res["serve"] = serve_trace()
        res["psf"] = psf_timing(cpu=not args.no_cpu_baseline)
        res["mixed_batch"] = mixed_batch_timing()
        res["single_requests"] = single_request_timing()
        res["adjoint"], adj_case = adjoint_timing()
        if not args.no_cpu_baseline:
            # the oracle as the checker: the timed results against FP64, and the CPU baseline
            res["adjoint"]["grad_rel_l2_vs_fp64"] = adjoint_grad_check(adj_case)
            del adj_case
            res["parity"] = parity_vs_fp64(check)
            res["rel_l2_vs_fp64"] = res["parity"]["rel_l2_intensity_volume"]
            del check
            v, t, sample = cpu_sample(4, NZ - 1)
            res["cpu_baseline"] = {"value": v, "unit": "voxel-updates/s", "cores": host_cores(), "kind": "port",
                                   "sample": sample + ", %.1f s" % t}
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
