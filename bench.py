#!/usr/bin/env python
"""FWI gradient benchmark (configuration c3) on GB300.

One step = one FWI gradient evaluation as the reference's FWI scripts do it
(scripts/fwi.py:70-113): nonlinear modelling of the current model (WEM
forward), the data residual, and the gradient as the Born adjoint of the
residual at the current model (BornFull::adjoint, compat mode), over all
32 shots x 96 frequencies of a 768 x 300 model (SSF, N = 768).

Reported: ``value`` = depth-steps/s with inputs resident on the GPU, where a
depth-step is one (shot, frequency) row advanced one depth in one one-way or
linearised pass of the reference's call sequence (2 passes for WEM forward,
10 for the Born adjoint), so the figure is comparable with the reference's
own work; ``s_per_iter`` = seconds per gradient; ``e2e`` = the same through
the C ABI with host buffers (copies inside the timed region); ``roofline``
for the dominant kernel from CUDA events on its launch stream, against HBM
bandwidth and (``roofline.issue``) against the SM instruction issue rate
that bounds it; ``cpu_baseline`` = the CPU restatement on the host cores on
a bounded sample.  ``--workload c1|c2`` prints timings of the other
configurations instead (not the benchmark line).

``--impl reference`` times the CPU restatement of the reference on the same
configuration and metric.  The reference's own sources compile only where
its checkout is (oracle/ref, against stand-ins for FFTW, TBB, Boost and the
SEP libraries: the pin of the restatement, not a build to time), so the arm
runs the restatement, which is held to that build's outputs.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "wem-fwi_gb300"))
sys.path.insert(0, ROOT)

METRIC = "FWI gradient s/iter & depth-steps/s, batched+adjoint vs plain GPU at L2<=1e-4"
PASSES_WEM = 2       # Down + Up (wem_prop.cpp:57,68)
PASSES_BORN_FWD = 9   # born_prop.cpp:75-113
PASSES_BORN_ADJ = 10  # born_prop.cpp:190-215: 1 down, 3 Up^H, 2 Down^H, 2 LinDown^H, 1 up, 1 LinUp^H


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is running: wait for
            # its first line and keep only what follows
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(small=False, small_shots=8):
    from wemgpu import synthetic as S
    cfg = S.c3()
    if small:  # a reduced case of the same kernels for profiling captures
        cfg["par"] = dict(cfg["par"], ns=small_shots, dsx=cfg["par"]["dsx"] * 32 // small_shots, fmax=6.0)
    return cfg


# DRAM bytes (read + write) per (row, depth) of the gradient's passes, from
# one ncu capture of the reduced case (16 shots x 21 frequencies, nz 300,
# N 768; profiles/fwi_gradient_passes_e24_c3_small16.md; kernels of commit
# 29b9584): the traffic of a launch scales with the rows it carries, so a
# full launch is this figure x rows x depths.  The Born adjoint pass of the
# gradient is kw_adj_down + kw_born_adj2 (its up sweep), summed.
TRAFFIC_PER_ROW_DEPTH = {
    "k_born_adj": ((699063808 + 1258508288) + (1939322112 + 74323200)) / (336 * 300),
    "k_wem": (735724288 + 1240831488) / (336 * 300),
}
# warp instructions per (row, depth) of the same passes (smsp__inst_executed
# of the same capture): the pass kernels are bound by instruction issue, so
# the line also reports the issue rate they reach against one warp
# instruction per SM sub-partition per cycle
INST_PER_ROW_DEPTH = {
    "k_born_adj": (254521722 + 897649314) / (336 * 300),
    "k_wem": 427428918 / (336 * 300),
}


def config_of(p, nf, world, small):
    """The workload block of both arms' JSON lines."""
    return {"workload": "c3 FWI gradient: WEM fwd + residual + Born adjoint (compat)",
            "nx": p.nx, "nz": p.nz, "dx": p.dx, "shots": p.ns * world, "freqs": nf, "fft_n": p.nx + 2 * p.pad,
            "prop": "ssf", "depth_steps_per_iter": row_steps(p, nf) * world,
            "l2": "inputs larger than L2 (stored wavefields ~17 GB per Born adjoint pass)",
            "small": bool(small)}


def rank_workload(cfg, rank, world):
    """Rank's block of the weak-scaling survey: the workload's shots shifted
    by rank / world of the shot interval (wemgpu.shard.interleave_par)."""
    from wemgpu.shard import interleave_par
    if world == 1:
        return cfg
    return dict(cfg, par=interleave_par(cfg["par"], world, rank))


def reduce_gradients(g0, g1, world):
    """The one exchange of a multi-rank gradient: both model gradients summed
    over ranks (NCCL on the GPU arm; any backend the tensors' device has)."""
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(g0, op=dist.ReduceOp.SUM)
        dist.all_reduce(g1, op=dist.ReduceOp.SUM)


def relaunch(args):
    """`--gpus N` outside torchrun: run the same command as N ranks under
    torch.distributed.run on this node and return its exit status."""
    import socket
    sock = socket.socket()
    sock.bind(("127.0.0.1", 0))
    port = sock.getsockname()[1]
    sock.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def row_steps(p, nfreq):
    return (PASSES_WEM + PASSES_BORN_ADJ) * p.ns * nfreq * (p.nz - 1)


def algorithmic_bytes(kernel, p, nfreq, G):
    """HBM bytes a launch must move: each row's wavefield read and written once per
    depth, plus the per-(frequency, depth) phase and split-step tables."""
    nxg = p.nx + 2 * p.pad
    N = nxg + 2 * p.tap
    rows = p.ns * nfreq
    groups = nfreq * ((p.ns + G - 1) // G)
    tables = nfreq * p.nz * (N * p.nref + nxg) * 8  # phase + split-step rows per (f, z)
    if kernel == "k_wem":
        return rows * p.nz * 16 * nxg + 2 * tables
    if kernel == "k_born_adj":
        # stored bg and T (and, with tap 0, the as-coded scatter adjoint and one
        # Taylor term, the filtered spectra of T) written once and read once
        fields = 3 if (p.tap == 0 and p.adjoint_mode == 0 and p.ntaylor == 1 and p.nref == 1) else 2
        return rows * p.nz * 16 * fields * nxg + groups * p.nz * 16 * nxg + 4 * tables
    if kernel == "k_born_fwd":
        return rows * p.nz * 32 * nxg + 2 * tables
    return None


def run_gpu(args, rank, world):
    import torch
    import wemgpu
    from wemgpu import _lib, synthetic as S
    from wemgpu.core import BornOp, FwiOp, WemOp

    wemgpu.build()
    lib = _lib.load()
    dev = torch.device(f"cuda:{int(os.environ.get('LOCAL_RANK', 0))}")
    torch.cuda.set_device(dev)
    # weak scaling: every rank runs a block of the workload's size, its own
    # shots of one survey of world x 32 shots
    cfg = rank_workload(workload(args.small, args.small_shots), rank, world)
    p = S.params_of(cfg)
    nf = WemOp(p, cfg["wavelet"]).nfreq()
    wav = cfg["wavelet"]
    s_true = torch.from_numpy(cfg["slow_true"]).to(dev)
    s0 = torch.from_numpy(cfg["slow"]).to(dev)
    rho = torch.from_numpy(cfg["rho"]).to(dev)
    wem = WemOp(p, wav)
    born = BornOp(p, wav, s0, rho)
    d_obs = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    wem.forward(s_true, rho, d_obs)
    g0, g1 = torch.zeros_like(s0), torch.zeros_like(s0)
    # one gradient step: modelling, residual and loss, Born adjoint of the
    # residual (the library's fused call, inputs resident on the device)
    fwi = FwiOp(p, wav)

    def step():
        fwi.gradient(s0, rho, d_obs, g0, g1)
        reduce_gradients(g0, g1, world)
        return g0

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    lib.wem_stats_reset()
    lib.wem_stats_enable(1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_launch0 = _lib.launch_count()
    with Clocks(dev.index) as clk:
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(args.steps):
            step()
        ev1.record()
        torch.cuda.synchronize()
    gpu_launches = _lib.launch_count() - n_launch0
    lib.wem_stats_enable(0)
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    s_per_iter = ms / 1e3 / args.steps
    steps_per_iter = row_steps(p, nf) * world
    value = steps_per_iter / s_per_iter

    # dominant kernel and its roofline
    kstats = {k: _lib.kernel_stats(k) for k in ("k_wem", "k_born_adj", "k_born_fwd")}
    kstats = {k: v for k, v in kstats.items() if v[1] > 0}
    top = max(kstats, key=lambda k: kstats[k][0])
    top_ms, top_n = kstats[top]
    G = min(p.ns, 8)
    algo = algorithmic_bytes(top, p, nf, G)
    peak, peak_src = peaks()
    achieved = algo / (top_ms / top_n / 1e3) / 1e9
    traffic = None
    if top in TRAFFIC_PER_ROW_DEPTH:
        traffic = TRAFFIC_PER_ROW_DEPTH[top] * p.ns * nf * p.nz
    clocks = clk.summary()
    issue = None
    if top in INST_PER_ROW_DEPTH:
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
        if mhz:
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            inst = INST_PER_ROW_DEPTH[top] * p.ns * nf * p.nz
            rate = inst / (top_ms / top_n / 1e3)
            peak_issue = sms * 4 * mhz * 1e6
            issue = {"kernel": top, "warp_inst_per_launch": inst, "achieved_ginst_s": rate / 1e9,
                     "peak_ginst_s": peak_issue / 1e9, "frac": rate / peak_issue,
                     "source": "instructions per row-depth from the ncu capture, sm clock sampled live"}

    # end to end through the public FWI call (wemgpu.autograd.FwiObjective):
    # each step copies the model in from pinned host memory and the loss and
    # gradient out; the observed data live on the device (uploaded once)
    from wemgpu.autograd import FwiObjective
    s0_pin = torch.from_numpy(cfg["slow"]).pin_memory()
    rho_pin = torch.from_numpy(cfg["rho"]).pin_memory()
    obj = FwiObjective(p, wav, d_obs)
    obj(s0_pin.numpy(), rho_pin.numpy())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        obj(s0_pin.numpy(), rho_pin.numpy())
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d, d2h = obj.h2d_bytes, obj.d2h_bytes

    # the reference's call pattern with host arrays (scripts/fwi.py: WEM
    # forward into a host array, residual on the host, Born adjoint of it):
    # synthetic data out and residual in cross the host link every step
    s0h, rhoh = cfg["slow"], cfg["rho"]
    d_obs_h = d_obs.cpu().numpy()
    d_syn_h = np.zeros_like(d_obs_h)
    g0h, g1h = np.zeros_like(s0h), np.zeros_like(s0h)

    def step_host():
        wem.forward(s0h, rhoh, d_syn_h)
        res = d_syn_h - d_obs_h
        born.set_background(s0h, rhoh)
        born.adjoint(g0h, g1h, res)

    step_host()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    torch.cuda.synchronize()
    ops_s = (time.perf_counter() - t0) / args.steps
    ops_h2d = 2 * s0h.nbytes + 2 * rhoh.nbytes + d_obs_h.nbytes
    ops_d2h = d_syn_h.nbytes + g0h.nbytes + g1h.nbytes

    # plain form: every (shot, frequency) row in its own launch, timed on a
    # sample of shots and scaled to the whole job
    plain = None
    if not args.no_plain and rank == 0:
        cfgp = dict(cfg)
        ns_p = 1
        cfgp["par"] = dict(cfg["par"], ns=ns_p)
        pp = S.params_of(cfgp)
        wp = WemOp(pp, wav)
        bp = BornOp(pp, wav, s0, rho)
        dp = torch.zeros((pp.ns, pp.nr, pp.nt), dtype=torch.float32, device=dev)
        a0, a1 = torch.zeros_like(s0), torch.zeros_like(s0)
        lib.wem_set_plain(1)
        try:
            wp.forward(s0, rho, dp)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            wp.forward(s0, rho, dp)
            bp.set_background(s0, rho)
            bp.adjoint(a0, a1, dp)
            e1.record()
            torch.cuda.synchronize()
            plain_s = e0.elapsed_time(e1) / 1e3 * p.ns / ns_p
        finally:
            lib.wem_set_plain(0)
        plain = {"s_per_iter": plain_s, "sample": f"{ns_p} shots x {nf} freqs, scaled to {p.ns} shots",
                 "batched_speedup": plain_s / s_per_iter}

    cpu, cpu_fft = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample(cfg, seconds=args.cpu_seconds)
        cpu_fft = cpu_fft_bound(p, nf)
    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_sample(cfg, p, wem, s0, rho, d_obs)

    line = {
        "metric": METRIC, "value": value, "unit": "depth-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded c3 model, see wemgpu/synthetic.py)",
        "config": config_of(p, nf, world, args.small),
        "s_per_iter": s_per_iter,
        "e2e": {"value": steps_per_iter / e2e_s, "unit": "depth-steps/s", "s_per_iter": e2e_s,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "api": "wemgpu.autograd.FwiObjective, pinned host model in, loss + gradient out"},
        "e2e_operator_api": {"value": steps_per_iter / ops_s, "unit": "depth-steps/s", "s_per_iter": ops_s,
                             "h2d_bytes_per_step": int(ops_h2d), "d2h_bytes_per_step": int(ops_d2h),
                             "api": "WemOp/BornOp with numpy host arrays, residual on the host"},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                     "algorithmic_bytes": algo, "ms_per_launch": top_ms / top_n, "traffic": traffic,
                     "issue": issue},
        "kernels": {k: {"ms": v[0] / args.steps, "launches": v[1] // args.steps} for k, v in kstats.items()},
        "gpu_launches": gpu_launches,
        "plain_gpu": plain,
        "cpu_baseline": cpu,
        "cpu_fft_bound": cpu_fft,
        "parity": parity,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def parity_sample(cfg, p, wem, s0, rho, d_obs):
    """rel-L2 of the benchmarked kernels' results against the oracle (fp32
    restatement and fp64 twin), outside the timed region: the first two
    shots of the full batch's modelling (the timed step's WEM pass), and the
    FWI gradient of a two-shot block (the timed call on 2 of the 32 shots;
    the tests hold the full call to the sum of its blocks)."""
    import torch
    from oracle import oracle as O
    from wemgpu import synthetic as S
    from wemgpu.core import FwiOp
    from wemgpu.params import WEM_DATA_TIME
    O.build()
    t0 = time.perf_counter()
    wav = cfg["wavelet"]
    d = torch.zeros_like(d_obs)
    wem.forward(s0, rho, d)
    cfg2 = dict(cfg, par=dict(cfg["par"], ns=2))
    p2 = S.params_of(cfg2)
    obs2 = d_obs[:2].contiguous()
    g0, g1 = torch.zeros_like(s0), torch.zeros_like(s0)
    FwiOp(p2, wav).gradient(s0, rho, obs2, g0, g1)
    torch.cuda.synchronize()
    d2 = d[:2].cpu().numpy()
    # the oracle's gradient of the block's own residual (a small difference
    # of two modelled data sets: each side's modelling error would be
    # amplified by |syn| / |res| were the oracle to form it itself)
    res = d2 - obs2.cpu().numpy()
    g0h, g1h = g0.cpu().numpy(), g1.cpu().numpy()

    def rel(a, b):
        a, b = np.asarray(a, np.complex128), np.asarray(b, np.complex128)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    out = {"tolerance": 1e-4}
    for prec in (32, 64):
        syn = O.wem_forward(p2, wav, cfg["slow"], cfg["rho"], kind=WEM_DATA_TIME, prec=prec)
        o0, o1 = O.born_adjoint(p2, wav, cfg["slow"], cfg["rho"], res, kind=WEM_DATA_TIME, prec=prec)
        out[f"wem_vs_fp{prec}"] = rel(d2, syn)
        out[f"gradient_vs_fp{prec}"] = max(rel(g0h, o0), rel(g1h, o1))
    out["sample"] = ("shots 0-1 of the full-batch modelling; fwi_gradient of a 2-shot block against the "
                     f"oracle's Born adjoint of its residual (oracle {time.perf_counter() - t0:.0f} s on the host)")
    return out


def cpu_fft_bound(p, nfreq, seconds=5.0):
    """The bare split-step depth step of the rows of one shot (forward FFT,
    phase-shift multiply, inverse FFT, split-step multiply; no injection,
    recording, tables or imaging) with torch.fft (pocketfft, vectorised) on
    every host thread: what a library FFT gives on the host cores for the
    transform pair that every depth-step of the reference's SSF passes
    takes.  It is a second CPU figure beside the oracle's, not a proven
    bound: a code tuned for these cores (FFTW with ISPC, one row per thread)
    may run faster."""
    import torch
    nthreads = os.cpu_count() or 1
    torch.set_num_threads(nthreads)
    n = p.nx + 2 * (p.pad + p.tap)
    rows = nfreq  # one shot's rows
    g = torch.Generator().manual_seed(0)
    x = torch.randn(rows, n, dtype=torch.complex64, generator=g)
    ph = torch.exp(1j * torch.rand(rows, n, generator=g)).to(torch.complex64)
    fac = torch.exp(1j * torch.rand(rows, n, generator=g)).to(torch.complex64) / n
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(10):
            x = torch.fft.ifft(torch.fft.fft(x) * ph, norm="forward") * fac
        steps += 10
    dt = time.perf_counter() - t0
    return {"value": rows * steps / dt, "unit": "depth-steps/s", "cores": nthreads, "kind": "fft-bound",
            "sample": f"{rows} rows of N = {n}, {steps} bare split-step depth steps with torch.fft, {dt:.1f} s"}


def cpu_sample(cfg, seconds=15.0, nthreads=0, nshots=0):
    """The CPU restatement (oracle, fp32) on a bounded sample of the same
    workload: the first shots (``nshots``, or as many as take about
    ``seconds``), every frequency, all depths."""
    from oracle import oracle as O
    from wemgpu import synthetic as S
    O.build()
    nthreads = nthreads or os.cpu_count() or 1
    # grow the sample (shots, each with the workload's full frequency axis and
    # all depths) until it takes about `seconds`
    p_full = S.params_of(cfg)
    nsk = nshots or 1
    while True:
        par = dict(cfg["par"], ns=nsk)
        c = dict(cfg, par=par)
        p = S.params_of(c)
        nf = O.count_freqs(p)[0]
        t0 = time.perf_counter()
        syn = O.wem_forward(p, cfg["wavelet"], cfg["slow"], cfg["rho"], kind=0, prec=32, nthreads=nthreads)
        O.born_adjoint(p, cfg["wavelet"], cfg["slow"], cfg["rho"], syn, kind=0, prec=32, nthreads=nthreads,
                       fchunks=max(1, nthreads))
        dt = time.perf_counter() - t0
        if nshots or dt > 0.5 * seconds or nsk >= p_full.ns:
            break
        nsk = min(p_full.ns, max(nsk + 1, int(nsk * seconds / max(dt, 1e-3))))
    rate = row_steps(p, nf) / dt
    return {"value": rate, "unit": "depth-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{nsk} shots x {nf} freqs of c3 (all {p.nz} depths), WEM fwd + Born adjoint, {dt:.1f} s",
            "s_per_iter_extrapolated": row_steps(p_full, nf) / rate}


def run_reference(args, rank, world):
    """CPU restatement on the host cores, same config / metric / unit."""
    if rank != 0:
        return
    cfg = workload(args.small, args.small_shots)
    # the sample is sized once, so that all warm-up and timed steps together
    # take about two minutes (1-10 s each), then every step repeats it
    per_step = min(10.0, max(1.0, 120.0 / (args.warmup + args.steps)))
    first = cpu_sample(cfg, seconds=per_step)
    nshots = int(first["sample"].split()[0])
    res, durs = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        # the sizing run counts as the first warm-up step; every timed step
        # runs its own sample
        r = first if (i == 0 and args.warmup > 0) else cpu_sample(cfg, nshots=nshots)
        if i >= args.warmup:
            res.append(r["value"])
            durs.append(time.perf_counter() - t0)
    v = float(np.median(res))
    from oracle import oracle as O
    from wemgpu import synthetic as S
    p = S.params_of(cfg)
    nf = O.count_freqs(p)[0]
    per_iter = row_steps(p, nf) / v
    # a step is one timed sample of the workload (its duration); s_per_iter
    # is the whole gradient at the measured rate
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "depth-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median(durs)) * 1e3,
            "s_per_iter": per_iter,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded c3 model, see wemgpu/synthetic.py)",
            "config": config_of(p, nf, 1, args.small),
            "cpu_baseline": {"value": v, "unit": "depth-steps/s", "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": "depth-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_config(args):
    """The other configurations, timed for the record (not the contract
    line): c1 = WEM forward + Born adjoint (migration) of one shot; c2 = Born
    forward and Born adjoint (exact, with its dot test) of 48 shots.  GPU
    times are CUDA events around each call on resident inputs; the CPU
    restatement is timed on one shot (c1 all of it) with every host thread."""
    import torch
    import wemgpu
    from wemgpu import synthetic as S
    from wemgpu.core import BornOp, WemOp
    from oracle import oracle as O

    wemgpu.build()
    dev = torch.device("cuda:0")
    par = {"adjoint_mode": "exact"} if args.workload == "c2" else {}
    cfg = S.CONFIGS[args.workload]()
    cfg["par"] = dict(cfg["par"], **par)
    if args.small:  # a reduced case of the same kernels for profiling captures
        f0 = cfg["par"]["fmin"]
        cfg["par"] = dict(cfg["par"], ns=min(cfg["par"]["ns"], args.small_shots), fmax=f0 + 2.0)
    p = S.params_of(cfg)
    wav = cfg["wavelet"]
    s = torch.from_numpy(cfg["slow"]).to(dev)
    rho = torch.from_numpy(cfg["rho"]).to(dev)
    nf = WemOp(p, wav).nfreq()
    d = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    g0, g1 = torch.zeros_like(s), torch.zeros_like(s)
    born = BornOp(p, wav, s, rho)
    if args.workload == "c1":
        wem = WemOp(p, wav)
        ops = {"wem_forward": (lambda: wem.forward(s, rho, d), PASSES_WEM),
               "born_adjoint": (lambda: born.adjoint(g0, g1, d), PASSES_BORN_ADJ)}
    else:
        ds = torch.from_numpy(cfg["dslow"]).to(dev)
        dr = torch.from_numpy(cfg["drho"]).to(dev)
        ops = {"born_forward": (lambda: born.forward(ds, dr, d), PASSES_BORN_FWD),
               "born_adjoint": (lambda: born.adjoint(g0, g1, d), PASSES_BORN_ADJ)}
    out = {"workload": args.workload, "small": bool(args.small), "nx": p.nx, "nz": p.nz, "shots": p.ns, "freqs": nf,
           "fft_n": p.nx + 2 * (p.pad + p.tap), "prop": "pspi" if p.prop else "ssf", "nref": p.nref, "ops": {}}
    for name, (fn, passes) in ops.items():
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.steps):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / args.steps
        steps = passes * p.ns * nf * (p.nz - 1)
        out["ops"][name] = {"ms": ms, "depth_steps_per_s": steps / (ms / 1e3), "passes": passes}
    if args.workload == "c2":
        # dot test of the exact adjoint at full size (d = L n keeps both
        # inner products away from cancellation)
        rng = np.random.default_rng(5)
        cplx = lambda sc: torch.from_numpy((sc * (rng.standard_normal(s.shape) + 1j * rng.standard_normal(s.shape))).astype(np.complex64)).to(dev)
        m0, m1, n0, n1 = cplx(1e-7), cplx(1e-2), cplx(1e-7), cplx(1e-2)
        dn, lm = torch.zeros_like(d), torch.zeros_like(d)
        born.forward(n0 + 0.5 * m0, n1 + 0.5 * m1, dn)
        born.forward(m0, m1, lm)
        born.adjoint(g0, g1, dn)
        lhs = float(torch.sum(dn.double() * lm.double()))
        z = lambda a: a.to(torch.complex128)
        rhs = float((z(g0).conj() * z(m0)).sum().real + (z(g1).conj() * z(m1)).sum().real)
        out["dot_ratio"] = abs(lhs - rhs) / abs(lhs)
    if not args.no_cpu:
        O.build()
        nt = os.cpu_count() or 1
        one = dict(cfg, par=dict(cfg["par"], ns=1))
        p1 = S.params_of(one)
        t0 = time.perf_counter()
        if args.workload == "c1":
            syn = O.wem_forward(p1, wav, cfg["slow"], cfg["rho"], kind=0, nthreads=nt)
            passes = PASSES_WEM + PASSES_BORN_ADJ
        else:
            syn = O.born_forward(p1, wav, cfg["slow"], cfg["rho"], cfg["dslow"], cfg["drho"], kind=0, nthreads=nt)
            passes = PASSES_BORN_FWD + PASSES_BORN_ADJ
        O.born_adjoint(p1, wav, cfg["slow"], cfg["rho"], syn, kind=0, nthreads=nt, fchunks=nt)
        dt = time.perf_counter() - t0
        out["cpu_oracle"] = {"s_one_shot": dt, "depth_steps_per_s": passes * nf * (p.nz - 1) / dt,
                             "cores": nt, "kind": "port"}
    print(json.dumps(out), flush=True)


def run_c4(args):
    """The subsurface-offset extended Born (c4: nh = 21 lags, 64 shots of
    uneven aperture), timed for the record: forward (reflectivity -> time
    traces) and adjoint (traces -> lag image), CUDA events around each call
    on resident inputs, with the per-kernel times, a full-size dot test, and
    the first shot against the oracle (fp32 and fp64, the oracle also timed
    on it with every host thread)."""
    import torch
    import wemgpu
    from wemgpu import _lib, synthetic as S
    from wemgpu.core import BornOffsetOp
    from oracle import oracle as O

    wemgpu.build()
    dev = torch.device("cuda:0")
    cfg = S.c4()
    if args.small:  # a reduced case of the same kernels for profiling captures
        ns = min(cfg["par"]["ns"], args.small_shots)
        cfg["par"] = dict(cfg["par"], ns=ns, dsx=cfg["par"]["dsx"], fmax=cfg["par"]["fmin"] + 2.0)
        cfg["apertures"] = cfg["apertures"][:ns]
    p = S.params_of(cfg)
    wav, nh, ap = cfg["wavelet"], cfg["nh"], cfg["apertures"]
    op = BornOffsetOp(p, wav, cfg["slow"], nh, ap)
    nf = op.nfreq()
    r = torch.from_numpy(cfg["refl"]).to(dev)
    d = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    img = torch.zeros_like(r)
    n_rows, _ = op.rows()
    rows = p.ns * nf
    lib = _lib.load()
    out = {"workload": "c4 extended Born (subsurface offset): forward and adjoint", "small": bool(args.small),
           "nx": p.nx, "nz": p.nz, "shots": p.ns, "freqs": nf, "nh": nh, "aperture_cells": [int(ap[:, 1].min()),
           int(ap[:, 1].max())], "row_lengths": {str(n): int((n_rows == n).sum()) for n in sorted(set(n_rows))},
           "prop": "ssf", "ops": {}}
    for name, fn in (("forward", lambda: op.forward(r, d)), ("adjoint", lambda: op.adjoint(img, d))):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        lib.wem_stats_reset()
        lib.wem_stats_enable(1)
        fn()
        lib.wem_stats_enable(0)
        kern = {k: round(_lib.kernel_stats(k)[0], 3) for k in ("k_off_down", "k_off_up", "k_off_upadj",
                                                                "k_off_source", "k_off_image")}
        kern = {k: v for k, v in kern.items() if v > 0}
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.steps):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / args.steps
        steps = 2 * rows * (p.nz - 1)  # two sweeps per row
        out["ops"][name] = {"ms": ms, "depth_steps_per_s": steps / (ms / 1e3), "sweeps": 2, "kernels_ms": kern}
    # algorithmic bytes of the lag kernels: each reads two fields and writes
    # at most one, 8 bytes a point of every row's aperture
    pts = float(sum(nf * p.nz * (int(w) + 2 * p.pad) for w in ap[:, 1]))
    hbm = peaks()[0]
    for k, op_name, nbytes in (("k_off_source", "forward", 16 * pts), ("k_off_image", "adjoint", 16 * pts)):
        ms = out["ops"][op_name]["kernels_ms"].get(k)
        if ms:
            out["ops"][op_name][k + "_gbs"] = nbytes / (ms / 1e3) / 1e9
            out["ops"][op_name][k + "_frac_of_measured_hbm"] = nbytes / (ms / 1e3) / 1e9 / hbm
    # dot test at full size: <L r, g> = <r, L^H g> with complex bins
    rng = np.random.default_rng(7)
    nb = p.nt + p.tpad
    df = torch.zeros((p.ns, p.nr, nb), dtype=torch.complex64, device=dev)
    op.forward(r, df)
    g = torch.from_numpy((rng.standard_normal(df.shape) + 1j * rng.standard_normal(df.shape)).astype(np.complex64)).to(dev)
    im2 = torch.zeros_like(img)
    op.adjoint(im2, g)
    lhs = complex(torch.vdot(df.flatten().to(torch.complex128), g.flatten().to(torch.complex128)))
    rhs = complex(torch.vdot(r.flatten().to(torch.complex128), im2.flatten().to(torch.complex128)))
    out["dot_ratio"] = abs(lhs - rhs) / abs(lhs)
    if not args.no_parity:
        one = dict(cfg, par=dict(cfg["par"], ns=1))
        p1 = S.params_of(one)
        op1 = BornOffsetOp(p1, wav, cfg["slow"], nh, ap[:1])
        taps = list(op1.rows()[1])
        d1 = d[:1].cpu().numpy()  # the full batch's first shot
        gd = rng.standard_normal(d1.shape).astype(np.float32)
        i1 = np.zeros((nh, p.nz, p.nx), np.complex64)
        op1.adjoint(i1, gd)
        nt = os.cpu_count() or 1
        par = {}
        t0 = time.perf_counter()
        for prec in (32, 64):
            o = O.offborn_forward(p1, wav, cfg["slow"], cfg["refl"], ap[:1], taps, kind=0, prec=prec, nthreads=nt)
            if prec == 32:
                t1 = time.perf_counter()
            oi = O.offborn_adjoint(p1, wav, cfg["slow"], nh, gd, ap[:1], taps, kind=0, prec=prec, nthreads=nt)
            if prec == 32:
                t2 = time.perf_counter()
            par[f"forward_vs_fp{prec}"] = float(np.linalg.norm(d1 - o) / np.linalg.norm(o))
            par[f"adjoint_vs_fp{prec}"] = float(np.linalg.norm(i1 - oi) / np.linalg.norm(oi))
        out["parity"] = dict(par, tolerance=1e-4, sample="shot 0 at full size (the full batch's forward; "
                             "a one-shot operator's adjoint)")
        w0 = int(ap[0, 1]) + 2 * p.pad
        out["cpu_oracle"] = {"s_one_shot_forward": t1 - t0, "s_one_shot_adjoint": t2 - t1, "cores": nt, "kind": "port",
                             "depth_steps_per_s": 4 * nf * (p.nz - 1) / (t2 - t0), "aperture_cells": w0}
    print(json.dumps(out), flush=True)


def run_c5(args):
    """3D PSPI with a 2D FFT per slice (c5), timed for the record: the
    modelling (WEM on planes), the reflectivity Born forward and its adjoint
    (the migration), all 16 shots x 64 frequencies batched, the down field
    checkpointed every 20 depths; CUDA events around each call on resident
    inputs, and a full-size dot test of the migration pair."""
    import torch
    import wemgpu
    from wemgpu import synthetic as S
    from wemgpu.core import Refl3DOp, Wem3DOp

    wemgpu.build()
    dev = torch.device("cuda:0")
    cfg = S.c5()
    q, wav = cfg["q"], cfg["wavelet"]
    if args.small:  # a reduced case of the same kernels for profiling captures
        q.p.fmax = q.p.fmin + 1.0
    s = torch.from_numpy(cfg["slow"]).to(dev)
    rho = torch.from_numpy(cfg["rho"]).to(dev)
    r = torch.from_numpy(cfg["refl"]).to(dev)
    wem = Wem3DOp(q, wav)
    nf = wem.nfreq()
    op = Refl3DOp(q, wav, s)
    d = torch.zeros((q.p.ns, q.p.nr, q.p.nt), dtype=torch.float32, device=dev)
    img = torch.zeros_like(r)
    ck = 20
    rows = q.p.ns * nf
    out = {"workload": "c5 3D PSPI, 2D FFT per depth slice: modelling and migration", "small": bool(args.small),
           "nx": cfg["nx"], "ny": cfg["ny"], "nz": cfg["nz"], "shots": q.p.ns, "receivers": q.p.nr, "freqs": nf,
           "nref": q.p.nref, "checkpoint": ck, "ops": {}}
    for name, fn, sweeps in (("wem_forward", lambda: wem.forward(s, rho, d, checkpoint=ck), 3),
                             ("migration_forward", lambda: op.forward(r, d, checkpoint=ck), 3),
                             ("migration_adjoint", lambda: op.adjoint(img, d), 2)):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(max(1, args.steps)):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / max(1, args.steps)
        # depth-steps of the two one-way sweeps (the checkpointed forwards
        # recompute the down sweep once more: `sweeps` counts it)
        out["ops"][name] = {"ms": ms, "plane_steps_per_s": 2 * rows * (cfg["nz"] - 1) / (ms / 1e3),
                            "sweeps_run": sweeps}
    rng = np.random.default_rng(8)
    g = torch.from_numpy(rng.standard_normal(tuple(d.shape)).astype(np.float32)).to(dev)
    op.forward(r, d, checkpoint=ck)
    op.adjoint(img, g)
    lhs = float(torch.sum(d.double() * g.double()))
    rhs = float((r.to(torch.complex128).conj() * img.to(torch.complex128)).sum().real)
    out["dot_ratio"] = abs(lhs - rhs) / abs(lhs)
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--small", action="store_true", help="reduced case (profiling captures)")
    ap.add_argument("--small-shots", type=int, default=8, help="shots of the reduced case")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the results")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="c3", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c3 is the benchmark line; c1, c2, c4 and c5 print their own timings for the record")
    args = ap.parse_args()
    if args.workload == "c4":
        run_c4(args)
        return
    if args.workload == "c5":
        run_c5(args)
        return
    if args.workload != "c3":
        run_config(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.gpus < 1:
        sys.exit("bench.py: --gpus must be at least 1")
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        sys.exit(relaunch(args))
    if args.gpus != world:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}; launch one rank per GPU")
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gpu" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
