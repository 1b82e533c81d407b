#!/usr/bin/env python
"""Benchmark: prices/s and p50/p99 latency of the served stream, served form
(continuous batching + control variate) against the plain method.

Headline workload (the served stream): pricing requests arrive as a Poisson
process at 2000 req/s (numpy default_rng(1) exponential gaps); each request
is a basket call from the mix law (d ~ U{1..8}, steps log-U[32, 512], pilot paths =
the instance's path count log-U[2^12, 2^18], K ~ U(0.8, 1.2), sigma_i ~
U(0.1, 0.4), jump rate ~ U(0.5, 3), rho 0.3, log-jumps N(-0.1, 0.2)) with a
target relative error drawn from {1e-2, 3e-3, 1e-3}; a request is one run_mc
(pilot sizes the main run for a 95% half-width of target x |price|).  One
step = the requests arriving in one 0.1 s window of that stream; the K timed
windows are released back to back at their arrival times.

* `value`: requests / device busy time of the server's ticks (the kernels,
  uploads and readbacks the server enqueued; inputs are descriptors).
* `e2e`: requests / wall time from the first arrival to the last result,
  through the public API (descriptors submitted from the host, results read
  back to the host); latencies are arrival -> result.
* `plain`: the same stream served by the plain method one request at a time
  (pilot K1 launch + readback, main K1 launch + readback).
* `rainbow2d_plain`: the 2D rainbow at 1e-3 relative error with K1 — the
  per-path kernel every form shares — and its FP32 roofline.
* `rainbow2d_mlmc`, `batched_mix` (the 512-instance basket mix), `cv_learned`
  (the learned control variate on the 2D rainbow): the other
  forms, measured once.
`--impl reference` prices the same stream's requests with the CPU
restatement of the reference's algorithm (oracle port) on all host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "prices/s and p50/p99 latency at 1e-3 rel. error: CV+batched+served vs plain"
UNIT = "prices/s"
RATE = 2000.0
WINDOW_S = 0.1
WORKLOAD = ("served stream: Poisson arrivals at 2000 req/s (default_rng(1) exponential gaps), each a "
            "basket call from the mix law (d~U{1..8}, steps log-U[32,512], pilot paths log-U[2^12,2^18], K~U(0.8,1.2), "
            "sigma_i~U(0.1,0.4), jump rate~U(0.5,3), rho 0.3, logN(-0.1,0.2) jumps, r 0.02, T 1) with target "
            "relative error from {1e-2,3e-3,1e-3}; one step = the requests of one 0.1 s window of the stream")
RAINBOW_WORKLOAD = ("2D rainbow (call on max), Merton assets with independent per-asset jumps "
               "(rate 1.0, logN(-0.05,0.15)), sigma (0.2,0.3), rho 0.5, r 0.02, T 1, K 1, 256 jump-adapted steps; "
               "one price = plain MC at 1e-3 relative 95% half-width")
MIX_WORKLOAD = ("basket mix: 512 correlated Merton basket calls, d~U{1..8}, steps log-U[32,512], "
                "paths log-U[2^12,2^18], K~U(0.8,1.2), sigma_i~U(0.1,0.4), rate~U(0.5,3), rho 0.3, "
                "logN(-0.1,0.2) jumps; numpy default_rng(0)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-windows", type=int, default=10,
                    help="windows of the stream the plain one-request-per-launch server replays")
    ap.add_argument("--sections", default="rainbow,materialise,mlmc,mix,cv,cvserved,accuracy",
                    help="extra sections measured once: rainbow, materialise, mlmc, mix, cv, cvserved, accuracy "
                         "(comma list, or 'none')")
    ap.add_argument("--profile-store", type=int, default=0,
                    help="profiling driver: materialise this many 2D rainbow paths (K4, AdaptedPathData "
                         "layout) three times, then exit")
    ap.add_argument("--profile-paths", type=int, default=0,
                    help="profiling driver: three 2D-rainbow price launches at this many paths, then exit")
    ap.add_argument("--profile-serve", type=float, default=0.0,
                    help="profiling driver: serve this many seconds of the stream, then exit")
    ap.add_argument("--profile-cv", type=int, default=0,
                    help="profiling driver: K7 over this many 2D-rainbow paths and K5 (tcgen05) over a quarter "
                         "of them materialised, three launches each, then exit")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def make_problem(seed=1):
    import torch
    import sde_mc_gb300 as sm
    corr = sm.get_corr_matrix([0.5])
    sde = sm.IndependentJumpsMerton(0.02, torch.tensor([0.2, 0.3]), [1.0, 1.0], -0.05, 0.15, torch.ones(2), 2,
                                    corr_matrix=corr)
    return sm.JumpEulerSolver(sde, 1.0, 256, seed=seed, device="cuda"), sm.Rainbow(1.0), sm.ConstantShortRate(0.02)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
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
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_flops_per_path_step(d):
    """F(d) = 5 + 10 d + d (d+1) [d > 1] FP32 flops per path-step: Box-Muller
    (4 flops + 2 MUFU per normal), sqrt(dt) scaling, the Cholesky product, the
    Euler update (5 per component) and the time bookkeeping."""
    return 5 + 10 * d + (d * (d + 1) if d > 1 else 0)


# one earlier measurement on a GB300 each (copy bandwidth; cuBLAS bf16 burst),
# used only when MEASURED_PEAKS.json is absent
HBM_FALLBACK_GBS = 6800.0
BF16_FALLBACK_TFLOPS = 1900.0


def load_json_file(name):
    p = os.path.join(ROOT, name)
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return None


def _probe(dev, name, iters):
    import ctypes
    import torch
    from sde_mc_gb300 import _native as N
    lib = N.load()
    sink = torch.zeros(16, dtype=torch.float32, device=dev)
    fl = ctypes.c_double(0.0)
    best = 0.0
    s = N.stream_handle(dev)
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        N.check(getattr(lib, name)(iters, N.ptr(sink), 16, ctypes.byref(fl), s), name)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, fl.value / (e0.elapsed_time(e1) * 1e-3))
    return best


def fp32_peak_tflops(dev):
    """Measured FFMA throughput of this GPU (best of 6 probe launches)."""
    return _probe(dev, "sdemc_fp32_probe", 4096) / 1e12


def mufu_peak_tops(dev):
    """Measured special-function (MUFU) throughput, tera-ops/s."""
    return _probe(dev, "sdemc_mufu_probe", 1024) / 1e12


def bind_roofline(roof):
    """The path kernels have two compute ceilings, the FP32 pipe and the
    special-function (MUFU) unit; the binding one is the one with the larger
    fraction.  Its figures go to the top level, both stay under "fp32" and
    "mufu"."""
    mu = roof.pop("mufu")
    roof["fp32"] = {k: roof[k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}
    roof["mufu"] = mu
    if mu["frac"] > roof["frac"]:
        roof.update(bound="mufu", achieved=mu["achieved"], peak=mu["peak"], unit=mu["unit"], frac=mu["frac"],
                    peak_source=mu["peak_source"])
    return roof


def mufu_per_path_step(d, jumps_per_step=0.0):
    """M(d) = 2d + 1 MUFU operations per path-step (two per Box-Muller normal,
    one for sqrt(dt)), plus 5 per jump event (log of the gap, a normal for the
    mark, its exp)."""
    return 2 * d + 1 + 5.0 * jumps_per_step


def stream_windows(first, count):
    """Requests of windows [first, first + count) of the stream, times relative
    to the start of window `first`."""
    from sde_mc_gb300 import stream as S
    return S.make_stream(RATE, (first + count) * WINDOW_S, seed=1, t_begin=first * WINDOW_S)


CPU_SAMPLE = 32          # requests of the stream both arms time on the host cores
CPU_SHARE_S = 0.5        # host seconds a main run is simulated for before extrapolating
CPU_PREFIX = 4096        # pilot paths simulated before extrapolating


def cpu_sample():
    """The fixed CPU sample both bench arms time: the stream's first
    CPU_SAMPLE requests (window 0)."""
    return stream_windows(0, 1)[:CPU_SAMPLE]


def cpu_price_request(r, threads):
    """Host seconds of one request priced by the plain method (run_mc: pilot
    sizes the main run, sde_mc/mc.py:418-440) through the oracle port on
    `threads` host threads.  The pilot is simulated on its first CPU_PREFIX
    paths and the main run on at most max(4096, CPU_SHARE_S / per-path time)
    paths; both times are extrapolated linearly to the full path counts (CPU
    time is proportional to paths).  Deterministic work: the same paths, the
    same sizes, on every run.  Returns (seconds, paths simulated)."""
    from oracle import oracle
    n0 = int(r.inst.num_paths)
    k0 = min(n0, CPU_PREFIX)
    t = time.perf_counter()
    out, _, _ = oracle.price(r.phase(k0, 0), nthreads=threads)
    t_prefix = time.perf_counter() - t
    per_path = t_prefix / max(k0, 1)
    mean0, var0 = float(out[3]), float(out[4])
    eps = r.target * abs(mean0)
    n = max(64, math.ceil(1.96 ** 2 * var0 / eps ** 2)) if var0 > 0 and eps > 0 else 0
    m = min(n, max(4096, int(CPU_SHARE_S / max(per_path, 1e-12))))
    t_main = 0.0
    if m > 0:
        t = time.perf_counter()
        oracle.price(r.phase(m, n0), nthreads=threads)
        t_main = (time.perf_counter() - t) * (n / m)
    return per_path * n0 + t_main, k0 + m


def cpu_baseline_of(reqs, threads):
    """(seconds per request, paths simulated) over a list of requests."""
    secs, paths = [], 0
    for r in reqs:
        s_, p_ = cpu_price_request(r, threads)
        secs.append(s_)
        paths += p_
    return statistics.mean(secs), paths


CPU_KIND = ("oracle port: the C restatement of the reference's algorithm (its jump-adapted Euler loop, "
            "payoff and estimator), plain estimator, on the host cores; pilot and main runs timed on a prefix "
            "of their paths and extrapolated")
REFERENCE_TORCH_NOTE = ("the reference's own torch CPU path is not installed on this box; in the build container "
                        "(8 x86 threads) it priced config 1 (1-D Merton, 2^16 paths, 100 steps) in 0.64 s")


def run_reference(args):
    """`--impl reference`: the plain method on the host cores (oracle port)
    over the same fixed sample of the stream's requests as the main arm's
    cpu_baseline, each request timed once: the timed steps partition the
    sample; warm-up steps price the first requests' pilots untimed."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    reqs = cpu_sample()
    threads = os.cpu_count() or 1
    for r in reqs[:max(args.warmup, 0)]:
        oracle.price(r.phase(min(int(r.inst.num_paths), CPU_PREFIX), 0), nthreads=threads)
    steps = max(args.steps, 1)
    groups = [reqs[i * len(reqs) // steps:(i + 1) * len(reqs) // steps] for i in range(steps)]
    secs, walls, paths = [], [], 0
    for g in groups:
        t0 = time.perf_counter()
        for r in g:
            s_, p_ = cpu_price_request(r, threads)
            secs.append(s_)
            paths += p_
        walls.append(time.perf_counter() - t0)
    sec_per_price = statistics.mean(secs)
    value = 1.0 / sec_per_price
    # config 1 on the same port and threads, for reading the port against the reference's torch timing
    import torch
    import sde_mc_gb300 as sm
    from sde_mc_gb300.lowering import lower
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    c1 = lower(sm.JumpEulerSolver(m, 1.0, 100), sm.EuroCall(1.0), sm.ConstantShortRate(0.02), num_paths=1 << 16)
    t0 = time.perf_counter()
    oracle.price(c1, nthreads=threads)
    c1_s = time.perf_counter() - t0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "reference_kind": CPU_KIND,
            "config": {"workload": WORKLOAD, "form": "plain run_mc per request (oracle port, host cores)",
                       "step": "a share of the fixed %d-request sample (the stream's first requests), each "
                               "request timed once; value = requests / their pilot + main time" % len(reqs),
                       "ms_per_price": sec_per_price * 1e3, "config1_port_s": c1_s, "threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "the stream's first %d requests (pilot + main, plain estimator, %d paths "
                                       "simulated, extrapolated to the full counts) on %d threads"
                                       % (len(reqs), paths, threads),
                             "config1_port_s": c1_s, "reference_torch": REFERENCE_TORCH_NOTE},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def csrc_digest():
    """Digest of the kernel sources (csrc and the ABI header): an ncu figure in
    profiles/ is reported only when it was captured from these sources."""
    import hashlib
    h = hashlib.sha256()
    base = os.path.join(ROOT, "sde_mc_gb300", "csrc")
    for f in sorted(os.listdir(base)):
        if f.endswith((".cu", ".cuh")):
            with open(os.path.join(base, f), "rb") as fh:
                h.update(f.encode() + b"\0" + fh.read())
    with open(os.path.join(ROOT, "include", "sdemc.h"), "rb") as fh:
        h.update(fh.read())
    return h.hexdigest()[:16]


def profiled(kernel):
    """The ncu record of `kernel` in profiles/kernel_traffic.json when it was
    captured from the current kernel sources, else None."""
    rec = (load_json_file(os.path.join("profiles", "kernel_traffic.json")) or {}).get(kernel)
    if rec and rec.get("csrc_digest") == csrc_digest():
        return rec
    return None


# ------------------------------------------------------------ sections ----
def bench_rainbow_plain(dev, steps, warmup, fp32_peak, mufu_peak):
    """The 2D rainbow at 1e-3 relative error with K1 (+K10), device-timed, L2
    flushed between steps; the FP32 roofline of price_kernel<2>."""
    import ctypes
    import torch
    import sde_mc_gb300 as sm
    from sde_mc_gb300 import _native as N
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    lib = N.load()
    pilot = K.price(lower(solver, payoff, disc, num_paths=1 << 18, path_offset=0, seed=7)).cpu().tolist()
    price, var = pilot[3], pilot[4]
    n_target = int(math.ceil((1.96 * math.sqrt(var) / (1e-3 * price)) ** 2))
    n_target = (n_target + 127) // 128 * 128
    m = K.materialise(lower(solver, payoff, disc, num_paths=1 << 14, path_offset=1 << 40, seed=7),
                      solver.num_steps + solver.max_jumps, want=("steps",))
    steps_per_path = float(m["steps"].double().mean())
    flops = n_target * steps_per_path * algorithmic_flops_per_path_step(2)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    need = lib.sdemc_price_scratch_bytes(ctypes.byref(lower(solver, payoff, disc, num_paths=n_target)))
    scratch = N.SCRATCH.get(need, dev)
    out = torch.empty(6, dtype=torch.float64, device=dev)
    nch = (n_target + N.CHUNK_PATHS - 1) // N.CHUNK_PATHS
    s = N.stream_handle(dev)

    def one(i, ev=None):
        inst = lower(solver, payoff, disc, num_paths=n_target, path_offset=(i + 1) * n_target, seed=1)
        if ev:
            ev[0].record()
        N.check(lib.sdemc_price_chunks(ctypes.byref(inst), None, N.ptr(scratch), scratch.numel(), None, s), "chunks")
        if ev:
            ev[1].record()
        N.check(lib.sdemc_reduce_chunks(N.ptr(scratch), nch, 3, N.ptr(out), s), "reduce")
        if ev:
            ev[2].record()

    for i in range(warmup):
        one(i)
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    res = []
    for i in range(steps):
        flush.fill_(i & 0xFF)
        one(warmup + i, evs[i])
        res.append(out.clone())
    torch.cuda.synchronize()
    k_ms = [e[0].elapsed_time(e[1]) for e in evs]
    r_ms = [e[1].elapsed_time(e[2]) for e in evs]
    rows = [r.cpu().tolist() for r in res]
    for r in rows:
        N.status_error(r[5], "bench rainbow2d")
    e2e = []
    for i in range(warmup + min(steps, 10)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sm.mc_simple(n_target, solver, payoff, disc, bs=n_target, payoff_time='adapted')
        if i >= warmup:
            e2e.append(time.perf_counter() - t0)
    kernel_s = statistics.mean(k_ms) * 1e-3
    achieved = flops / kernel_s / 1e12
    mufu_ops = n_target * steps_per_path * mufu_per_path_step(2, 2.0 / steps_per_path)
    mufu_achieved = mufu_ops / kernel_s / 1e12
    traffic = profiled("price_kernel<2,diag>")
    return {"workload": RAINBOW_WORKLOAD, "paths_per_price": n_target, "steps_per_path": steps_per_path,
            "prices_per_s": steps / (sum(k_ms) + sum(r_ms)) * 1e3, "ms_per_price": statistics.mean(
                [a + b for a, b in zip(k_ms, r_ms)]),
            "e2e_prices_per_s": len(e2e) / sum(e2e), "price": statistics.mean(r[3] for r in rows),
            "rel_halfwidth": statistics.mean(1.96 * math.sqrt(r[4] / r[2]) / r[3] for r in rows),
            "path_steps_per_s": n_target * steps_per_path / kernel_s,
            "roofline": bind_roofline({"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak,
                         "traffic": traffic["dram_bytes"] if traffic else None,
                         "traffic_note": "DRAM bytes of one ncu-captured launch (2^20 paths) of these kernel "
                                         "sources (null when profiles/ holds no capture of them): descriptor "
                                         "and chunk partials only; paths stay in registers",
                         "issue_active_ncu": traffic.get("issue_active") if traffic else None,
                         "issue_note": "share of cycles an instruction issued (ncu, profiles/): the path loop is "
                                       "issue-bound, mostly Philox's integer rounds, which count as no flop",
                         "kernel": "price_kernel<2,diag>", "kernel_ms": kernel_s * 1e3,
                         "flops_per_path_step": algorithmic_flops_per_path_step(2),
                         "peak_source": "measured FFMA probe on this GPU (sdemc_fp32_probe)",
                         "mufu": {"achieved": mufu_achieved, "peak": mufu_peak, "unit": "Tops/s",
                                  "frac": mufu_achieved / mufu_peak,
                                  "ops_per_path_step": mufu_per_path_step(2, 2.0 / steps_per_path),
                                  "peak_source": "measured rsqrt.approx probe (sdemc_mufu_probe)"}}),
            "l2": "flushed (256 MB write) between timed steps", "gpu_launches": 2 * steps}


def bench_materialise(dev, hbm_peak, peak_source="MEASURED_PEAKS.json hbm_gbs (copy, read + write)"):
    """Materialised mode (K4): the 2D rainbow's paths in the AdaptedPathData
    layout (paths, left limits, time, jumps: S + 1 rows; normals: S rows),
    2^20 paths, timed on the kernel alone; HBM roofline of the stores."""
    import ctypes
    import torch
    from sde_mc_gb300 import _native as N
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    n, d = 1 << 20, 2
    S = solver.num_steps + solver.max_jumps
    f32 = dict(dtype=torch.float32, device=dev)
    bufs = {"paths": torch.empty((n, S + 1, d), **f32), "left": torch.empty((n, S + 1, d), **f32),
            "time": torch.empty((n, S + 1), **f32), "jumps": torch.empty((n, S + 1, d), **f32),
            "normals": torch.empty((n, S, d), **f32), "payoffs": torch.empty(n, **f32),
            "steps": torch.empty(n, dtype=torch.int32, device=dev)}
    nbytes = sum(b.numel() * b.element_size() for b in bufs.values())
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = N.load()
    s = N.stream_handle(dev)

    def run(i):
        inst = lower(solver, payoff, disc, num_paths=n, path_offset=(i + 1) * n, seed=3)
        g = bufs.get
        N.check(lib.sdemc_materialise(ctypes.byref(inst), S, N.ptr(g("paths")), N.ptr(g("left")),
                                      N.ptr(g("time")), N.ptr(g("jumps")), N.ptr(g("normals")),
                                      N.ptr(g("payoffs")), N.ptr(g("steps")), None, 0, None, None, None, 0,
                                      N.ptr(status), s), "materialise")

    for i in range(3):
        run(i)
    torch.cuda.synchronize()
    ms = []
    for i in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run(3 + i)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    N.status_error(int(status.item()), "materialise")
    t = statistics.mean(ms) * 1e-3
    executed = float(bufs["steps"].double().sum())
    gbs = nbytes / t / 1e9
    # DRAM bytes of an ncu-captured launch of these sources (a smaller case),
    # scaled by paths: the layout's bytes grow in proportion to the paths
    rec = profiled("materialise_kernel<2,diag>")
    traffic = rec["dram_bytes"] * n / rec["paths"] if rec and rec.get("paths") else None
    return {"workload": "2D rainbow, 2^20 paths, AdaptedPathData layout at %d step rows" % S,
            "bytes_written": nbytes, "ms": t * 1e3, "path_steps_per_s": executed / t,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": gbs / hbm_peak if hbm_peak else None,
                         "peak_source": peak_source,
                         "bytes": "the layout's arrays: (S + 1) rows x (3d + 1) floats + S rows x d floats "
                                  "per path, + payoff and step count",
                         "traffic": traffic,
                         "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu-captured launch "
                                         "(%s paths) scaled to %d paths; null when profiles/ holds no capture of "
                                         "these kernel sources" % (rec.get("paths") if rec else "-", n)},
            "l2": "outputs (%.1f GB) far larger than L2" % (nbytes / 1e9)}


def bench_rainbow_mlmc(dev):
    """The 2D rainbow with MLMC (levels 0..6, 2^(l+2) steps) at eps = 1e-3 x price:
    Giles' allocation from a 2^14-path pilot per level, then one run; both
    timed warm (mean of 3 after an untimed call)."""
    import torch
    import sde_mc_gb300 as sm
    solver, payoff, disc = make_problem()
    levels = [2 ** (l + 2) for l in range(7)]
    ref = sm.mc_simple(1 << 20, solver, payoff, disc, bs=1 << 20, payoff_time='adapted')
    eps = 1e-3 * ref.sample_mean
    # the pilot warm (the first call also loads each level's kernel), then timed
    sm.get_optimal_trials(1 << 14, levels, eps, solver, payoff, disc)
    pilot_times = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trials = sm.get_optimal_trials(1 << 14, levels, eps, solver, payoff, disc)
        pilot_times.append(time.perf_counter() - t0)
    t_pilot = statistics.mean(pilot_times)
    times = []
    for i in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = sm.mc_multilevel(trials, levels, solver, payoff, disc)
        times.append(time.perf_counter() - t0)
    run_s = statistics.mean(times[1:])
    fine_steps = sum(n * (lv + 1.0) for n, lv in zip(trials, levels))
    return {"levels": levels, "trials": trials, "eps": eps, "price": st.sample_mean,
            "halfwidth": 1.96 * st.sample_std, "prices_per_s": 1.0 / run_s,
            "prices_per_s_with_pilot": 1.0 / (run_s + t_pilot), "path_steps_fine_equiv": fine_steps,
            "note": "MLMC estimates E[P_L] at L = 256 steps (level 6); the plain rainbow2d section prices the same target"}


def bench_batched_mix(steps, warmup):
    """The basket mix: the whole mix per step, batched (K8, autotuned, CUDA graph)
    against the plain method one request per launch (K1 + K10 each)."""
    import torch
    from sde_mc_gb300 import batch as B
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300 import workloads
    mix = workloads.basket_mix(512)
    n = len(mix)
    insts = B.lower_mix(mix, [0] * n)
    plan = B.BatchPlan(insts)
    tune = B.autotune(plan, repeats=2)
    steps = max(1, min(steps, 10))
    plan.set_path_offsets([1 << 40 for _ in mix])
    plan.run()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.upload()
        plan.launch()
    ms = []
    for s in range(warmup + steps):
        plan.set_path_offsets([(s + 2) * (1 << 24) for _ in mix])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize()
        if s >= warmup:
            ms.append(e0.elapsed_time(e1))
    rows = plan.out[:n].cpu().numpy()
    batched_ms = sum(ms) / len(ms)
    plain_insts = B.lower_mix(mix, [(1 << 41)] * n)
    outs = [torch.empty(6, dtype=torch.float64, device="cuda") for _ in range(n)]
    pm = []
    for s in range(max(1, warmup // 2) + steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for ins, o in zip(plain_insts, outs):
            K.price(ins, out=o)
        e1.record()
        torch.cuda.synchronize()
        if s >= max(1, warmup // 2):
            pm.append(e0.elapsed_time(e1))
    plain_ms = sum(pm) / len(pm)
    work = sum(m.paths * (m.solver.num_steps + float(m.solver.sde.jump_rate())) for m in mix)
    return {"workload": MIX_WORKLOAD, "instances": n, "steps": steps,
            "batched": {"prices_per_s": n / (batched_ms * 1e-3), "ms_per_mix": batched_ms,
                        "launch": {"block_threads": tune["choice"][0], "side_streams": tune["choice"][1],
                                   "paths_per_lane_by_class": tune["choice"][2] if len(tune["choice"]) > 2 else None,
                                   "classes": ["d%d" % c.dim for c in plan.classes[:plan.header.n_class]]},
                        "graph": True, "gpu_launches_per_mix": 1 + 1 + len(plan.classes[:plan.header.n_class])},
            "plain_one_per_launch": {"prices_per_s": n / (plain_ms * 1e-3), "ms_per_mix": plain_ms,
                                     "gpu_launches_per_mix": 2 * n},
            "speedup_batched_vs_plain": plain_ms / batched_ms,
            "path_steps_per_mix": work, "batched_path_steps_per_s": work / (batched_ms * 1e-3),
            "status_ok": bool((rows[:, 5] == 0).all())}


def bench_cv_learned(dev, epochs=10):
    """The learned control variate on the 2D rainbow model — train
    Mlp(3, [64, 64, 64], 2) with Adam (lr 1e-3, batch 4096) on 2^18 paths the
    solver generates (K4 + K5/K6), evaluate on 2^22 fresh paths (K4 + K5);
    VRF against the plain estimator on the same fresh paths and the bias."""
    import torch
    import sde_mc_gb300 as sm
    solver, payoff, disc = make_problem()
    torch.manual_seed(0)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    opt = torch.optim.Adam(f.parameters(), lr=1e-3)
    models = [f, sm.ZeroFunction(2)]
    sm.simulate_adapted_data(1 << 18, solver, payoff, disc, bs=4096)  # warm-up: allocator, first launches
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dl = sm.simulate_adapted_data(1 << 18, solver, payoff, disc, bs=4096)
    torch.cuda.synchronize()
    t_sim = time.perf_counter() - t0
    train_steps = int(dl.dataset.normals.shape[1])
    t0 = time.perf_counter()
    losses = sm.train_adapted_control_variates(models, opt, dl, solver, disc, epochs=epochs, print_losses=False)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del dl
    n_eval = 1 << 22
    start = solver.path_cursor
    t0 = time.perf_counter()
    st_cv = sm.mc_apply_cvs(models, solver, n_eval, payoff, disc, sim_bs=1 << 18, bs=4096)
    torch.cuda.synchronize()
    t_eval = time.perf_counter() - t0
    eval_steps = train_steps  # same model and grid: the adapted step count per batch
    plain = sm.price_stats(solver, payoff, disc, n_eval, payoff_time='adapted', path_offset=start)
    mean_p, se_p, _ = sm.finish_stats(plain)
    vrf = (se_p / st_cv.sample_std) ** 2
    bias = st_cv.sample_mean - mean_p
    # tensor-core work: K5 forward 2(3*64 + 64*64 + 64*64 + 64*2) flops per
    # (path, step) row; a training step runs K5 and K6 (forward recompute,
    # input and weight gradients: three forwards' worth)
    fwd = 2 * (3 * 64 + 64 * 64 + 64 * 64 + 64 * 2)
    rows_train = epochs * ((1 << 18) // 4096) * 4096 * train_steps
    rows_eval = n_eval * eval_steps
    peaks = load_json_file("MEASURED_PEAKS.json") or {}
    bf16 = peaks.get("bf16_tflops")
    bf16_source = "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"
    if not bf16:
        bf16, bf16_source = BF16_FALLBACK_TFLOPS, "fallback 1.9 PFLOP/s (MEASURED_PEAKS.json absent)"
    tf_train = rows_train * 4 * fwd / t_train / 1e12
    tf_eval = rows_eval * fwd / t_eval / 1e12
    # the served form's regression control variate on the same model and target
    from sde_mc_gb300 import serve
    with serve.Server(max_slots=8, mem_budget=1 << 30, device=dev) as srv:
        for tag, est in ((1, "plain"), (2, "linear_cv")):
            srv.submit(solver, payoff, disc, rel_target=1e-3, pilot_paths=1 << 18, estimator=est, tag=tag,
                       stream_id=1000)
        reg = {r.tag: r for r in srv.wait(2)}
    return {"workload": "learned CV on the 2D rainbow model, Mlp(3,[64,64,64],2) ReLU no BN, Adam lr 1e-3 "
                        "batch 4096, %d epochs on 2^18 solver paths, evaluated on 2^22 fresh paths" % epochs,
            "vrf": vrf, "mean_cv": st_cv.sample_mean, "se_cv": st_cv.sample_std, "mean_plain": mean_p,
            "se_plain": se_p, "bias": bias, "bias_in_se": bias / math.hypot(st_cv.sample_std, se_p),
            "loss_first_last": [losses[0], losses[-1]], "simulate_s": t_sim, "train_s": t_train, "eval_s": t_eval,
            "train_rows": rows_train, "eval_rows": rows_eval,
            "train_tflops": tf_train, "eval_tflops_incl_paths": tf_eval,
            "bf16_peak_tflops": bf16, "bf16_peak_source": bf16_source, "train_frac_of_bf16_peak": tf_train / bf16,
            "regression_cv_same_model": {"vrf": reg[2].vrf, "mean": reg[2].mean, "se": reg[2].se,
                                         "plain_mean": reg[1].mean, "plain_se": reg[1].se,
                                         "main_paths_cv": reg[2].main_paths, "main_paths_plain": reg[1].main_paths},
            "eval_kernel": "K7 price_cv_kernel: paths + payoff + network on tcgen05 in one pass",
            "note": "the plain estimate uses the same 2^22 fresh paths as the control-variate estimate; eval "
                    "simulates the paths inside the same kernel (nothing materialised)"}


def bench_cv_learned_served(dev, n_requests=24, epochs=4):
    """The learned control variate on the served stream's requests with d <= 2
    (the dimensions the network form covers), one request at a time through
    the reference's run_cv_mc flow (sde_mc/mc.py:443-467): train
    Mlp(1 + d, [64, 64, 64], d) on the request's pilot paths (K4 + K5/K6),
    size the main run for a 95% half-width of target x |price| from a
    control-variate pilot of the same size on fresh paths, then price the main
    run with K7.  Reported beside the served regression control variate and
    the plain estimator on the same requests (device time to the target)."""
    import numpy as np
    import torch
    import sde_mc_gb300 as sm
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300 import serve
    from sde_mc_gb300 import stream as S
    reqs = [r for r in S.make_stream(RATE, 1.0, seed=1) if r.dim <= 2][:n_requests + 1]
    warm, reqs = reqs[0], reqs[1:]
    rows = []
    for r in [warm] + reqs:  # the first one untimed: kernel loading and allocator warm-up
        m = r.instance()
        solver, payoff, disc, d = m.solver, m.payoff, m.discounter, m.dim
        torch.manual_seed(r.idx)
        f = sm.Mlp(1 + d, [64, 64, 64], d, batch_norm=False, batch_norm_init=False)
        opt = torch.optim.Adam(f.parameters(), lr=1e-3)
        models = [f, sm.ZeroFunction(d)]
        n0 = int(r.inst.num_paths)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dl = sm.simulate_adapted_data(n0, solver, payoff, disc, bs=min(4096, n0))
        sm.train_adapted_control_variates(models, opt, dl, solver, disc, epochs=epochs, print_losses=False)
        del dl
        pilot = sm.mc_apply_cvs(models, solver, n0, payoff, disc)
        sd = pilot.sample_std * math.sqrt(n0)
        n = max(64, int(math.ceil((1.96 * sd / (r.target * abs(pilot.sample_mean))) ** 2)))
        st = sm.mc_apply_cvs(models, solver, n, payoff, disc)
        torch.cuda.synchronize()
        t_cv = time.perf_counter() - t0
        # the plain estimator on the same request: its pilot variance sizes its main run
        pl = K.price(r.phase(n0, 1 << 40)).cpu().tolist()
        n_plain = max(64, int(math.ceil(1.96 ** 2 * pl[4] / (r.target * abs(pl[3])) ** 2)))
        if r is warm:
            continue
        rows.append({"idx": r.idx, "dim": d, "target": r.target, "pilot_paths": n0, "main_paths": n,
                     "vrf": pl[4] / max(sd * sd, 1e-300), "service_s": t_cv, "mean": st.sample_mean,
                     "plain_main_paths": n_plain})
    # the served regression control variate on the same requests, alone in a server
    with serve.Server(max_slots=64, mem_budget=4 << 30, device=dev) as srv:
        t0 = time.perf_counter()
        for r in reqs:
            srv.submit_inst(r.inst, r.target, estimator="linear_cv", tag=r.idx)
        res = {x.tag: x for x in srv.wait(len(reqs))}
        t_reg = time.perf_counter() - t0
        busy = srv.stats()["busy_s"]
    for row in rows:
        x = res[row["idx"]]
        row.update(regression_vrf=x.vrf, regression_main_paths=x.main_paths,
                   regression_vs_learned_in_se=(x.mean - row["mean"]) / max(x.se, 1e-300))
    svc = np.asarray([row["service_s"] for row in rows])
    return {"workload": "the served stream's requests with d <= 2 (the network form's dimensions), %d after one "
                        "untimed warm-up request" % len(rows),
            "form": "learned CV per request: train on the pilot paths (%d epochs, Adam lr 1e-3, batch 4096), "
                    "CV pilot on fresh paths, main run with K7" % epochs,
            "requests": len(rows), "learned_prices_per_s": len(rows) / float(svc.sum()),
            "learned_service_p50_ms": float(np.percentile(svc, 50) * 1e3),
            "learned_service_p99_ms": float(np.percentile(svc, 99) * 1e3),
            "learned_vrf_median": float(np.median([row["vrf"] for row in rows])),
            "regression_prices_per_s_busy": len(rows) / busy, "regression_wall_s": t_reg,
            "regression_vrf_median": float(np.median([row["regression_vrf"] for row in rows])),
            "main_paths_learned_over_regression": float(np.median([row["main_paths"] / max(row["regression_main_paths"], 1)
                                                                   for row in rows])),
            "rows": rows,
            "note": "a network is trained per request (the reference's learned CV has no form shared across "
                    "instances), so its cost is the training, not the main run"}


def _err(mean, se, ref, ref_se):
    e = mean - ref
    return {"price": mean, "err": e, "rel_err": e / ref, "err_in_se": e / math.hypot(se, ref_se)}


def bench_accuracy(dev, line, served):
    """Every price of the bench against an FP64 oracle: the Merton series for
    the 1-D Merton call; for the 2D rainbow (no closed form) a 2^26-path run
    of K11, which repeats the path arithmetic in FP64; for the served stream a
    sample of requests, each against its own K11 run on fresh paths.  K11 on
    the same paths as an FP32 run isolates the FP32 arithmetic's error."""
    import torch
    import sde_mc_gb300 as sm
    from sde_mc_gb300 import _native as N
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower
    out = {}
    # the 1-D Merton call (100 steps, 2^16 paths)
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    inst = lower(sm.JumpEulerSolver(m, 1.0, 100, seed=1), sm.EuroCall(1.0), sm.ConstantShortRate(0.02),
                 num_paths=1 << 16)
    a, b = K.price(inst).cpu().tolist(), K.price_f64(inst).cpu().tolist()
    series = sm.merton_call(1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0)
    out["merton1d"] = {"workload": "1-D Merton call, 100 jump-adapted steps, 2^16 paths",
                       "oracle": "Merton series (FP64)", "oracle_value": series,
                       "fp32": _err(a[3], math.sqrt(a[4] / a[2]), series, 0.0),
                       "fp64_same_paths": _err(b[3], math.sqrt(b[4] / b[2]), series, 0.0),
                       "fp32_minus_fp64_same_paths_rel": (a[3] - b[3]) / b[3]}
    # the 2D rainbow: FP64 reference run on 2^26 paths
    solver, payoff, disc = make_problem()
    n_ref = 1 << 26
    ref_inst = lower(solver, payoff, disc, num_paths=n_ref, path_offset=1 << 44, seed=99)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = K.price_f64(ref_inst).cpu().tolist()
    t_ref = time.perf_counter() - t0
    N.status_error(r[5], "fp64 reference")
    ref, ref_se = r[3], math.sqrt(r[4] / r[2])
    rb = {"workload": RAINBOW_WORKLOAD, "oracle": "K11 FP64 run, 2^26 paths", "oracle_value": ref,
          "oracle_se": ref_se, "oracle_s": t_ref, "fp64_path_steps_per_s": None}
    plain = line.get("rainbow2d_plain") or {}
    if "price" in plain:
        n = plain["paths_per_price"]
        se = plain["rel_halfwidth"] * plain["price"] / 1.96
        rb["plain_fp32"] = _err(plain["price"], se, ref, ref_se)
        same = lower(solver, payoff, disc, num_paths=n, path_offset=n, seed=1)
        a, b = K.price(same).cpu().tolist(), K.price_f64(same).cpu().tolist()
        rb["fp32_minus_fp64_same_paths_rel"] = (a[3] - b[3]) / b[3]
        rb["fp32_minus_fp64_same_paths_in_se"] = (a[3] - b[3]) / math.sqrt(b[4] / b[2])
        rb["fp64_path_steps_per_s"] = n_ref * plain["steps_per_path"] / t_ref
    ml = line.get("rainbow2d_mlmc") or {}
    if "price" in ml:
        rb["mlmc"] = _err(ml["price"], ml["halfwidth"] / 1.96, ref, ref_se)
    cv = line.get("cv_learned") or {}
    if "mean_cv" in cv:
        rb["learned_cv"] = _err(cv["mean_cv"], cv["se_cv"], ref, ref_se)
        reg = cv.get("regression_cv_same_model") or {}
        if "mean" in reg:
            rb["served_regression_cv"] = _err(reg["mean"], reg["se"], ref, ref_se)
    out["rainbow2d"] = rb
    # served requests: every k-th timed request against its own FP64 run
    if served:
        res, timed = served["results"], served["timed"]
        step = max(1, len(timed) // 16)
        rows = []
        t0 = time.perf_counter()
        for q in timed[::step][:16]:
            x = res[q.idx]
            sd = x.pilot_se * math.sqrt(x.pilot_paths)
            n_q = int(min(1 << 24, max(1 << 20, 9 * (sd / max(x.se, 1e-300)) ** 2)))
            rr = K.price_f64(q.phase(n_q, 1 << 44)).cpu().tolist()
            N.status_error(rr[5], "fp64 served reference")
            e = _err(x.mean, x.se, rr[3], math.sqrt(rr[4] / rr[2]))
            e.update(target=q.target, dim=q.dim, fp64_paths=n_q, estimator=x.estimator_name,
                     within_target=abs(e["err"]) <= q.target * abs(rr[3]))
            rows.append(e)
        out["served_sample"] = {
            "requests": len(rows), "seconds": time.perf_counter() - t0,
            "within_target": sum(1 for e in rows if e["within_target"]),
            "within_1.96_se": sum(1 for e in rows if abs(e["err_in_se"]) <= 1.96),
            "max_abs_err_in_se": max(abs(e["err_in_se"]) for e in rows),
            "median_rel_err_over_target": statistics.median(abs(e["rel_err"]) / e["target"] for e in rows),
            "rows": rows,
            "note": "each request's price vs a K11 FP64 run of the same instance on fresh paths "
                    "(2^20..2^24 paths, about a third of the request's standard error)"}
    return out


def shard(reqs, rank, world):
    """Requests of one rank: the stream is partitioned by request index (each
    request is independent; no exchange on the data path)."""
    return [r for r in reqs if r.idx % world == rank]


def bench_served(dev, steps, warmup, plain_windows, rank=0, world=1):
    """The headline: K windows of the served stream through the server, and
    the plain one-request-per-launch server on the first windows."""
    import torch
    from sde_mc_gb300 import serve
    from sde_mc_gb300 import stream as S
    srv = serve.Server(max_slots=4096, mem_budget=40 << 30, side_streams=8, policy="srpt", device=dev)
    warm = shard(stream_windows(0, warmup), rank, world)
    S.run_served(warm, srv)
    timed = shard(stream_windows(warmup, steps), rank, world)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    flush.fill_(1)
    torch.cuda.synchronize()
    st0 = srv.stats()
    res, summ = S.run_served(timed, srv)
    st1 = srv.stats()
    srv.close()
    busy = st1["busy_s"] - st0["busy_s"]
    delta = {k: st1[k] - st0[k] for k in ("ticks", "launches", "h2d_bytes", "d2h_bytes", "path_steps")}
    flops = mufu = 0.0
    for r in timed:
        x = res[r.idx]
        flops += (x.pilot_paths + x.main_paths) * r.path_steps * algorithmic_flops_per_path_step(r.dim)
        jps = r.rate * float(r.inst.T) / r.path_steps
        mufu += (x.pilot_paths + x.main_paths) * r.path_steps * mufu_per_path_step(r.dim, jps)
    # capacity: the same requests released at once (no arrival gaps)
    import copy
    burst = [copy.copy(r) for r in timed]
    for r in burst:
        r.t = 0.0
    srv = serve.Server(max_slots=4096, mem_budget=40 << 30, side_streams=8, policy="srpt", device=dev)
    c0 = srv.stats()
    _, csumm = S.run_served(burst, srv)
    c1 = srv.stats()
    srv.close()
    capacity = {"requests": csumm["requests"], "prices_per_s_busy": csumm["requests"] / (c1["busy_s"] - c0["busy_s"]),
                "prices_per_s_e2e": csumm["prices_per_s"], "p50_ms": csumm["p50_ms"], "p99_ms": csumm["p99_ms"]}
    plain_reqs = [r for r in timed if r.t < min(steps, plain_windows) * WINDOW_S]
    S.run_plain(warm[:50])
    _, psumm = S.run_plain(plain_reqs)
    # price agreement between the two servers (each within its own error)
    return {"summary": summ, "busy_s": busy, "delta": delta, "flops": flops, "mufu": mufu, "plain": psumm,
            "capacity": capacity,
            "plain_windows": min(steps, plain_windows), "results": res, "timed": timed}


def profile_serve(seconds):
    """The served stream for `seconds` seconds (600 windows = the full 60 s
    stream of the served-stream workload): prices/s, p50/p99 per 10 s segment
    (does the server drift?), the tick-duration histogram and the server's
    counters."""
    import numpy as np
    import torch
    from sde_mc_gb300 import serve
    from sde_mc_gb300 import stream as S
    reqs = S.make_stream(RATE, seconds, seed=1)
    with serve.Server(max_slots=4096, mem_budget=40 << 30, side_streams=8, policy="srpt") as srv:
        res, summ = S.run_served(reqs, srv)
        st = srv.stats()
    torch.cuda.synchronize()
    segs = []
    for a in range(0, int(math.ceil(seconds)), 10):
        lat = [res[r.idx].latency_s for r in reqs if a <= r.t < a + 10]
        if lat:
            segs.append({"from_s": a, "requests": len(lat), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                         "p99_ms": float(np.percentile(lat, 99) * 1e3)})
    edges = ["<0.125"] + ["%g-%g" % (0.125 * 2 ** (b - 1), 0.125 * 2 ** b) for b in range(1, 15)] + [">=2048"]
    summ.update(stats=st, segments=segs, busy_prices_per_s=len(reqs) / st["busy_s"],
                tick_ms_hist={e: n for e, n in zip(edges, st["tick_hist"]) if n})
    print(json.dumps(summ))


def profile_cv(n):
    import torch
    import sde_mc_gb300 as sm
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300 import varred as V
    solver, payoff, disc = make_problem()
    dev = torch.device("cuda")
    torch.manual_seed(0)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    cv = V.GpuCv(f, 2, dev)
    for i in range(3):
        r = K.price_cv(solver.lower(payoff, disc, num_paths=n), cv.params, 0.02)
    dl = sm.simulate_adapted_data(n // 4, solver, payoff, disc, bs=n // 4, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, dev)
    for i in range(3):
        g = cv.forward_tc(data, 0.02)
    idx = torch.arange(min(4096, data.n), device=dev)
    gb = cv.forward(data, 0.02, idx)
    for i in range(3):
        cv.backward_tc(data, 0.02, gb, idx)
    torch.cuda.synchronize()
    print(json.dumps({"profile_cv": n, "k7": r.cpu().tolist(), "tc_status": int(cv._tc_status.item()),
                      "tc_mean": float(g.double().mean()), "bwd_status": int(cv._bwd_status.item()),
                      "grad_norm": float(cv.grad.norm())}))


def profile_store(n):
    import torch
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    S = solver.num_steps + solver.max_jumps
    for i in range(3):
        m = K.materialise(lower(solver, payoff, disc, num_paths=n, path_offset=i * n, seed=3), S,
                          want=("paths", "left", "time", "jumps", "normals", "payoffs", "steps"))
    torch.cuda.synchronize()
    print(json.dumps({"profile_store": n, "status": int(m["status"].item()),
                      "steps_mean": float(m["steps"].double().mean())}))


def profile_launches(n):
    import torch
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    for i in range(3):
        r = K.price(lower(solver, payoff, disc, num_paths=n, path_offset=i * n, seed=1))
    torch.cuda.synchronize()
    print(json.dumps({"profile_paths": n, "result": r.cpu().tolist()}))


def _section(fn, *a):
    try:
        return fn(*a)
    except Exception as e:  # an auxiliary section must not hide the headline
        return {"error": "%s: %s" % (type(e).__name__, e)}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_paths:
        return profile_launches(args.profile_paths)
    if args.profile_store:
        return profile_store(args.profile_store)
    if args.profile_serve:
        return profile_serve(args.profile_serve)
    if args.profile_cv:
        return profile_cv(args.profile_cv)
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    fp32_peak = fp32_peak_tflops(dev)
    mufu_peak = mufu_peak_tops(dev)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        b = bench_served(dev, args.steps, args.warmup, args.plain_windows, rank, world)
    if world > 1:
        dist.barrier()
    summ, busy = b["summary"], b["busy_s"]
    n_req = summ["requests"]
    wall = summ["seconds"]
    if world > 1:
        t = torch.tensor([busy, wall], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        busy, wall = float(t[0]), float(t[1])
        c = torch.tensor([n_req], device=dev, dtype=torch.float64)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        n_req = int(c.item())
    value = n_req / busy
    e2e = n_req / wall
    achieved = b["flops"] / busy / 1e12
    plain = b["plain"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": busy * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "served: continuous-batching server (SRPT ticks, up to 4 in flight, 8 side streams each, "
                                              "40 GB admission budget) + delta-weighted regression control "
                                              "variate on every request",
                   "requests": n_req, "windows": args.steps, "window_s": WINDOW_S, "arrival_rate": RATE,
                   "l2": "inputs are descriptors; L2 flushed (256 MB write) before the timed stream",
                   "parallelism": ("stream sharded by request index over %d GPUs" % world) if world > 1
                   else "single GPU",
                   "vs_plain": {"served_prices_per_s_e2e": e2e, "served_p50_ms": summ["p50_ms"],
                                "served_p99_ms": summ["p99_ms"], "plain_prices_per_s": plain["prices_per_s"],
                                "plain_p50_ms": plain["p50_ms"], "plain_p99_ms": plain["p99_ms"],
                                "speedup_e2e": e2e / plain["prices_per_s"],
                                "speedup_p50": plain["p50_ms"] / summ["p50_ms"],
                                "speedup_p99": plain["p99_ms"] / summ["p99_ms"],
                                "capacity_prices_per_s": b["capacity"]["prices_per_s_e2e"],
                                "capacity_p99_ms": b["capacity"]["p99_ms"],
                                "median_vrf": summ.get("vrf_median"),
                                "cv_share": summ["control_variate_used"] / max(summ["requests"], 1)}},
        "latency_ms": {"p50": summ["p50_ms"], "p99": summ["p99_ms"], "mean": summ["mean_ms"], "max": summ["max_ms"]},
        "served": summ,
        "plain": {"prices_per_s": plain["prices_per_s"], "p50_ms": plain["p50_ms"], "p99_ms": plain["p99_ms"],
                  "requests": plain["requests"], "windows": b["plain_windows"], "paths": plain["paths"],
                  "form": "plain run_mc, one request at a time: pilot K1 + readback, main K1 + readback"},
        "served_capacity": dict(b["capacity"], form="the timed requests released at once (no arrival gaps)"),
        "speedup_vs_plain": {"prices_per_s_e2e": e2e / plain["prices_per_s"],
                             "p50": plain["p50_ms"] / summ["p50_ms"], "p99": plain["p99_ms"] / summ["p99_ms"]},
        "roofline": bind_roofline({"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak,
                     "traffic": (profiled("serve_kernel<6,0,0,1>") or {}).get("dram_bytes"),
                     "traffic_note": "DRAM bytes of one ncu-captured serve_kernel launch (d = 6 main run) of "
                                     "these kernel sources (null when profiles/ holds no capture of them): slot "
                                     "state and chunk partials only; paths stay in registers",
                     "issue_active_ncu": (profiled("serve_kernel<6,0,0,1>") or {}).get("issue_active"),
                     "issue_note": "share of cycles an instruction issued (ncu, profiles/)",
                     "kernel": "serve_kernel (all classes) over the server's device busy time",
                     "flops": "sum over requests of (pilot + main paths) x (steps + jump rate x T) x F(d)",
                     "peak_source": "measured FFMA probe on this GPU (sdemc_fp32_probe)",
                     "mufu": {"achieved": b["mufu"] / busy / 1e12, "peak": mufu_peak, "unit": "Tops/s",
                              "frac": b["mufu"] / busy / 1e12 / mufu_peak,
                              "ops": "sum over requests of paths x (steps x (2d + 1) + 5 x jumps)",
                              "peak_source": "measured rsqrt.approx probe (sdemc_mufu_probe)"}}),
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": b["delta"]["h2d_bytes"] / args.steps,
                "d2h_bytes_per_step": b["delta"]["d2h_bytes"] / args.steps},
        "gpu_launches": b["delta"]["launches"],
        "server": {"ticks": b["delta"]["ticks"], "busy_s": busy, "wall_s": wall},
    }
    if rank == 0:
        line["clocks"] = clk.summary()
        secs = [s.strip() for s in args.sections.split(",") if s.strip() and s.strip() != "none"]
        if "rainbow" in secs:
            line["rainbow2d_plain"] = _section(bench_rainbow_plain, dev, 20, 5, fp32_peak, mufu_peak)
        if "materialise" in secs:
            peaks = load_json_file("MEASURED_PEAKS.json") or {}
            if peaks.get("hbm_gbs"):
                line["materialised_mode"] = _section(bench_materialise, dev, peaks["hbm_gbs"])
            else:
                line["materialised_mode"] = _section(bench_materialise, dev, HBM_FALLBACK_GBS,
                                                     "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)")
        if "mlmc" in secs:
            line["rainbow2d_mlmc"] = _section(bench_rainbow_mlmc, dev)
        if "mix" in secs:
            line["batched_mix"] = _section(bench_batched_mix, 5, 3)
        if "cv" in secs:
            line["cv_learned"] = _section(bench_cv_learned, dev)
        if "cvserved" in secs:
            line["cv_learned_served"] = _section(bench_cv_learned_served, dev)
        if "accuracy" in secs:
            line["accuracy"] = _section(bench_accuracy, dev, line, b)
        threads = os.cpu_count() or 1
        reqs = cpu_sample()
        spr, paths = cpu_baseline_of(reqs, threads)
        line["cpu_baseline"] = {"value": 1.0 / spr, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "the stream's first %d requests (pilot + main, plain estimator, %d paths "
                                          "simulated, extrapolated to the full counts) on %d threads; the "
                                          "reference arm times the same requests" % (len(reqs), paths, threads),
                                "method": CPU_KIND, "reference_torch": REFERENCE_TORCH_NOTE}
        # the comparison the target is stated in, compact and last (read from the end of the output)
        line["vs_plain"] = dict(line["config"]["vs_plain"])
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
