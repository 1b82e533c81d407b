#!/usr/bin/env python
"""Benchmark: prices/s of the config-2 Levy rainbow at 1e-3 relative error.

Workload (BASELINE config 2, one price = one plain Monte Carlo estimate whose
95% half-width is 1e-3 of the price): 2D call on the max of two Merton assets
with independent per-asset compound-Poisson jumps (rate 1.0 each, log-jumps
N(-0.05, 0.15)), sigma = (0.2, 0.3), Brownian correlation 0.5, r = 0.02, T = 1,
K = 1, 256 jump-adapted Euler steps, float32 state, FP64 cross-block sums.
The path count N of one price comes from a 2^18-path pilot, as the reference's
find_num_trials does (sde_mc/mc.py:418-427).  Inputs are synthetic by
construction (the descriptor is the only input; paths are generated on the
device), so L2 is flushed with a 256 MB write between timed steps.

One step = one price = K1 (fused paths + payoff + chunk sums) + K10 (FP64
reduce) over N fresh paths.  `value` is device time (CUDA events, summed over
the K timed steps); `e2e` calls the public API mc_simple(...) with host objects
every step (descriptor lowering, launch parameters host->device, 48-byte
result device->host, MCStatistics).  `--impl reference` times the CPU
restatement of the reference's algorithm on the host cores.
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
WORKLOAD = ("config-2 2D rainbow (call on max), Merton assets with independent per-asset jumps "
            "(rate 1.0, logN(-0.05,0.15)), sigma (0.2,0.3), rho 0.5, r 0.02, T 1, K 1, 256 jump-adapted steps; "
            "one price = plain MC at 1e-3 relative 95% half-width")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rel", type=float, default=1e-3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-paths", type=int, default=0,
                    help="profiling driver: make three price launches of the workload at this many paths "
                         "and exit (the case ncu captures)")
    return ap.parse_args()


def profile_launches(n):
    import torch
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    for i in range(3):
        r = K.price(lower(solver, payoff, disc, num_paths=n, path_offset=i * n, seed=1))
    torch.cuda.synchronize()
    print(json.dumps({"profile_paths": n, "result": r.cpu().tolist()}))


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


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return {}


def load_profile_traffic():
    p = os.path.join(ROOT, "profiles", "price_kernel_traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return None


def cpu_sample(inst_factory, n_target, budget_s):
    """Time the oracle port (C, all host threads) on a bounded sample of paths."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    n = 4096
    while True:
        inst = inst_factory(n)
        t0 = time.perf_counter()
        oracle.price(inst, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or n >= n_target:
            break
        n = min(n_target, int(n * min(8.0, max(2.0, budget_s / 4 / max(dt, 1e-3)))))
    paths_per_s = n / dt
    return paths_per_s, n, dt, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import torch
    from sde_mc_gb300.lowering import lower
    solver, payoff, disc = make_problem()
    # N for one price: from the pilot statistics the GPU arm uses (same model)
    n_target = int(os.environ.get("SDEMC_BENCH_N", "6200000"))

    def factory(n):
        return lower(solver, payoff, disc, num_paths=n, path_offset=0, seed=1)
    per_step = max(args.cpu_seconds / max(args.steps + args.warmup, 1), 0.5)
    times = []
    n_used = 0
    threads = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        pps, n, dt, threads = cpu_sample(factory, n_target, per_step)
        if i >= args.warmup:
            times.append(n_target / pps)
            n_used = n
    sec_per_price = statistics.mean(times)
    value = 1.0 / sec_per_price
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec_per_price * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "paths_per_price": n_target},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d paths per step timed on %d threads, extrapolated to %d paths per price"
                                       % (n_used, threads, n_target)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


MIX_WORKLOAD = ("config-3 mix: 512 correlated Merton basket calls, d~U{1..8}, steps log-U[32,512], "
                "paths log-U[2^12,2^18], K~U(0.8,1.2), sigma_i~U(0.1,0.4), rate~U(0.5,3), rho 0.3, "
                "logN(-0.1,0.2) jumps; numpy default_rng(0)")


def bench_batched_mix(steps, warmup):
    """Config 3: the whole mix per step, batched (K8, autotuned, CUDA graph)
    against the plain method one request per launch (K1 + K10 each)."""
    import torch
    from sde_mc_gb300 import batch as B
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300 import workloads
    mix = workloads.basket_mix(512)
    n = len(mix)
    offs = [0] * n
    insts = B.lower_mix(mix, offs)
    plan = B.BatchPlan(insts)
    tune = B.autotune(plan, repeats=2)
    steps = max(1, min(steps, 10))
    plan.set_path_offsets([(1 << 40) + m.paths * 0 for m in mix])
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
    # plain: one request per launch, descriptors lowered ahead of time
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
                        "launch": {"block_threads": tune["choice"][0], "side_streams": tune["choice"][1]},
                        "graph": True, "gpu_launches_per_mix": 1 + 1 + len(plan.classes[:plan.header.n_class])},
            "plain_one_per_launch": {"prices_per_s": n / (plain_ms * 1e-3), "ms_per_mix": plain_ms,
                                     "gpu_launches_per_mix": 2 * n},
            "speedup_batched_vs_plain": plain_ms / batched_ms,
            "path_steps_per_mix": work, "batched_path_steps_per_s": work / (batched_ms * 1e-3),
            "status_ok": bool((rows[:, 5] == 0).all())}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_paths:
        return profile_launches(args.profile_paths)
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import ctypes
    import sde_mc_gb300 as sm
    from sde_mc_gb300 import _native as N
    from sde_mc_gb300 import kernels as K
    from sde_mc_gb300.lowering import lower

    solver, payoff, disc = make_problem()
    dev = torch.device("cuda", local)
    lib = N.load()

    # pilot -> paths per price for the target relative error
    pilot = K.price(lower(solver, payoff, disc, num_paths=1 << 18, path_offset=0, seed=7)).cpu().tolist()
    price, var = pilot[3], pilot[4]
    n_target = int(math.ceil((1.96 * math.sqrt(var) / (args.rel * price)) ** 2))
    n_target = (n_target + 127) // 128 * 128

    # mean executed steps per path (jump-adapted grid: 256 + jumps + end steps)
    m = K.materialise(lower(solver, payoff, disc, num_paths=1 << 14, path_offset=1 << 40, seed=7),
                      solver.num_steps + solver.max_jumps, want=("steps",))
    steps_per_path = float(m["steps"].double().mean())
    path_steps = n_target * steps_per_path
    flops = path_steps * algorithmic_flops_per_path_step(2)

    # measured FP32 peak (FFMA chains at full occupancy), best of 5
    sink = torch.zeros(16, dtype=torch.float32, device=dev)
    fl = ctypes.c_double(0.0)
    best = 0.0
    s = N.stream_handle(dev)
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        N.check(lib.sdemc_fp32_probe(4096, N.ptr(sink), 16, ctypes.byref(fl), s), "fp32 probe")
        e1.record()
        torch.cuda.synchronize()
        best = max(best, fl.value / (e0.elapsed_time(e1) * 1e-3))
    fp32_peak_tflops = best / 1e12

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    need = lib.sdemc_price_scratch_bytes(ctypes.byref(lower(solver, payoff, disc, num_paths=n_target)))
    scratch = N.SCRATCH.get(need, dev)
    out = torch.empty(6, dtype=torch.float64, device=dev)
    nch = (n_target + N.CHUNK_PATHS - 1) // N.CHUNK_PATHS
    base = rank * (1 << 44)

    def one_step(i, ev=None):
        inst = lower(solver, payoff, disc, num_paths=n_target, path_offset=base + (i + 1) * n_target, seed=1)
        if ev:
            ev[0].record()
        N.check(lib.sdemc_price_chunks(ctypes.byref(inst), None, N.ptr(scratch), scratch.numel(), None, s), "chunks")
        if ev:
            ev[1].record()
        N.check(lib.sdemc_reduce_chunks(N.ptr(scratch), nch, 3, N.ptr(out), s), "reduce")
        if ev:
            ev[2].record()

    for i in range(args.warmup):
        one_step(i)
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    results = []
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        w0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            one_step(args.warmup + i, evs[i])
            results.append(out.clone())
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    if world > 1:
        dist.barrier()
    k_ms = [e[0].elapsed_time(e[1]) for e in evs]
    r_ms = [e[1].elapsed_time(e[2]) for e in evs]
    step_ms = [a + b for a, b in zip(k_ms, r_ms)]
    total_s = sum(step_ms) * 1e-3
    if world > 1:
        t = torch.tensor([total_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    value = world * args.steps / total_s
    res = [r.cpu().tolist() for r in results]
    for r in res:
        N.status_error(r[5], "bench")
    rel_err = statistics.mean(1.96 * math.sqrt(r[4] / r[2]) / r[3] for r in res)

    # end to end through the public API (host objects in, Python floats out)
    e2e_t = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = sm.mc_simple(n_target, solver, payoff, disc, bs=n_target, payoff_time='adapted')
        if i >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    e2e_value = world * len(e2e_t) / sum(e2e_t) if world == 1 else None
    if world > 1:
        t = torch.tensor([sum(e2e_t)], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_value = world * len(e2e_t) / float(t.item())

    kernel_s = statistics.mean(k_ms) * 1e-3
    achieved = flops / kernel_s / 1e12
    traffic = load_profile_traffic()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "paths_per_price": n_target, "form": "plain",
                   "steps_per_path": steps_per_path, "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "price": statistics.mean(r[3] for r in res), "rel_halfwidth": rel_err,
        "path_steps_per_s": path_steps / kernel_s * world,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak_tflops,
                     "traffic": (traffic["bytes_per_path"] * n_target) if traffic else None,
                     "kernel": "price_kernel<2,diag>", "kernel_ms": kernel_s * 1e3,
                     "flops_per_path_step": algorithmic_flops_per_path_step(2),
                     "peak_source": "measured FFMA probe on this GPU (sdemc_fp32_probe)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ctypes.sizeof(N.SdemcInst),
                "d2h_bytes_per_step": 48},
        "gpu_launches": 2 * args.steps,
        "wall_s": wall,
    }
    if rank == 0:
        line["clocks"] = clk.summary()
        line["batched_mix"] = bench_batched_mix(args.steps, args.warmup)
        from sde_mc_gb300.lowering import lower as lw

        def factory(n):
            return lw(solver, payoff, disc, num_paths=n, path_offset=0, seed=1)
        pps, n, dt, threads = cpu_sample(factory, n_target, args.cpu_seconds)
        line["cpu_baseline"] = {"value": pps / n_target, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d paths in %.2f s on %d threads, extrapolated to %d paths per price"
                                          % (n, dt, threads, n_target)}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
