"""Served-stream workload (config 5) and its two servers.

Requests arrive as a Poisson process (exponential gaps from numpy's
default_rng(seed)); each is a config-3 basket instance (d ~ U{1..8}, steps
log-U[32, 512], pilot paths = the instance's path count log-U[2^12, 2^18],
K ~ U(0.8, 1.2), sigma_i ~ U(0.1, 0.4), jump rate ~ U(0.5, 3)) with a target
relative error drawn from {1e-2, 3e-3, 1e-3}.  A request is one run_mc
(sde_mc/mc.py:418-440): pilot, then a main run sized for a 95% half-width of
target x |price|.

* :func:`run_served` feeds the stream to the continuous-batching server
  (:class:`sde_mc_gb300.serve.Server`) from a submitter thread that releases
  each request at its arrival time.
* :func:`run_plain` serves the same stream with the plain method one request
  at a time: pilot launch, readback, main launch, readback (K1 + K10 each).
Both return per-request latencies (arrival -> result) and the throughput.
"""
import math
import threading
import time

import numpy as np

from . import kernels as K
from . import workloads
from .lowering import lower

TARGETS = (1e-2, 3e-3, 1e-3)


class StreamRequest:
    def __init__(self, idx, t, inst, target):
        self.idx, self.t, self.inst, self.target = idx, float(t), inst, float(target)


def make_stream(rate=2000.0, seconds=60.0, seed=1, max_requests=None):
    """Arrival times and requests of the served stream (deterministic)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds or (max_requests is not None and len(out) >= max_requests):
            break
        params = workloads.draw_basket_params(rng)
        target = TARGETS[int(rng.integers(0, len(TARGETS)))]
        m = workloads.basket_instance(len(out), *params)
        out.append(StreamRequest(len(out), t, m, target))
    return out


def _percentiles(lat):
    a = np.sort(np.asarray(lat))
    return {"p50_ms": float(np.percentile(a, 50) * 1e3), "p99_ms": float(np.percentile(a, 99) * 1e3),
            "mean_ms": float(a.mean() * 1e3), "max_ms": float(a.max() * 1e3)}


def run_served(stream, server, estimator="linear_cv", cv_max_dim=8, timeout=1800.0):
    """Release the stream into ``server`` at its arrival times; returns
    (results by request index, summary)."""
    t0 = time.monotonic_ns() + int(5e6)
    err = []

    def submitter():
        try:
            for r in stream:
                delay = t0 + int(r.t * 1e9) - time.monotonic_ns()
                if delay > 0:
                    time.sleep(delay * 1e-9)
                m = r.inst
                est = estimator if m.dim <= cv_max_dim else "plain"
                server.submit(m.solver, m.payoff, m.discounter, rel_target=r.target, pilot_paths=m.paths,
                              estimator=est, tag=r.idx, stream_id=r.idx)
        except Exception as e:  # surfaced by the caller
            err.append(e)

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    res = {}
    t_end = time.monotonic() + timeout
    while len(res) < len(stream):
        if err:
            raise err[0]
        if time.monotonic() > t_end:
            raise TimeoutError("served stream: %d of %d results" % (len(res), len(stream)))
        for r in server.poll(4096, wait=0.05):
            res[r.tag] = r
    th.join()
    lat = [res[r.idx].latency_s for r in stream]
    first = t0
    last = max(r.t_done_ns for r in res.values())
    span = (last - first) * 1e-9
    summ = {"requests": len(stream), "seconds": span, "prices_per_s": len(stream) / span,
            "failed": sum(1 for r in res.values() if r.status != 0),
            "linear_cv_used": sum(1 for r in res.values() if r.estimator == 1),
            "mean_vrf_cv": float(np.mean([r.vrf for r in res.values() if r.estimator == 1] or [1.0])),
            "paths": int(sum(r.pilot_paths + r.main_paths for r in res.values()))}
    summ.update(_percentiles(lat))
    return res, summ


def run_plain(stream, device=None):
    """The plain method, one request at a time in arrival order (FIFO):
    pilot K1 launch + readback, main K1 launch + readback."""
    import torch
    t0 = time.monotonic_ns() + int(5e6)
    out = {}
    lat = []
    for r in stream:
        arrive = t0 + int(r.t * 1e9)
        now = time.monotonic_ns()
        if now < arrive:
            time.sleep((arrive - now) * 1e-9)
        m = r.inst
        n0 = m.paths
        pil = K.price(lower(m.solver, m.payoff, m.discounter, num_paths=n0, path_offset=0, stream_id=r.idx))
        p = pil.cpu().tolist()
        mean0, var0 = p[3], p[4]
        eps = r.target * abs(mean0)
        n = max(64, math.ceil(1.96 ** 2 * var0 / eps ** 2)) if var0 > 0 and eps > 0 else 0
        if n > 0:
            main = K.price(lower(m.solver, m.payoff, m.discounter, num_paths=n, path_offset=n0, stream_id=r.idx))
            q = main.cpu().tolist()
            out[r.idx] = (q[3], math.sqrt(q[4] / q[2]), n)
        else:
            out[r.idx] = (mean0, 0.0, 0)
        lat.append((time.monotonic_ns() - arrive) * 1e-9)
    torch.cuda.synchronize()
    span = (time.monotonic_ns() - t0) * 1e-9
    summ = {"requests": len(stream), "seconds": span, "prices_per_s": len(stream) / span,
            "paths": int(sum(r.inst.paths + out[r.idx][2] for r in stream))}
    summ.update(_percentiles(lat))
    return out, summ
