"""The served-stream workload and its two GPU servers.

Requests arrive as a Poisson process (exponential gaps from numpy's
default_rng(seed)); each is a basket call from the mix law (d ~ U{1..8}, steps
log-U[32, 512], pilot paths = the instance's path count log-U[2^12, 2^18],
K ~ U(0.8, 1.2), sigma_i ~ U(0.1, 0.4), jump rate ~ U(0.5, 3), rho = 0.3,
log-jumps N(-0.1, 0.2), S0 = 1, r = 0.02, T = 1) with a target relative
error drawn from {1e-2, 3e-3, 1e-3}.  A request is one run_mc
(sde_mc/mc.py:418-440): pilot, then a main run sized for a 95% half-width of
target x |price|.  Request i prices on RNG stream i.

* :func:`run_served` feeds the stream to the continuous-batching server
  (:class:`sde_mc_gb300.serve.Server`) from a submitter thread that releases
  each request at its arrival time.
* :func:`run_plain` serves the same stream with the plain method one request
  at a time: pilot launch, readback, main launch, readback (K1 + K10 each).
Both return per-request results, latencies (arrival -> result) and the
throughput.
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
    """One request: arrival time ``t`` (s), its pilot descriptor ``inst``
    (num_paths = pilot paths, stream_id = idx), its relative target and the
    mix-law parameters it was drawn with (``params``, as
    workloads.basket_instance takes them)."""

    __slots__ = ("idx", "t", "inst", "target", "dim", "steps", "rate", "params")

    def __init__(self, idx, t, inst, target, params=None):
        self.idx, self.t, self.inst, self.target = idx, float(t), inst, float(target)
        self.dim, self.steps, self.rate = int(inst.dim), int(inst.num_steps), float(inst.rate)
        self.params = params

    def instance(self, device="cuda"):
        """The request's model objects (a workloads.MixInstance)."""
        return workloads.basket_instance(self.idx, *self.params, device=device)

    def phase(self, num_paths, path_offset):
        """Descriptor of num_paths paths starting at local index path_offset."""
        c = self.inst.copy()
        c.num_paths = int(num_paths)
        c.path_offset = int(path_offset)
        return c

    @property
    def path_steps(self):
        """Expected executed steps of one path (nominal steps plus jumps)."""
        return self.steps + self.rate * float(self.inst.T)


def make_stream(rate=2000.0, seconds=60.0, seed=1, t_begin=0.0):
    """Requests of the stream arriving in [t_begin, seconds), in arrival order
    (times relative to t_begin); deterministic for a given seed."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    idx = 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        params = workloads.draw_basket_params(rng)
        target = TARGETS[int(rng.integers(0, len(TARGETS)))]
        if t >= t_begin:
            m = workloads.basket_instance(idx, *params)
            inst = lower(m.solver, m.payoff, m.discounter, num_paths=m.paths, path_offset=0, stream_id=idx)
            out.append(StreamRequest(idx, t - t_begin, inst, target, params))
        idx += 1
    return out


def _percentiles(lat):
    a = np.sort(np.asarray(lat, dtype=np.float64))
    return {"p50_ms": float(np.percentile(a, 50) * 1e3), "p99_ms": float(np.percentile(a, 99) * 1e3),
            "mean_ms": float(a.mean() * 1e3), "max_ms": float(a.max() * 1e3)}


def run_served(stream, server, estimator="linear_cv", timeout=1800.0):
    """Release the stream into ``server`` at its arrival times and collect the
    results; returns (results by request index, summary)."""
    t0 = time.monotonic_ns() + int(5e6)
    err = []

    def submitter():
        try:
            for r in stream:
                delay = t0 + int(r.t * 1e9) - time.monotonic_ns()
                if delay > 0:
                    time.sleep(delay * 1e-9)
                server.submit_inst(r.inst, r.target, estimator=estimator, tag=r.idx)
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
    last = max(r.t_done_ns for r in res.values())
    span = (last - t0) * 1e-9
    cv = [r for r in res.values() if r.estimator == 1]
    summ = {"requests": len(stream), "seconds": span, "prices_per_s": len(stream) / span,
            "failed": sum(1 for r in res.values() if r.status != 0),
            "control_variate_used": len(cv),
            "vrf_median": float(np.median([r.vrf for r in cv])) if cv else 1.0,
            "paths": int(sum(r.pilot_paths + r.main_paths for r in res.values()))}
    summ.update(_percentiles(lat))
    return res, summ


def run_plain(stream):
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
        n0 = int(r.inst.num_paths)
        p = K.price(r.phase(n0, 0)).cpu().tolist()
        mean0, var0 = p[3], p[4]
        eps = r.target * abs(mean0)
        n = max(64, math.ceil(1.96 ** 2 * var0 / eps ** 2)) if var0 > 0 and eps > 0 else 0
        if n > 0:
            q = K.price(r.phase(n, n0)).cpu().tolist()
            out[r.idx] = (q[3], math.sqrt(q[4] / q[2]), n)
        else:
            out[r.idx] = (mean0, 0.0, 0)
        lat.append((time.monotonic_ns() - arrive) * 1e-9)
    torch.cuda.synchronize()
    span = (time.monotonic_ns() - t0) * 1e-9
    summ = {"requests": len(stream), "seconds": span, "prices_per_s": len(stream) / span,
            "paths": int(sum(int(r.inst.num_paths) + out[r.idx][2] for r in stream)),
            "gpu_launches": 2 * sum(2 if out[r.idx][2] else 1 for r in stream)}
    summ.update(_percentiles(lat))
    return out, summ

