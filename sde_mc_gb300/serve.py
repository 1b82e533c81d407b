"""Pricing server (K9): continuous batching of run_mc requests on one GPU.

A request is what the reference's ``run_mc(problem, eps)`` computes
(sde_mc/mc.py:418-440): a pilot of ``pilot_paths`` paths estimates the
payoff's variance, the main run prices ``ceil((1.96 sd / eps)^2)`` fresh paths
with ``eps = rel_target * |pilot price|``.  The server is native: one host
thread inside the library drives the device in ticks, every request lives in
a device-resident slot (descriptor, RNG path counter, FP64 running sums), and
requests arriving while others run are admitted between ticks as slots and
the memory budget allow.  A request's slices depend on the request alone, so
its result is bit-identical whether it ran alone or in any mix.

With ``estimator='linear_cv'`` the pilot also fits, by regression, the
coefficients of 2d + 1 control variates — per asset, the integrals of w X^i
against the Brownian increments and against the compensated jump measure,
with w a Black-Scholes delta of the payoff's underlying, and the integral of
a gamma weight against the compensated measure of squared jumps; all have
mean exactly zero under the Euler scheme — and the main run prices payoff -
beta . r, which needs far fewer paths for the same target.  The plain
estimator stays the fallback when the pilot shows no gain.

Example::

    with Server() as srv:
        srv.submit(solver, Basket(1.0), ConstantShortRate(0.02), rel_target=1e-3,
                   pilot_paths=1 << 14, tag=7)
        (res,) = srv.wait(1)
        print(res.mean, res.se, res.latency_s)
"""
import ctypes
import time

from . import _native as N
from .lowering import lower

EST_PLAIN, EST_LINEAR_CV = 0, 1
SERVE_FIFO, SERVE_SRPT = 0, 1
_ESTIMATORS = {"plain": EST_PLAIN, "linear_cv": EST_LINEAR_CV}
_POLICIES = {"fifo": SERVE_FIFO, "srpt": SERVE_SRPT}


class ServerCfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_slots", ctypes.c_int32), ("mem_budget", ctypes.c_int64),
                ("tick_work", ctypes.c_int64), ("slice_work", ctypes.c_int64), ("block_threads", ctypes.c_int32),
                ("side_streams", ctypes.c_int32), ("policy", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("inst", N.SdemcInst), ("rel_target", ctypes.c_double), ("max_paths", ctypes.c_int64),
                ("tag", ctypes.c_uint64), ("estimator", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("estimator", ctypes.c_int32),
                ("mean", ctypes.c_double), ("se", ctypes.c_double), ("pilot_mean", ctypes.c_double),
                ("pilot_se", ctypes.c_double), ("vrf", ctypes.c_double), ("pilot_paths", ctypes.c_int64),
                ("main_paths", ctypes.c_int64), ("t_arrive_ns", ctypes.c_int64), ("t_admit_ns", ctypes.c_int64),
                ("t_done_ns", ctypes.c_int64), ("beta", ctypes.c_float * (2 * N.MAX_DIM + 1)),
                ("reserved1", ctypes.c_float)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("pending", ctypes.c_int64), ("active", ctypes.c_int64), ("ticks", ctypes.c_int64),
                ("mem_in_use", ctypes.c_int64), ("mem_peak", ctypes.c_int64), ("path_steps", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("busy_s", ctypes.c_double), ("tick_hist", ctypes.c_int64 * 16)]


def struct_sizes():
    """(cfg, request, result, stats) sizes as the library sees them."""
    arr = (ctypes.c_size_t * 4)()
    N.check(N.load().sdemc_serve_sizes(arr, 4), "sdemc_serve_sizes")
    return tuple(arr)


class ServeResult:
    """One finished request.  ``mean``/``se`` are the main run's price and
    standard error; times are CLOCK_MONOTONIC nanoseconds (time.monotonic_ns)."""

    __slots__ = ("tag", "status", "estimator", "mean", "se", "pilot_mean", "pilot_se", "vrf", "pilot_paths",
                 "main_paths", "t_arrive_ns", "t_admit_ns", "t_done_ns", "beta")

    def __init__(self, r):
        for f in self.__slots__:
            v = getattr(r, f)
            setattr(self, f, list(v) if f == "beta" else v)

    @property
    def latency_s(self):
        return (self.t_done_ns - self.t_arrive_ns) * 1e-9

    @property
    def estimator_name(self):
        return "linear_cv" if self.estimator == EST_LINEAR_CV else "plain"

    def raise_for_status(self):
        N.status_error(self.status, "request %d" % self.tag)
        return self

    def key(self):
        """The bits of the estimate (for identity checks)."""
        return (self.status, self.estimator, self.mean, self.se, self.pilot_mean, self.pilot_se, self.main_paths)

    def __repr__(self):
        return "ServeResult(tag=%d, mean=%.6g, se=%.3g, est=%s, vrf=%.2f, paths=%d+%d, latency=%.4fs)" % (
            self.tag, self.mean, self.se, self.estimator_name, self.vrf, self.pilot_paths, self.main_paths,
            self.latency_s)


class Server:
    """Handle of a native pricing server on one CUDA device.

    ``max_slots`` requests are resident at once and ``mem_budget`` bytes hold
    the slot table and the tick buffers' chunk partials (admission waits for
    both).  ``tick_work`` caps a tick's work and ``slice_work`` the work one
    request contributes to a tick, both in path-step x dimension units (0:
    the library's defaults, 2^33 — in effect no cap — and 2^27).  Class kernels run in
    ``block_threads``-thread CTAs spread over ``side_streams`` streams per
    tick; up to four ticks are in flight.  ``policy``: "srpt" (shortest
    remaining work first) or "fifo"."""

    def __init__(self, max_slots=4096, mem_budget=40 << 30, tick_work=0, slice_work=0, block_threads=256,
                 side_streams=8, policy="srpt", device=None):
        dev = N.require_cuda(device)
        self.device = dev
        cfg = ServerCfg(device=dev.index, max_slots=int(max_slots), mem_budget=int(mem_budget),
                        tick_work=int(tick_work), slice_work=int(slice_work), block_threads=int(block_threads),
                        side_streams=int(side_streams), policy=_POLICIES[policy] if isinstance(policy, str) else int(policy))
        lib = N.load()
        sizes = struct_sizes()
        mine = (ctypes.sizeof(ServerCfg), ctypes.sizeof(Request), ctypes.sizeof(Result), ctypes.sizeof(ServerStats))
        if sizes != mine:
            raise RuntimeError("server struct layout mismatch: library %r, binding %r" % (sizes, mine))
        h = ctypes.c_void_p()
        N.check(lib.sdemc_server_create(ctypes.byref(cfg), ctypes.byref(h)), "sdemc_server_create")
        self._h = h
        self.cfg = cfg
        self._next_tag = 1

    # ------------------------------------------------------------------
    def submit_inst(self, inst, rel_target, estimator="linear_cv", tag=None, max_paths=0):
        """Enqueue a lowered descriptor (inst.num_paths = pilot paths).  Returns the tag."""
        if self._h is None:
            raise RuntimeError("server is closed")
        if tag is None:
            tag = self._next_tag
        self._next_tag = max(self._next_tag, int(tag) + 1)
        req = Request(inst=inst, rel_target=float(rel_target), max_paths=int(max_paths), tag=int(tag),
                      estimator=_ESTIMATORS[estimator] if isinstance(estimator, str) else int(estimator))
        N.check(N.load().sdemc_server_admit(self._h, ctypes.byref(req)), "sdemc_server_admit")
        return int(tag)

    def submit(self, solver, payoff, discounter, rel_target, pilot_paths, estimator="linear_cv", tag=None,
               stream_id=None, path_offset=0, seed=None, max_paths=0, payoff_time="adapted"):
        """Enqueue one run_mc request for (solver, payoff, discounter).

        Each request draws from its own RNG stream: ``stream_id`` (default: the
        tag) selects it, pilot paths are local indices [path_offset,
        path_offset + pilot_paths) and the main run continues after them."""
        if tag is None:
            tag = self._next_tag
        sid = int(tag if stream_id is None else stream_id) & 0xFFFFFFFF
        inst = lower(solver, payoff, discounter, num_paths=int(pilot_paths), path_offset=int(path_offset),
                     stream_id=sid, seed=seed)
        if payoff_time == "terminal" and solver.has_jumps:
            inst.flags |= 1  # SDEMC_INST_PAYOFF_AT_NOMINAL_STEP
        return self.submit_inst(inst, rel_target, estimator, tag, max_paths)

    def poll(self, max_results=1024, wait=0.0):
        """Finished results (possibly none); waits up to ``wait`` seconds for one."""
        buf = (Result * max(1, int(max_results)))()
        n = ctypes.c_int(0)
        N.check(N.load().sdemc_server_poll(self._h, ctypes.cast(buf, ctypes.c_void_p), int(max_results),
                                           ctypes.byref(n), int(wait * 1e9)), "sdemc_server_poll")
        return [ServeResult(buf[i]) for i in range(n.value)]

    def wait(self, count, timeout=600.0):
        """Block until ``count`` results arrived (or raise TimeoutError)."""
        out = []
        t_end = time.monotonic() + timeout
        while len(out) < count:
            left = t_end - time.monotonic()
            if left <= 0:
                raise TimeoutError("%d of %d results after %.1f s" % (len(out), count, timeout))
            out += self.poll(count - len(out), wait=min(left, 0.5))
        return out

    def stats(self):
        s = ServerStats()
        N.check(N.load().sdemc_server_stats_get(self._h, ctypes.byref(s)), "sdemc_server_stats_get")
        out = {f: getattr(s, f) for f, _ in ServerStats._fields_}
        out["tick_hist"] = list(out["tick_hist"])
        return out

    def close(self):
        if getattr(self, "_h", None) is not None:
            N.load().sdemc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
