"""Batched heterogeneous pricing (K8): many instances, one planned pass.

``BatchPlan`` turns a list of lowered descriptors into the library's plan
blob (classes of equal dimension, cost-ordered), keeps it in pinned host
memory plus a device copy, owns the scratch and the (n, 6) FP64 result rows,
and launches with ``sdemc_price_batch``.  Because the blob lives in pinned
memory and the upload is a plain stream copy, a whole step (upload + class
kernels + reduction) can be captured once in a CUDA graph and replayed after
editing path offsets in place (:meth:`BatchPlan.set_path_offsets`).

``autotune`` is the project's launch-shape tuner: it times the plan under a
few CTA sizes and side-stream counts, then chooses one or two paths per lane
for each class, and caches the winner per batch signature (a JSON file under ``$SDEMC_CACHE_DIR``, default
``~/.cache/sde_mc_gb300``).
"""
import ctypes
import hashlib
import json
import os

import torch

from . import _native as N


class BatchHeader(ctypes.Structure):
    _fields_ = [("n_inst", ctypes.c_int32), ("n_class", ctypes.c_int32), ("total_chunks", ctypes.c_int64),
                ("total_groups", ctypes.c_int64), ("off_classes", ctypes.c_int64), ("off_insts", ctypes.c_int64),
                ("off_order", ctypes.c_int64), ("off_chunk_prefix", ctypes.c_int64),
                ("off_group_prefix", ctypes.c_int64)]


class BatchClass(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("noise", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("count", ctypes.c_int32), ("first", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("chunk_begin", ctypes.c_int64), ("chunk_end", ctypes.c_int64)]


class BatchPlan:
    def __init__(self, insts, device=None):
        self.device = N.require_cuda(device)
        lib = N.load()
        n = len(insts)
        self.n = n
        arr = (N.SdemcInst * max(n, 1))(*insts)
        nbytes = lib.sdemc_batch_plan_bytes(n)
        self.h_blob = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        N.check(lib.sdemc_batch_plan(ctypes.cast(arr, ctypes.c_void_p), n, N.ptr(self.h_blob), nbytes),
                "sdemc_batch_plan")
        self.header = BatchHeader.from_address(self.h_blob.data_ptr())
        self.d_blob = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.scratch = torch.zeros(lib.sdemc_batch_scratch_bytes(N.ptr(self.h_blob)), dtype=torch.uint8,
                                   device=self.device)
        self.out = torch.empty((max(n, 1), 6), dtype=torch.float64, device=self.device)
        base = self.h_blob.data_ptr()
        self.classes = (BatchClass * max(self.header.n_class, 1)).from_address(base + self.header.off_classes)
        self.plan_insts = (N.SdemcInst * max(n, 1)).from_address(base + self.header.off_insts)
        self.order = (ctypes.c_int32 * max(n, 1)).from_address(base + self.header.off_order)
        self.cfgs = None
        self.n_side = 0
        self._side = []

    # ------------------------------------------------------------------
    def set_path_offsets(self, offsets):
        """offsets[i] = first global path index of caller instance i."""
        for j in range(self.n):
            self.plan_insts[j].path_offset = int(offsets[self.order[j]])

    def set_config(self, block_threads=0, n_side=0, interleave=None):
        """CTA size and side streams for every class; ``interleave[j]`` = paths
        per lane (1 or 2) of class j."""
        nc = max(self.header.n_class, 1)
        il = [1] * nc if interleave is None else [int(v) for v in interleave]
        if len(il) != nc:
            raise ValueError("interleave needs one entry per class (%d)" % nc)
        self.cfgs = (N.SdemcCfg * nc)(*[N.SdemcCfg(block_threads=block_threads, interleave=il[j])
                                        for j in range(nc)])
        self.interleave = il
        self.n_side = int(n_side)
        while len(self._side) < self.n_side:
            self._side.append(torch.cuda.Stream(device=self.device))

    def upload(self):
        self.d_blob.copy_(self.h_blob, non_blocking=True)

    def launch(self):
        lib = N.load()
        side = None
        if self.n_side:
            side = (ctypes.c_void_p * self.n_side)(*[s.cuda_stream for s in self._side[:self.n_side]])
        rc = lib.sdemc_price_batch(N.ptr(self.h_blob), N.ptr(self.d_blob), N.ptr(self.scratch), self.scratch.numel(),
                                   N.ptr(self.out), ctypes.cast(self.cfgs, ctypes.c_void_p) if self.cfgs is not None else None,
                                   ctypes.cast(side, ctypes.c_void_p) if side is not None else None, self.n_side,
                                   N.stream_handle(self.device))
        N.check(rc, "sdemc_price_batch")
        return self.out[:self.n]

    def run(self):
        """Upload the blob and launch; returns the (n, 6) result rows (async)."""
        self.upload()
        return self.launch()

    def signature(self):
        parts = ["%d:%d:%d:%d" % (c.dim, c.noise, c.mode, (c.chunk_end - c.chunk_begin).bit_length())
                 for c in self.classes[:self.header.n_class]]
        return hashlib.sha1(",".join(parts).encode()).hexdigest()[:16]


def _cache_path():
    root = os.environ.get("SDEMC_CACHE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "sde_mc_gb300"))
    return os.path.join(root, "autotune.json")


def _load_cache():
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(cache):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path + ".tmp", "w") as fh:
            json.dump(cache, fh, indent=1)
        os.replace(path + ".tmp", path)
    except OSError:
        pass


CANDIDATES = [(128, 0), (64, 0), (256, 0), (128, 4), (128, 8), (64, 8)]


def autotune(plan, candidates=CANDIDATES, repeats=2, use_cache=True):
    """Pick the launch shape for this plan: ``sdemc_batch_autotune`` times
    every (block_threads, side streams) candidate with CUDA events, then, class
    by class, two paths per lane instead of one where that makes the whole
    batch >1% faster.  The choice is cached per batch signature."""
    sig = plan.signature()
    cache = _load_cache() if use_cache else {}
    nc = max(plan.header.n_class, 1)
    if sig in cache:
        choice = cache[sig]["choice"]
        il = choice[2] if len(choice) > 2 and len(choice[2]) == nc else None
        plan.set_config(choice[0], choice[1], il)
        return cache[sig]
    plan.upload()
    nca = len(candidates)
    bts = (ctypes.c_int32 * nca)(*[c[0] for c in candidates])
    sides = (ctypes.c_int32 * nca)(*[c[1] for c in candidates])
    max_side = max(c[1] for c in candidates)
    plan.set_config(0, max_side)
    streams = (ctypes.c_void_p * max(max_side, 1))(*[s.cuda_stream for s in plan._side[:max_side]])
    cfgs = (N.SdemcCfg * nc)()
    n_side, ms = ctypes.c_int(0), ctypes.c_float(0.0)
    cand_ms = (ctypes.c_float * nca)()
    lib = N.load()
    N.check(lib.sdemc_batch_autotune(N.ptr(plan.h_blob), N.ptr(plan.d_blob), N.ptr(plan.scratch),
                                     plan.scratch.numel(), N.ptr(plan.out), ctypes.cast(bts, ctypes.c_void_p),
                                     ctypes.cast(sides, ctypes.c_void_p), nca,
                                     ctypes.cast(streams, ctypes.c_void_p) if max_side else None, max_side,
                                     int(repeats), ctypes.cast(cfgs, ctypes.c_void_p), ctypes.byref(n_side),
                                     ctypes.byref(ms), ctypes.cast(cand_ms, ctypes.c_void_p),
                                     N.stream_handle(plan.device)), "sdemc_batch_autotune")
    bt = int(cfgs[0].block_threads)
    il = [int(cfgs[j].interleave) for j in range(nc)]
    plan.set_config(bt, n_side.value, il)
    entry = {"choice": [bt, n_side.value, il], "ms": ms.value,
             "tried": sorted([[float(cand_ms[c]), candidates[c][0], candidates[c][1]] for c in range(nca)])}
    if use_cache:
        cache[sig] = entry
        _store_cache(cache)
    return entry


def lower_mix(instances, path_offsets=None, seed=None):
    """Descriptors for a list of workloads.MixInstance (stream id = instance id)."""
    from .lowering import lower
    out = []
    for k, m in enumerate(instances):
        off = 0 if path_offsets is None else path_offsets[k]
        out.append(lower(m.solver, m.payoff, m.discounter, num_paths=m.paths, path_offset=off,
                         stream_id=m.stream_id, seed=seed))
    return out
