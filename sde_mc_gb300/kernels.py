"""Thin typed wrappers over the C ABI: each call takes a lowered instance
descriptor plus torch CUDA tensors and launches on the current stream.

These are the only entry points the estimator modules use; they are also
registered as torch ops (``torch.ops.sdemc.*``) in :mod:`sde_mc_gb300.torch_ops`.
"""
import ctypes

import torch

from . import _native as N


def _dev(device):
    return N.require_cuda(device)


def price(inst, cfg=None, payoffs=None, device=None, out=None):
    """Fused K1 launch.  Returns a float64 CUDA tensor
    (sum, sum_sq, n, mean, var, status) without synchronising."""
    dev = _dev(device)
    lib = N.load()
    need = lib.sdemc_price_scratch_bytes(ctypes.byref(inst))
    scratch = N.SCRATCH.get(need, dev)
    if out is None:
        out = torch.empty(6, dtype=torch.float64, device=dev)
    if payoffs is not None:
        assert payoffs.is_cuda and payoffs.dtype == torch.float32 and payoffs.numel() >= inst.num_paths
    rc = lib.sdemc_price(ctypes.byref(inst), N.byref(cfg), N.ptr(scratch), scratch.numel(), N.ptr(out),
                         N.ptr(payoffs), N.stream_handle(dev))
    N.check(rc, "sdemc_price")
    return out


def price_f64(inst, device=None, out=None):
    """K11, the FP64 reference run on the same paths as :func:`price`.  Returns
    a float64 CUDA tensor (sum, sum_sq, n, mean, var, status)."""
    dev = _dev(device)
    lib = N.load()
    need = lib.sdemc_price_scratch_bytes(ctypes.byref(inst))
    scratch = N.SCRATCH.get(need, dev)
    if out is None:
        out = torch.empty(6, dtype=torch.float64, device=dev)
    rc = lib.sdemc_price_f64(ctypes.byref(inst), N.ptr(scratch), scratch.numel(), N.ptr(out),
                             N.stream_handle(dev))
    N.check(rc, "sdemc_price_f64")
    return out


def mlmc_level(inst, fine, coarse, h_fine, h_coarse, cfg=None, ys=None, device=None, out=None):
    """K2 launch for one level.  Returns float64 CUDA tensor
    (sumY, sumY2, n, sumPf, sumPf2, mean, var, status)."""
    dev = _dev(device)
    lib = N.load()
    need = lib.sdemc_mlmc_scratch_bytes(ctypes.byref(inst))
    scratch = N.SCRATCH.get(need, dev)
    if out is None:
        out = torch.empty(8, dtype=torch.float64, device=dev)
    rc = lib.sdemc_mlmc_level(ctypes.byref(inst), int(fine), int(coarse), float(h_fine), float(h_coarse),
                              N.byref(cfg), N.ptr(scratch), scratch.numel(), N.ptr(out), N.ptr(ys),
                              N.stream_handle(dev))
    N.check(rc, "sdemc_mlmc_level")
    return out


def price_cv(inst, params, disc_rate, gamma=None, device=None, out=None):
    """K7: paths + payoff + learned control variate (f on the tensor cores) in
    one launch.  Returns float64 CUDA tensor (sum G, sum G^2, n, sum P,
    sum P^2, mean G, var G, status); ``gamma`` (nullable, float32 (n,))
    receives each path's Gamma."""
    dev = _dev(device)
    lib = N.load()
    need = lib.sdemc_price_cv_scratch_bytes(ctypes.byref(inst))
    scratch = N.SCRATCH.get(need, dev)
    if out is None:
        out = torch.empty(8, dtype=torch.float64, device=dev)
    if gamma is not None:
        assert gamma.is_cuda and gamma.dtype == torch.float32 and gamma.numel() >= inst.num_paths
    rc = lib.sdemc_price_cv(ctypes.byref(inst), N.ptr(params), float(disc_rate), N.ptr(scratch), scratch.numel(),
                            N.ptr(out), N.ptr(gamma), N.stream_handle(dev))
    N.check(rc, "sdemc_price_cv")
    return out


def zdim(dim, noise):
    return dim if noise == N.NOISE_DIAG else (dim + 1 if noise == N.NOISE_INDEP_SHARED else 2 * dim)


def materialise(inst, steps_cap, want=("paths", "left", "time", "jumps", "normals", "payoffs", "steps"),
                export_draws=False, jcap=0, device=None):
    """K4: full storage of num_paths paths at steps_cap columns.  Returns a dict
    of CUDA tensors (plus 'status').  export_draws adds raw normals 'z' and the
    jump stream 'jt', 'jm', 'jsel' (jcap entries per path) for the oracle."""
    dev = _dev(device)
    n, d, S = int(inst.num_paths), int(inst.dim), int(steps_cap)
    nw = 1 if inst.noise == N.NOISE_DIAG else 2
    f32 = dict(dtype=torch.float32, device=dev)
    out = {}
    if "paths" in want:
        out["paths"] = torch.empty((n, S + 1, d), **f32)
    if "left" in want:
        out["left"] = torch.empty((n, S + 1, d), **f32)
    if "time" in want:
        out["time"] = torch.empty((n, S + 1), **f32)
    if "jumps" in want:
        out["jumps"] = torch.empty((n, S + 1, d), **f32)
    if "normals" in want:
        out["normals"] = torch.empty((n, S, d) if nw == 1 else (n, S, d, 2), **f32)
    if "payoffs" in want:
        out["payoffs"] = torch.empty(n, **f32)
    if "steps" in want:
        out["steps"] = torch.empty(n, dtype=torch.int32, device=dev)
    zd = zdim(d, inst.noise)
    if export_draws:
        out["z"] = torch.empty((n, S, zd), **f32)
        if jcap > 0:
            out["jt"] = torch.empty((n, jcap), **f32)
            out["jm"] = torch.empty((n, jcap), **f32)
            out["jsel"] = torch.empty((n, jcap), dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    g = out.get
    rc = N.load().sdemc_materialise(
        ctypes.byref(inst), S, N.ptr(g("paths")), N.ptr(g("left")), N.ptr(g("time")), N.ptr(g("jumps")),
        N.ptr(g("normals")), N.ptr(g("payoffs")), N.ptr(g("steps")), N.ptr(g("z")), zd, N.ptr(g("jt")),
        N.ptr(g("jm")), N.ptr(g("jsel")), int(jcap) if export_draws else 0, N.ptr(status),
        N.stream_handle(dev))
    N.check(rc, "sdemc_materialise")
    out["status"] = status
    return out


def serve_cv_weights(inst):
    """The served control variate's weight parameters for a descriptor (host only)."""
    cw = N.SdemcCvWeights()
    N.check(N.load().sdemc_serve_cv_weights(ctypes.byref(inst), ctypes.byref(cw)), "sdemc_serve_cv_weights")
    return cw


def serve_cv_paths(inst, steps_cap=0, jcap=0, wcap=0, device=None):
    """The served control variate path by path: each path's discounted payoff
    'payoff' (n) and its 2d + 1 regressors 'reg' (n, 2d + 1), exactly as the
    server's kernels compute them.  steps_cap > 0 also exports the raw normals
    'z' (n, steps_cap, d); jcap > 0 the jump stream 'jt', 'jm', 'jsel'; wcap > 0
    the weights 'wg' (n, wcap, 2) of every 4-step block.  Plus 'status'."""
    dev = _dev(device)
    n, d = int(inst.num_paths), int(inst.dim)
    f32 = dict(dtype=torch.float32, device=dev)
    out = {"payoff": torch.empty(n, **f32), "reg": torch.empty((n, 2 * d + 1), **f32)}
    if steps_cap > 0:
        out["z"] = torch.zeros((n, steps_cap, d), **f32)
    if jcap > 0:
        out["jt"] = torch.empty((n, jcap), **f32)
        out["jm"] = torch.empty((n, jcap), **f32)
        out["jsel"] = torch.empty((n, jcap), dtype=torch.int32, device=dev)
    if wcap > 0:
        out["wg"] = torch.zeros((n, wcap, 2), **f32)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    g = out.get
    rc = N.load().sdemc_serve_cv_paths(
        ctypes.byref(inst), int(steps_cap), N.ptr(out["payoff"]), N.ptr(out["reg"]), N.ptr(g("z")),
        N.ptr(g("jt")), N.ptr(g("jm")), N.ptr(g("jsel")), int(jcap), N.ptr(g("wg")), int(wcap), N.ptr(status),
        N.stream_handle(dev))
    N.check(rc, "sdemc_serve_cv_paths")
    out["status"] = status
    return out


def replay(inst, dw, jump_times=None, marks=None, asset=None, device=None):
    """K3: replay recorded draws.  dw (bs, S, d[, 2]); jump_times (bs, MJ);
    marks/asset (bs, S).  Returns dict of paths/left/time/jumps/payoffs/steps/status."""
    dev = _dev(device)
    bs, S = int(dw.shape[0]), int(dw.shape[1])
    d = int(inst.dim)
    f32 = dict(dtype=torch.float32, device=dev)

    def c(t, dt=torch.float32):
        return None if t is None else t.to(device=dev, dtype=dt).contiguous()
    dw, jump_times, marks, asset = c(dw), c(jump_times), c(marks), c(asset, torch.int32)
    out = dict(paths=torch.empty((bs, S + 1, d), **f32), left=torch.empty((bs, S + 1, d), **f32),
               time=torch.empty((bs, S + 1), **f32), jumps=torch.empty((bs, S + 1, d), **f32),
               payoffs=torch.empty(bs, **f32), steps=torch.empty(bs, dtype=torch.int32, device=dev),
               status=torch.zeros(1, dtype=torch.int32, device=dev))
    mj = int(jump_times.shape[1]) if jump_times is not None else 0
    rc = N.load().sdemc_replay(ctypes.byref(inst), bs, S, mj, N.ptr(jump_times), N.ptr(dw), N.ptr(marks),
                               N.ptr(asset), N.ptr(out["paths"]), N.ptr(out["left"]), N.ptr(out["time"]),
                               N.ptr(out["jumps"]), N.ptr(out["payoffs"]), N.ptr(out["steps"]),
                               N.ptr(out["status"]), N.stream_handle(dev))
    N.check(rc, "sdemc_replay")
    return out


def mlmc_paths(inst, fine, coarse, h_fine, h_coarse, cols, normals=False, device=None):
    """K2 with every column multilevel_solve returns: dict of 'paths_fine',
    'paths_coarse', 'steps' (own coarse steps per path), 'status' and, on the
    uniform grid with normals=True, the fine increments 'normals'.  cols =
    (fine columns, coarse columns)."""
    dev = _dev(device)
    n, d = int(inst.num_paths), int(inst.dim)
    cf, cc = int(cols[0]), int(cols[1])
    f32 = dict(dtype=torch.float32, device=dev)
    out = {"paths_fine": torch.empty((n, cf, d), **f32), "paths_coarse": torch.empty((n, cc, d), **f32),
           "steps": torch.zeros(n, dtype=torch.int32, device=dev)}
    if normals and inst.grid == N.GRID_UNIFORM:
        nw = 1 if inst.noise == N.NOISE_DIAG else 2
        out["normals"] = torch.empty((n, int(fine), d) if nw == 1 else (n, int(fine), d, 2), **f32)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = N.load().sdemc_mlmc_paths(ctypes.byref(inst), int(fine), int(coarse), float(h_fine), float(h_coarse), cf, cc,
                                   N.ptr(out["paths_fine"]), N.ptr(out["paths_coarse"]), N.ptr(out.get("normals")),
                                   N.ptr(out["steps"]), N.ptr(status), N.stream_handle(dev))
    N.check(rc, "sdemc_mlmc_paths")
    out["status"] = status
    return out


def mlmc_replay(inst, fine, coarse, h_fine, h_coarse, dw, coarse_cap, jump_times=None, marks=None,
                asset=None, device=None, cols=None):
    """K2 on recorded draws: terminal states 'xf', 'xc' (and with cols = (fine
    columns, coarse columns) also 'paths_fine', 'paths_coarse', 'steps')."""
    dev = _dev(device)
    bs, Sf = int(dw.shape[0]), int(dw.shape[1])
    d = int(inst.dim)

    def c(t, dt=torch.float32):
        return None if t is None else t.to(device=dev, dtype=dt).contiguous()
    dw, jump_times, marks, asset = c(dw), c(jump_times), c(marks), c(asset, torch.int32)
    xf = torch.empty((bs, d), dtype=torch.float32, device=dev)
    xc = torch.empty((bs, d), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    mj = int(jump_times.shape[1]) if jump_times is not None else 0
    if cols is not None:
        cf, cc = int(cols[0]), int(cols[1])
        pf = torch.empty((bs, cf, d), dtype=torch.float32, device=dev)
        pc = torch.empty((bs, cc, d), dtype=torch.float32, device=dev)
        steps = torch.zeros(bs, dtype=torch.int32, device=dev)
        rc = N.load().sdemc_mlmc_replay_paths(ctypes.byref(inst), int(fine), int(coarse), float(h_fine),
                                              float(h_coarse), bs, Sf, int(coarse_cap), mj, N.ptr(jump_times),
                                              N.ptr(dw), N.ptr(marks), N.ptr(asset), cf, cc, N.ptr(pf), N.ptr(pc),
                                              N.ptr(xf), N.ptr(xc), N.ptr(steps), N.ptr(status),
                                              N.stream_handle(dev))
        N.check(rc, "sdemc_mlmc_replay_paths")
        return dict(xf=xf, xc=xc, paths_fine=pf, paths_coarse=pc, steps=steps, status=status)
    rc = N.load().sdemc_mlmc_replay(ctypes.byref(inst), int(fine), int(coarse), float(h_fine),
                                    float(h_coarse), bs, Sf, int(coarse_cap), mj, N.ptr(jump_times),
                                    N.ptr(dw), N.ptr(marks), N.ptr(asset), N.ptr(xf), N.ptr(xc),
                                    N.ptr(status), N.stream_handle(dev))
    N.check(rc, "sdemc_mlmc_replay")
    return dict(xf=xf, xc=xc, status=status)


def philox(seed, stream_id, tag, path, first_block, nblocks, device=None):
    dev = _dev(device)
    out = torch.empty((nblocks, 4), dtype=torch.int32, device=dev)
    rc = N.load().sdemc_philox(int(seed), int(stream_id), int(tag), int(path), int(first_block),
                               int(nblocks), N.ptr(out), N.stream_handle(dev))
    N.check(rc, "sdemc_philox")
    return out
