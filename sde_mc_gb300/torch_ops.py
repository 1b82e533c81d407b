"""The C ABI as torch ops: ``torch.ops.sdemc.*``.

Each op validates device, dtype and contiguity of its tensor arguments,
launches on the current CUDA stream through :mod:`sde_mc_gb300.kernels` /
the ctypes binding, and returns CUDA tensors without synchronising.  A
descriptor travels as a CPU ``uint8`` tensor holding the bytes of one
``sdemc_inst`` (:func:`inst_tensor`).  Ops:

* ``sdemc::price(inst, block_threads)`` -> f64[6] (sum, sum_sq, n, mean, var, status)
  — K1 + K10, ``mc_simple``'s batched loop (sde_mc/mc.py:101-123).
* ``sdemc::mlmc_level(inst, fine, coarse, h_fine, h_coarse)`` -> f64[8] — K2,
  one level of ``mc_multilevel`` (sde_mc/mlmc.py:57-69).
* ``sdemc::cv_forward(params, time, paths, normals, payoffs, index, rate)`` ->
  f32[n] Gamma — K5, ``apply_adapted_control_variates`` (sde_mc/varred.py:98-131).
* ``sdemc::cv_backward(params, time, paths, normals, gamma, index, rate)`` ->
  f32[nparams] gradient of Var(Gamma) — K6 (sde_mc/varred.py:160-180).
* ``sdemc::adam_step(params!, grad, m!, v!, step, lr, beta1, beta2, eps)`` — one
  torch.optim.Adam step in place.
* ``sdemc::philox(seed, stream_id, tag, path, first_block, nblocks)`` -> i32[nblocks, 4].
* ``sdemc::price_f64(inst)`` -> f64[6] — K11, the FP64 run on the same paths.
* ``sdemc::materialise(inst, steps_cap)`` -> (paths, left, time, jumps, normals,
  payoffs, steps, status) — K4, ``solve`` with storage (sde_mc/solvers.py:150-226).
* ``sdemc::replay(inst, dw, jump_times, marks, asset)`` -> (paths, left, time,
  jumps, payoffs, steps, status) — K3, the loop on recorded draws.
* ``sdemc::cv_backward_tc(...)`` — K6 on tcgen05, arguments as ``cv_backward``.
* ``sdemc::price_cv(inst, params, disc_rate)`` -> f64[8] — K7, ``mc_apply_cvs``
  for a trained network (sde_mc/mc.py:214-243).
"""
import ctypes
from typing import Optional, Tuple

import torch

from . import _native as N
from . import kernels as K


def inst_tensor(inst):
    """The bytes of a lowered descriptor as a CPU uint8 tensor (op argument)."""
    return torch.frombuffer(bytearray(inst.to_bytes()), dtype=torch.uint8).clone()


def _inst(t):
    if t.device.type != "cpu" or t.dtype != torch.uint8 or t.numel() != ctypes.sizeof(N.SdemcInst):
        raise ValueError("inst must be a CPU uint8 tensor of %d bytes (sdemc_inst)" % ctypes.sizeof(N.SdemcInst))
    inst = N.SdemcInst()
    ctypes.memmove(ctypes.byref(inst), t.contiguous().data_ptr(), ctypes.sizeof(N.SdemcInst))
    return inst


def _check(t, name, dtype, ndim=None):
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % name)
    if t.dtype != dtype:
        raise ValueError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if ndim is not None and t.dim() != ndim:
        raise ValueError("%s must have %d dimensions" % (name, ndim))


@torch.library.custom_op("sdemc::price", mutates_args=())
def price(inst: torch.Tensor, block_threads: int = 0) -> torch.Tensor:
    I = _inst(inst)
    cfg = N.SdemcCfg(block_threads=int(block_threads)) if block_threads else None
    return K.price(I, cfg=cfg)


@price.register_fake
def _(inst, block_threads=0):
    return torch.empty(6, dtype=torch.float64, device="cuda")


@torch.library.custom_op("sdemc::mlmc_level", mutates_args=())
def mlmc_level(inst: torch.Tensor, fine: int, coarse: int, h_fine: float, h_coarse: float) -> torch.Tensor:
    return K.mlmc_level(_inst(inst), fine, coarse, h_fine, h_coarse)


@mlmc_level.register_fake
def _(inst, fine, coarse, h_fine, h_coarse):
    return torch.empty(8, dtype=torch.float64, device="cuda")


def _cv_args(params, time, paths, normals, index):
    _check(params, "params", torch.float32, 1)
    _check(time, "time", torch.float32, 2)
    _check(paths, "paths", torch.float32, 3)
    _check(normals, "normals", torch.float32, 3)
    n_all, s1 = time.shape
    d = int(normals.shape[2])
    if paths.shape != (n_all, s1, d) or normals.shape != (n_all, s1 - 1, d):
        raise ValueError("expected time (N, S+1), paths (N, S+1, d), normals (N, S, d)")
    if params.numel() != N.load().sdemc_cv_nparams(d):
        raise ValueError("params must hold sdemc_cv_nparams(%d) values" % d)
    if index is not None:
        _check(index, "index", torch.int64, 1)
    return d, s1 - 1, (int(index.numel()) if index is not None else n_all)


@torch.library.custom_op("sdemc::cv_forward", mutates_args=())
def cv_forward(params: torch.Tensor, time: torch.Tensor, paths: torch.Tensor, normals: torch.Tensor,
               payoffs: torch.Tensor, index: Optional[torch.Tensor], rate: float) -> torch.Tensor:
    d, S, n = _cv_args(params, time, paths, normals, index)
    _check(payoffs, "payoffs", torch.float32, 1)
    gamma = torch.empty(n, dtype=torch.float32, device=params.device)
    rc = N.load().sdemc_cv_forward(d, N.ptr(params), N.ptr(time), N.ptr(paths), N.ptr(normals), N.ptr(payoffs),
                                   N.ptr(index), n, S, float(rate), N.ptr(gamma), None,
                                   N.stream_handle(params.device))
    N.check(rc, "sdemc_cv_forward")
    return gamma


@cv_forward.register_fake
def _(params, time, paths, normals, payoffs, index, rate):
    n = index.numel() if index is not None else time.shape[0]
    return params.new_empty(n)


def _sms():
    v = ctypes.c_int(0)
    N.check(N.load().sdemc_device_sms(ctypes.byref(v)), "sdemc_device_sms")
    return v.value


@torch.library.custom_op("sdemc::cv_backward", mutates_args=())
def cv_backward(params: torch.Tensor, time: torch.Tensor, paths: torch.Tensor, normals: torch.Tensor,
                gamma: torch.Tensor, index: Optional[torch.Tensor], rate: float) -> torch.Tensor:
    d, S, n = _cv_args(params, time, paths, normals, index)
    _check(gamma, "gamma", torch.float32, 1)
    if gamma.numel() != n:
        raise ValueError("gamma must hold one value per selected path")
    nparts = 2 * _sms()
    partials = torch.empty((nparts, params.numel()), dtype=torch.float32, device=params.device)
    grad = torch.empty_like(params)
    rc = N.load().sdemc_cv_backward(d, N.ptr(params), N.ptr(time), N.ptr(paths), N.ptr(normals), N.ptr(index), n,
                                    S, float(rate), N.ptr(gamma), N.ptr(partials), nparts, N.ptr(grad),
                                    N.stream_handle(params.device))
    N.check(rc, "sdemc_cv_backward")
    return grad


@cv_backward.register_fake
def _(params, time, paths, normals, gamma, index, rate):
    return torch.empty_like(params)


@torch.library.custom_op("sdemc::adam_step", mutates_args=("params", "m", "v"))
def adam_step(params: torch.Tensor, grad: torch.Tensor, m: torch.Tensor, v: torch.Tensor, step: int, lr: float,
              beta1: float, beta2: float, eps: float) -> None:
    for t, name in ((params, "params"), (grad, "grad"), (m, "m"), (v, "v")):
        _check(t, name, torch.float32, 1)
        if t.numel() != params.numel():
            raise ValueError("%s must match params" % name)
    rc = N.load().sdemc_adam_step(N.ptr(params), N.ptr(grad), N.ptr(m), N.ptr(v), params.numel(), int(step),
                                  float(lr), float(beta1), float(beta2), float(eps), N.stream_handle(params.device))
    N.check(rc, "sdemc_adam_step")


@torch.library.custom_op("sdemc::philox", mutates_args=())
def philox(seed: int, stream_id: int, tag: int, path: int, first_block: int, nblocks: int) -> torch.Tensor:
    return K.philox(seed, stream_id, tag, path, first_block, nblocks)


@philox.register_fake
def _(seed, stream_id, tag, path, first_block, nblocks):
    return torch.empty((nblocks, 4), dtype=torch.int32, device="cuda")


@torch.library.custom_op("sdemc::price_f64", mutates_args=())
def price_f64(inst: torch.Tensor) -> torch.Tensor:
    return K.price_f64(_inst(inst))


@price_f64.register_fake
def _(inst):
    return torch.empty(6, dtype=torch.float64, device="cuda")


_STORE = ("paths", "left", "time", "jumps", "normals", "payoffs", "steps", "status")
_T8 = Tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor,
            torch.Tensor]


@torch.library.custom_op("sdemc::materialise", mutates_args=())
def materialise(inst: torch.Tensor, steps_cap: int) -> _T8:
    out = K.materialise(_inst(inst), int(steps_cap))
    return tuple(out[k] for k in _STORE)


def _store_fakes(I, S, n):
    d = int(I.dim)
    nw = 1 if I.noise == N.NOISE_DIAG else 2
    f = dict(dtype=torch.float32, device="cuda")
    return (torch.empty((n, S + 1, d), **f), torch.empty((n, S + 1, d), **f), torch.empty((n, S + 1), **f),
            torch.empty((n, S + 1, d), **f), torch.empty((n, S, d) if nw == 1 else (n, S, d, 2), **f),
            torch.empty(n, **f), torch.empty(n, dtype=torch.int32, device="cuda"),
            torch.empty(1, dtype=torch.int32, device="cuda"))


@materialise.register_fake
def _(inst, steps_cap):
    I = _inst(inst)
    return _store_fakes(I, int(steps_cap), int(I.num_paths))


@torch.library.custom_op("sdemc::replay", mutates_args=())
def replay(inst: torch.Tensor, dw: torch.Tensor, jump_times: Optional[torch.Tensor], marks: Optional[torch.Tensor],
           asset: Optional[torch.Tensor]) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor,
                                                   torch.Tensor, torch.Tensor, torch.Tensor]:
    _check(dw, "dw", torch.float32)
    out = K.replay(_inst(inst), dw, jump_times, marks, asset)
    return tuple(out[k] for k in ("paths", "left", "time", "jumps", "payoffs", "steps", "status"))


@replay.register_fake
def _(inst, dw, jump_times, marks, asset):
    I = _inst(inst)
    bs, S = int(dw.shape[0]), int(dw.shape[1])
    p, l, t, j, _, pay, st, stat = _store_fakes(I, S, bs)
    return p, l, t, j, pay, st, stat


@torch.library.custom_op("sdemc::cv_backward_tc", mutates_args=())
def cv_backward_tc(params: torch.Tensor, time: torch.Tensor, paths: torch.Tensor, normals: torch.Tensor,
                   gamma: torch.Tensor, index: Optional[torch.Tensor], rate: float) -> torch.Tensor:
    d, S, n = _cv_args(params, time, paths, normals, index)
    _check(gamma, "gamma", torch.float32, 1)
    if gamma.numel() != n:
        raise ValueError("gamma must hold one value per selected path")
    nparts = 2 * _sms()
    partials = torch.empty((nparts, params.numel()), dtype=torch.float32, device=params.device)
    grad = torch.empty_like(params)
    status = torch.zeros(1, dtype=torch.int32, device=params.device)
    rc = N.load().sdemc_cv_backward_tc(d, N.ptr(params), N.ptr(time), N.ptr(paths), N.ptr(normals), N.ptr(index),
                                       n, S, float(rate), N.ptr(gamma), N.ptr(partials), nparts, N.ptr(grad),
                                       N.ptr(status), N.stream_handle(params.device))
    N.check(rc, "sdemc_cv_backward_tc")
    return grad


@cv_backward_tc.register_fake
def _(params, time, paths, normals, gamma, index, rate):
    return torch.empty_like(params)


@torch.library.custom_op("sdemc::price_cv", mutates_args=())
def price_cv(inst: torch.Tensor, params: torch.Tensor, disc_rate: float) -> torch.Tensor:
    _check(params, "params", torch.float32, 1)
    return K.price_cv(_inst(inst), params, float(disc_rate))


@price_cv.register_fake
def _(inst, params, disc_rate):
    return torch.empty(8, dtype=torch.float64, device="cuda")


OPS = ("price", "price_f64", "mlmc_level", "materialise", "replay", "cv_forward", "cv_backward", "cv_backward_tc",
       "price_cv", "adam_step", "philox")
