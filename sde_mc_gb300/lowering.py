"""Lower plug-in objects (Sde, solver, Option, discounter) into ``sdemc_inst``.

Known model classes — by class name, so the reference's own objects lower too —
become the affine coefficient form of the kernels:

    dx_i = (a_i + b_i x_i) dt + (s_i + q_i x_i) dW_i [+ (s2_i + q2_i x_i) dW2_i] + (g_i + k_i x_i^-) J

Every float is produced by the same float32 torch expression the reference
evaluates (e.g. Merton's ``mu - rate * jump_mean()``, sde_mc/sde.py:368-369,
the step ``h = T / num_steps``, sde_mc/solvers.py:166), so a replay on the GPU
can match the reference bit for bit.  Unknown classes raise
NotImplementedError: a user Sde's Python methods cannot run inside a kernel.
"""
import math

import numpy as np
import torch

from . import _native as N
from .levy import UNIFORM_TOL

_F32 = torch.float32


def _vec(v, d):
    t = torch.as_tensor(v).detach().to(device='cpu', dtype=_F32).reshape(-1)
    if t.numel() == 1:
        t = t.expand(d)
    if t.numel() != d:
        raise ValueError("coefficient of length %d for dimension %d" % (t.numel(), d))
    return [float(x) for x in t.tolist()]


def _f32(v):
    if torch.is_tensor(v):
        return float(v.detach().to(device='cpu', dtype=_F32).reshape(-1)[0])
    return float(np.float32(v))


def _set(arr, vals):
    for i, v in enumerate(vals):
        arr[i] = v


def _name(obj):
    return type(obj).__name__


def lower_sde(sde, inst):
    """Fill the model part of ``inst`` from an Sde object."""
    d = int(sde.dim)
    if d < 1 or d > N.MAX_DIM:
        raise NotImplementedError("dimension %d: the kernels support 1..%d" % (d, N.MAX_DIM))
    inst.dim = d
    _set(inst.x0, _vec(sde.init_value, d))
    name = _name(sde)
    zero, one = [0.0] * d, [1.0] * d
    inst.noise = N.NOISE_DIAG
    inst.model = N.MODEL_AFFINE
    inst.mark = N.MARK_NONE
    inst.jump_target = N.JUMP_COMMON
    inst.rate = 0.0
    inst.inv_rate = 0.0
    for arr in (inst.drift_a, inst.drift_b, inst.diff_s, inst.diff_q, inst.diff2_s, inst.diff2_q,
                inst.jump_g, inst.jump_k, inst.jump_cdf):
        _set(arr, [0.0] * N.MAX_DIM)

    def jumps_lognormal(rate_total):
        inst.mark = N.MARK_LOGNORMAL
        inst.mark_p[0] = _f32(sde.alpha)
        inst.mark_p[1] = _f32(sde.gamma)
        inst.rate = rate_total
        inst.inv_rate = float(np.float32(1.0) / np.float32(rate_total)) if rate_total > 0 else 0.0

    if name in ("Merton",):
        coef = torch.as_tensor(sde.mu - sde.rate * sde.jump_mean())
        _set(inst.drift_b, _vec(coef, d))
        _set(inst.diff_q, _vec(sde.sigma, d))
        _set(inst.jump_k, one)
        jumps_lognormal(_f32(torch.as_tensor(sde.jump_rate()).sum()))
    elif name == "IndependentJumpsMerton":
        rates = torch.as_tensor(sde.jump_rate(), dtype=_F32).reshape(-1).expand(d)
        coef = torch.as_tensor(sde.mu - rates * sde.jump_mean())
        _set(inst.drift_b, _vec(coef, d))
        _set(inst.diff_q, _vec(sde.sigma, d))
        _set(inst.jump_k, one)
        inst.jump_target = N.JUMP_ONE_ASSET
        cdf = torch.cumsum(rates / rates.sum(), 0)
        cdf[-1] = 1.0
        _set(inst.jump_cdf, [float(v) for v in cdf.tolist()])
        jumps_lognormal(_f32(rates.sum()))
    elif name in ("Gbm",):
        _set(inst.drift_b, _vec(sde.mu, d))
        _set(inst.diff_q, _vec(sde.sigma, d))
    elif name == "LogGbm":
        _set(inst.drift_a, _vec(sde.drift(0.0, torch.zeros(1, d)).reshape(-1), d))
        _set(inst.diff_s, _vec(sde.diffusion(0.0, torch.zeros(1, d)).reshape(-1), d))
    elif name == "DoubleGbm":
        inst.noise = N.NOISE_INDEP_PAIR
        _set(inst.drift_b, _vec(sde.mu, d))
        _set(inst.diff_q, _vec(sde.sigma1, d))
        _set(inst.diff2_q, _vec(sde.sigma2, d))
    elif name == "LevySde":
        lower_levy(sde, inst, d)
    elif name == "Heston":
        # sde_mc/sde.py:258-279: drift (r S, 0), diffusion (sqrt(v) S, 0) and
        # the quadratic's coefficients as torch forms them from Python floats:
        # kappa*h, (kappa*theta)*h, xi*dW, (0.5*h)*(xi**2)
        inst.model = N.MODEL_HESTON
        _set(inst.drift_b, [_f32(sde.r), 0.0])
        k, th, xi = float(sde.kappa), float(sde.theta), float(sde.xi)
        _set(inst.mark_p, [_f32(k), _f32(k * th), _f32(xi), _f32(xi ** 2)] + [0.0] * (N.MARK_PARAMS - 4))
    elif name == "AsianWrapper":
        # sde_mc/sde.py:378-406: a 1-D model in component 0, its time
        # integral in component 1 (no diffusion, no jumps)
        base = sde.base_sde
        if int(base.dim) != 1:
            raise NotImplementedError("AsianWrapper lowers around a 1-D model only")
        sub = lower_sde(base, N.SdemcInst())
        if sub.model != N.MODEL_AFFINE or sub.noise != N.NOISE_DIAG:
            raise NotImplementedError("AsianWrapper lowers around an affine 'diag' model only")
        for f in ("drift_a", "drift_b", "diff_s", "diff_q", "jump_g", "jump_k"):
            getattr(inst, f)[0] = getattr(sub, f)[0]
        inst.mark, inst.rate, inst.inv_rate = sub.mark, sub.rate, sub.inv_rate
        _set(inst.mark_p, list(sub.mark_p))
        inst.model = N.MODEL_ASIAN
    else:
        raise NotImplementedError(
            "no GPU lowering for Sde class %r (supported: Merton, IndependentJumpsMerton, Gbm, LogGbm, "
            "DoubleGbm, Heston, AsianWrapper, LevySde over ExpExampleLevy/ExampleLevy/Levy2d)" % name)
    return inst


def lower_levy(sde, inst, d):
    lev = sde.levy
    lname = _name(lev)
    inst.noise = N.NOISE_INDEP_SHARED
    gam, beta = float(lev.gamma()), float(lev.beta())
    if lname == "ExpExampleLevy":
        # drift r x - (f x) gamma, diffusion [sigma x, (f x) beta], jumps f x J
        f = _vec(lev.f, d)
        _set(inst.drift_b, [float(np.float32(np.float32(r) - np.float32(fi) * np.float32(gam)))
                            for r, fi in zip(_vec(lev.r, d), f)])
        _set(inst.diff_q, _vec(lev.sigma, d))
        _set(inst.diff2_q, [float(np.float32(fi) * np.float32(beta)) for fi in f])
        _set(inst.jump_k, f)
    elif lname in ("ExampleLevy", "Levy2d"):
        # additive: drift a - f gamma, diffusion [sigma, f beta], jumps f J
        x1 = torch.ones(1, d)
        base = lev.drift(0.0, x1).reshape(-1)
        f = _vec(lev.jumps(0.0, x1, 1).reshape(-1), d)
        _set(inst.drift_a, [float(np.float32(a) - np.float32(fi) * np.float32(gam))
                            for a, fi in zip(_vec(base, d), f)])
        _set(inst.diff_s, _vec(lev.diffusion(0.0, x1).reshape(-1), d))
        _set(inst.diff2_s, [float(np.float32(fi) * np.float32(beta)) for fi in f])
        _set(inst.jump_g, f)
    else:
        raise NotImplementedError("no GPU lowering for Levy class %r" % lname)
    ic = lev.icdf
    inst.mark = N.MARK_INVCDF
    p = [ic.cm, ic.cp, ic.mu, ic.alpha, ic.eps, ic.lda, ic.y1, ic.y2, ic.y3, UNIFORM_TOL / 3,
         ic.eps ** (-ic.alpha), -1.0 / ic.alpha]
    _set(inst.mark_p, [float(np.float32(v)) for v in p])
    rate = _f32(sde.jump_rate())
    inst.rate = rate
    inst.inv_rate = float(np.float32(1.0) / np.float32(rate))


_PAYOFFS = {"EuroCall": N.PAYOFF_EUROCALL, "EuroPut": N.PAYOFF_EUROPUT, "BinaryAoN": N.PAYOFF_BINARY_AON,
            "Rainbow": N.PAYOFF_RAINBOW, "Digital": N.PAYOFF_DIGITAL, "BestOf": N.PAYOFF_BESTOF,
            "AsianCall": N.PAYOFF_ASIANCALL, "HestonRainbow": N.PAYOFF_HESTON_RAINBOW}


def lower_payoff(payoff, inst):
    name = _name(payoff)
    if name == "Basket":
        inst.payoff = N.PAYOFF_BASKET_ARITH if payoff.average_type == 'arithmetic' else N.PAYOFF_BASKET_GEO
    elif name in _PAYOFFS:
        inst.payoff = _PAYOFFS[name]
    else:
        raise NotImplementedError("no GPU lowering for payoff class %r" % name)
    inst.strike = _f32(payoff.strike)
    inst.payoff_log = 1 if payoff.log else 0
    inst.payoff_scale = _f32(payoff.discount)
    return inst


def lower_discount(discounter, T, inst):
    if discounter is None:
        inst.discount, inst.disc_rate = 1.0, 0.0
        return inst
    inst.discount = _f32(discounter(T))
    inst.disc_rate = _f32(getattr(discounter, "r", 0.0))
    return inst


def pack_cholesky(L, d):
    L = torch.as_tensor(L).detach().to(device='cpu', dtype=_F32)
    if L.numel() == 1:
        L = torch.ones(1, 1) * L.reshape(-1)[0]
    out = []
    for i in range(d):
        for j in range(i + 1):
            out.append(float(L[i, j]) if L.shape[0] > i and L.shape[1] > j else (1.0 if i == j else 0.0))
    return out


def solver_cholesky(solver):
    L = getattr(solver, "lower_cholesky", None)
    if L is None:
        corr = solver.sde.corr_matrix
        L = torch.linalg.cholesky(corr) if len(corr) > 1 else torch.tensor([[1.]])
    return L


def is_jump_solver(solver):
    return hasattr(solver, "max_jumps")


def lower(solver, payoff=None, discounter=None, num_paths=0, path_offset=0, stream_id=0, seed=None,
          num_steps=None):
    """Build the full descriptor for ``num_paths`` paths of ``solver``."""
    inst = N.SdemcInst()
    sde = solver.sde
    lower_sde(sde, inst)
    heston_scheme = _name(solver) == "HestonSolver"
    if heston_scheme and inst.model != N.MODEL_HESTON:
        raise NotImplementedError("HestonSolver steps a Heston model only")
    if inst.model == N.MODEL_HESTON and not heston_scheme:
        # EulerScheme on Heston: the variance has zero drift and diffusion, so
        # it stays at v0 and the price is a GBM with volatility sqrt(v0)
        inst.model = N.MODEL_AFFINE
        v0 = np.float32(inst.x0[1])
        inst.diff_q[0] = float(np.sqrt(v0))
        inst.mark_p[0] = inst.mark_p[1] = inst.mark_p[2] = inst.mark_p[3] = 0.0
    steps = int(num_steps if num_steps is not None else solver.num_steps)
    T = float(solver.time_interval)
    inst.num_steps = steps
    inst.T = float(np.float32(T))
    inst.h = float(np.float32(T / steps))
    if is_jump_solver(solver):
        inst.grid = N.GRID_ADAPTED
        inst.exact_jumps = 1 if getattr(solver, "exact_jumps", False) else 0
    else:
        inst.grid = N.GRID_UNIFORM
        if inst.rate > 0:
            raise NotImplementedError("a jump model needs the jump-adapted solver (JumpEulerSolver)")
        if inst.noise == N.NOISE_INDEP_SHARED:
            inst.noise = N.NOISE_INDEP_PAIR
    if inst.grid == N.GRID_ADAPTED and inst.noise == N.NOISE_INDEP_PAIR:
        raise NotImplementedError("two-Brownian 'indep' diffusions run on the uniform grid only")
    _set(inst.chol, pack_cholesky(solver_cholesky(solver), inst.dim) + [0.0] * (N.CHOL_LEN - inst.dim * (inst.dim + 1) // 2))
    if payoff is not None:
        lower_payoff(payoff, inst)
    lower_discount(discounter, T, inst)
    inst.seed = int(seed if seed is not None else getattr(solver, "seed", 1)) & 0xFFFFFFFFFFFFFFFF
    inst.path_offset = int(path_offset)
    inst.num_paths = int(num_paths)
    inst.stream_id = int(stream_id)
    return inst


def max_jumps_for(rate_total, T):
    """The reference's pre-drawn jump cap max(int(T * Poisson(rate).ppf(1-1e-9)), 5)
    (sde_mc/solvers.py:133), used to size materialised storage."""
    if rate_total <= 0:
        return 5
    from scipy.stats import poisson
    return max(int(T * poisson.ppf(1 - 1 / 1e9, rate_total)), 5)
