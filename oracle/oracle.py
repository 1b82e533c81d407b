"""CPU oracle for the sde_mc path-integration hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py may import this module, and only to check the
kernels' results (or as the timed CPU baseline) — the product package never
imports it.

Contents (each restating the reference, piers-hinds/sde_mc):
  * ctypes access to the C restatement ``sdemc_oracle.c`` of the solver loops
    (sde_mc/solvers.py:68-88, 164-226, 228-307), payoffs and reductions;
  * FP64 closed forms: Black-Scholes call and digital, asset-or-nothing,
    geometric Asian and the 40-term Merton series (sde_mc/options.py:8-153);
  * mc_estimates (sde_mc/helpers.py:51-68) and Giles' MLMC allocation
    (sde_mc/mlmc.py:77-97);
  * the pricing server's request flow (run_mc, sde_mc/mc.py:418-440, with the
    linear control variate): per-path regressors in C, then the pilot sums,
    the regression for beta, the main-run size (find_num_trials,
    sde_mc/mc.py:418-427) and the main run's sums;
  * the control-variate MLP (sde_mc/nets.py:39-93 without batch norm), its
    variance loss (sde_mc/varred.py:160-177, 202-214) with hand-derived
    gradients, and one Adam step, in numpy FP64.

Parity is pinned against the reference itself through the fixtures in
tests/golden/ (recorded by tests/golden/make_golden.py from the reference).
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsdemc_oracle.so")

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from . import build as _b  # noqa
            _b.build()
        lib = ctypes.CDLL(LIB)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        I64 = ctypes.c_int64
        sig = {
            "oracle_philox": (None, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                     ctypes.c_uint32, I, P]),
            "oracle_native_normals": (None, [P, I64, I, P]),
            "oracle_native_jumps": (None, [P, I64, I, P, P, P]),
            "oracle_replay": (I, [P, I, I, I, P, P, P, P, P, P, P, P, P, P]),
            "oracle_from_export": (I, [P, I64, I, P, I, P, P, P, I, I, P, P, P, P, P, P, P]),
            "oracle_mlmc_replay": (I, [P, I, F, F, I, I, I, I, P, P, P, P, P, P]),
            "oracle_price": (I, [P, I, P, P]),
            "oracle_mlmc_level": (I, [P, I, F, F, I, P, P]),
            "oracle_chunk_reduce": (None, [P, P, I64, P]),
            "oracle_payoff": (F, [P, P]),
            "oracle_serve_cv_weights": (I, [P, P]),
            "oracle_serve_cv_from_export": (I, [P, P, I64, I, P, P, P, P, I, P, I, P, P, P]),
            "oracle_serve_rows": (None, [I, I64, P, P, P, P]),
            "oracle_serve_slices": (None, [P, I64, I, I64, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _c(a, dt=np.float32):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


# --------------------------------------------------------------- RNG -------
def philox(seed, stream, tag, path, first, n):
    out = np.zeros((n, 4), np.uint32)
    load().oracle_philox(seed, stream, tag, path, first, n, _p(out))
    return out


def native_normals(inst, path, nsteps, zdim):
    out = np.zeros((nsteps, zdim), np.float32)
    load().oracle_native_normals(ctypes.byref(inst), path, nsteps, _p(out))
    return out


def native_jumps(inst, path, n):
    jt = np.zeros(n, np.float32)
    jm = np.zeros(n, np.float32)
    js = np.zeros(n, np.int32)
    load().oracle_native_jumps(ctypes.byref(inst), path, n, _p(jt), _p(jm), _p(js))
    return jt, jm, js


# ----------------------------------------------------------- solvers -------
def replay(inst, dw, jump_times=None, marks=None, asset=None):
    dw = _c(dw)
    bs, S = dw.shape[0], dw.shape[1]
    d = inst.dim
    jump_times, marks, asset = _c(jump_times), _c(marks), _c(asset, np.int32)
    out = dict(paths=np.zeros((bs, S + 1, d), np.float32), left=np.zeros((bs, S + 1, d), np.float32),
               time=np.zeros((bs, S + 1), np.float32), jumps=np.zeros((bs, S + 1, d), np.float32),
               payoffs=np.zeros(bs, np.float32), steps=np.zeros(bs, np.int32))
    mj = jump_times.shape[1] if jump_times is not None else 0
    rc = load().oracle_replay(ctypes.byref(inst), bs, S, mj, _p(jump_times), _p(dw), _p(marks), _p(asset),
                              _p(out["paths"]), _p(out["left"]), _p(out["time"]), _p(out["jumps"]),
                              _p(out["payoffs"]), _p(out["steps"]))
    out["rc"] = rc
    return out


def from_export(inst, z, S, jt=None, jm=None, jsel=None, exact=False):
    """Re-run paths from raw draws a GPU materialise call exported."""
    z = _c(z)
    n, zd = z.shape[0], z.shape[2]
    d = inst.dim
    nw = 1 if inst.noise == 0 else 2
    jt, jm, jsel = _c(jt), _c(jm), _c(jsel, np.int32)
    jcap = jt.shape[1] if jt is not None else 0
    out = dict(paths=np.zeros((n, S + 1, d), np.float32), left=np.zeros((n, S + 1, d), np.float32),
               time=np.zeros((n, S + 1), np.float32), jumps=np.zeros((n, S + 1, d), np.float32),
               normals=np.zeros((n, S, d) if nw == 1 else (n, S, d, 2), np.float32),
               payoffs=np.zeros(n, np.float32), steps=np.zeros(n, np.int32))
    rc = load().oracle_from_export(ctypes.byref(inst), n, S, _p(z), zd, _p(jt), _p(jm), _p(jsel), jcap,
                                   1 if exact else 0, _p(out["paths"]), _p(out["left"]), _p(out["time"]),
                                   _p(out["jumps"]), _p(out["normals"]), _p(out["payoffs"]), _p(out["steps"]))
    out["rc"] = rc
    return out


def mlmc_replay(inst, factor, hf, hc, dw, coarse_cap, jump_times=None, marks=None, asset=None):
    dw = _c(dw)
    bs, Sf = dw.shape[0], dw.shape[1]
    d = inst.dim
    jump_times, marks, asset = _c(jump_times), _c(marks), _c(asset, np.int32)
    xf = np.zeros((bs, d), np.float32)
    xc = np.zeros((bs, d), np.float32)
    mj = jump_times.shape[1] if jump_times is not None else 0
    rc = load().oracle_mlmc_replay(ctypes.byref(inst), factor, hf, hc, bs, Sf, coarse_cap, mj, _p(jump_times),
                                   _p(dw), _p(marks), _p(asset), _p(xf), _p(xc))
    return dict(xf=xf, xc=xc, rc=rc)


def price(inst, nthreads=None, payoffs=False):
    """Native-draw pricing on host threads: (sum, sum_sq, n, mean, var)."""
    nthreads = nthreads or os.cpu_count() or 1
    out = np.zeros(7, np.float64)
    pay = np.zeros(inst.num_paths, np.float32) if payoffs else None
    rc = load().oracle_price(ctypes.byref(inst), nthreads, _p(pay), _p(out))
    return out, pay, rc


def mlmc_level(inst, factor, hf, hc, nthreads=None):
    nthreads = nthreads or os.cpu_count() or 1
    out = np.zeros(7, np.float64)
    rc = load().oracle_mlmc_level(ctypes.byref(inst), factor, hf, hc, nthreads, None, _p(out))
    return out, rc


def chunk_reduce(vals, vals2=None):
    """The GPU kernels' reduction order restated (bit-exact given the values)."""
    vals = _c(vals)
    vals2 = _c(vals2)
    out = np.zeros(7 if vals2 is not None else 5, np.float64)
    load().oracle_chunk_reduce(_p(vals), _p(vals2), vals.shape[0], _p(out))
    return out


# ------------------------------------------------------ closed forms -------
def norm_cdf(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def bs_call(spot, strike, expiry, r, sigma):
    sd = sigma * math.sqrt(expiry)
    d1 = (math.log(spot / strike) + (r + 0.5 * sigma * sigma) * expiry) / sd
    return spot * norm_cdf(d1) - strike * math.exp(-r * expiry) * norm_cdf(d1 - sd)


def bs_binary_aon(spot, strike, expiry, r, sigma):
    """The reference integrates exp(-z^2/2)/sqrt(2 pi) up to d1 (quad): Phi(d1)."""
    d1 = (math.log(spot / strike) + (r + 0.5 * sigma * sigma) * expiry) / (math.sqrt(expiry) * sigma)
    return norm_cdf(d1)


def merton_call(spot, strike, expiry, r, sigma, alpha, gamma, rate, terms=40):
    beta = math.exp(alpha + 0.5 * gamma * gamma) - 1
    lam = (1 + beta) * rate * expiry
    total = 0.0
    for k in range(terms):
        r_k = r - rate * beta + k * math.log1p(beta) / expiry
        s_k = math.sqrt(sigma * sigma + k * gamma * gamma / expiry)
        total += math.exp(-lam) * lam ** k / math.factorial(k) * bs_call(spot, strike, expiry, r_k, s_k)
    return total


def bs_digital_call(spot, strike, expiry, r, sigma):
    sd = sigma * math.sqrt(expiry)
    d2 = (math.log(spot / strike) + (r - 0.5 * sigma * sigma) * expiry) / sd
    return norm_cdf(d2) * math.exp(-r * expiry)


def bs_asian_call(spot, strike, expiry, r, sigma):
    sg = sigma / math.sqrt(3)
    b = 0.5 * (r - 0.5 * sg * sg)
    sd = sg * math.sqrt(expiry)
    d1 = (math.log(spot / strike) + (b + 0.5 * sg * sg) * expiry) / sd
    return spot * math.exp((b - r) * expiry) * norm_cdf(d1) - strike * math.exp(-r * expiry) * norm_cdf(d1 - sd)


def heston_call(spot, v0, strike, expiry, r, kappa, theta, xi, rho):
    """European call under Heston by Fourier inversion of the characteristic
    function (Heston 1993), in the branch-cut-free form of Albrecher, Mayer,
    Schoutens and Tistaert, "The little Heston trap" (2007):
    C = S P1 - K e^{-rT} P2, P_j = 1/2 + (1/pi) int_0^inf Re[e^{-iu ln K} phi_j(u) / (iu)] du
    with phi_2 = phi and phi_1(u) = phi(u - i) / phi(-i).  An independent
    check of the Heston model kind (the reference has no closed form)."""
    from scipy.integrate import quad
    x0, lk = math.log(spot), math.log(strike)

    def phi(u):
        iu = 1j * u
        beta = kappa - rho * xi * iu
        d = np.sqrt(beta * beta + xi * xi * (iu + u * u))
        g = (beta - d) / (beta + d)
        e = np.exp(-d * expiry)
        c = kappa * theta / (xi * xi) * ((beta - d) * expiry - 2.0 * np.log((1.0 - g * e) / (1.0 - g)))
        dd = v0 / (xi * xi) * (beta - d) * (1.0 - e) / (1.0 - g * e)
        return np.exp(iu * (x0 + r * expiry) + c + dd)

    fwd = spot * math.exp(r * expiry)

    def p(j):
        if j == 1:
            f = lambda u: (np.exp(-1j * u * lk) * phi(u - 1j) / (1j * u * fwd)).real
        else:
            f = lambda u: (np.exp(-1j * u * lk) * phi(u) / (1j * u)).real
        return 0.5 + quad(f, 1e-10, 200.0, limit=400, epsabs=1e-12, epsrel=1e-10)[0] / math.pi

    return spot * p(1) - strike * math.exp(-r * expiry) * p(2)


# -------------------------------------------------------- estimators -------
def mc_estimates(s, s2, n):
    return s / n, (s2 - s * s / n) / (n - 1)


def optimal_trials(level_vars, levels, T, eps):
    v = np.asarray(level_vars, np.float64)
    h = T / np.asarray(levels, np.float64)
    return np.ceil((1.96 ** 2 / eps ** 2) * np.sqrt(v * h) * np.sqrt(v / h).sum()).astype(np.int64)


# ----------------------------------------------------------- CV MLP --------
def mlp_forward(params, x):
    """params: [W0, b0, W1, b1, ..., WL, bL] with W (out, in) as torch Linear.
    Returns output and the list of pre-activations / activations."""
    acts = [x]
    pre = []
    h = x
    nl = len(params) // 2
    for i in range(nl):
        W, b = params[2 * i], params[2 * i + 1]
        z = h @ W.T + b
        pre.append(z)
        h = np.maximum(z, 0.0) if i < nl - 1 else z
        acts.append(h)
    return h, pre, acts


def cv_loss_and_grads(params, f_in, normals, time, payoffs, r):
    """Gamma = payoff + sum_k e^{-r t_k} f(t_k, X_k) . dW_k; loss = Var(Gamma)
    (unbiased); gradients by hand-written backpropagation."""
    n, S, d = normals.shape
    out, pre, acts = mlp_forward(params, f_in)
    disc = np.exp(-time * r)[..., None] if time.ndim == 2 else np.exp(-time * r)
    fo = out.reshape(n, S, d)
    gamma = payoffs + (normals * fo * disc).sum(-1).sum(-1)
    gm = gamma.mean()
    loss = ((gamma - gm) ** 2).sum() / (n - 1)
    dgamma = 2.0 * (gamma - gm) / (n - 1)
    dout = (dgamma[:, None, None] * normals * disc).reshape(n * S, d)
    grads = [None] * len(params)
    g = dout
    nl = len(params) // 2
    for i in reversed(range(nl)):
        W = params[2 * i]
        grads[2 * i] = g.T @ acts[i]
        grads[2 * i + 1] = g.sum(0)
        if i > 0:
            g = (g @ W) * (pre[i - 1] > 0)
    return loss, gamma, grads


def adam_step(params, grads, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, state=None, step=1):
    """One torch.optim.Adam step (no weight decay, no amsgrad)."""
    if state is None:
        state = [(np.zeros_like(p), np.zeros_like(p)) for p in params]
    new, st = [], []
    for p, g, (m, v) in zip(params, grads, state):
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        mh = m / (1 - b1 ** step)
        vh = v / (1 - b2 ** step)
        new.append(p - lr * mh / (np.sqrt(vh) + eps))
        st.append((m, v))
    return new, st


# ----------------------------------------- mixed-precision restatement ----
# The GPU network kernels keep layer 1 and layer 4 in FP32 and run the two
# 64x64 layers on BF16 tensor cores with FP32 accumulation.  These functions
# restate that precision policy in numpy (BF16 roundings where the kernels
# round, FP64 sums elsewhere), so that kernel bugs separate from rounding: the
# GPU agrees with them to FP32 accumulation-order noise, and they agree with
# the FP32 reference network (mlp_forward / cv_loss_and_grads) to BF16 noise.
def bf16_round(x):
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def _f32(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32).astype(np.float64)


def mlp_forward_mixed(params, t, x):
    """Kernel-precision forward.  t (R,), x (R, d); params as mlp_forward.
    Returns (out, cache) with the BF16 activations the backward needs."""
    W1, b1, W2, b2, W3, b3, W4, b4 = [np.asarray(p, dtype=np.float32) for p in params]
    t = np.asarray(t, dtype=np.float32).astype(np.float64)
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    z = _f32(W1[:, 0].astype(np.float64)[None, :] * t[:, None] + b1.astype(np.float64)[None, :])
    for i in range(x.shape[1]):
        z = _f32(W1[:, 1 + i].astype(np.float64)[None, :] * x[:, i:i + 1] + z)
    h1b = bf16_round(np.maximum(z, 0.0)).astype(np.float64)
    w2b = bf16_round(W2).astype(np.float64)
    w3b = bf16_round(W3).astype(np.float64)
    z2 = _f32(h1b @ w2b.T + b2.astype(np.float64))
    h2b = bf16_round(np.maximum(z2, 0.0)).astype(np.float64)
    z3 = _f32(h2b @ w3b.T + b3.astype(np.float64))
    h3 = np.maximum(z3, 0.0)
    out = _f32(h3 @ W4.astype(np.float64).T + b4.astype(np.float64))
    return out, dict(h1b=h1b, h2b=h2b, h3=h3, w2b=w2b, w3b=w3b, W4=W4.astype(np.float64))


def cv_gamma_mixed(params, time, paths, normals, payoffs, r):
    """Gamma_p = payoff_p + sum_k e^{-r t_k} f(t_k, X_k) . dW_k at kernel
    precision.  time (n, S), paths (n, S, d), normals (n, S, d)."""
    n, S, d = normals.shape
    out, _ = mlp_forward_mixed(params, np.reshape(time, -1), np.reshape(paths, (n * S, d)))
    fo = out.reshape(n, S, d)
    disc = np.exp(-np.asarray(time, np.float64).reshape(n, S) * r)
    gam = np.asarray(payoffs, np.float64) + ((np.asarray(normals, np.float64) * fo).sum(-1) * disc).sum(-1)
    return gam, fo


def cv_grads_mixed(params, time, paths, normals, gamma, r):
    """Gradients of Var(Gamma) (unbiased) at kernel precision, given Gamma."""
    n, S, d = normals.shape
    t = np.reshape(time, -1)
    xin = np.reshape(paths, (n * S, d))
    _, c = mlp_forward_mixed(params, t, xin)
    g = np.asarray(gamma, np.float64)
    dgam = 2.0 * (g - g.mean()) / (n - 1)
    disc = np.exp(-np.asarray(time, np.float64).reshape(n, S) * r)
    dO = ((dgam[:, None] * disc)[..., None] * np.asarray(normals, np.float64)).reshape(n * S, d)
    dz3 = (dO @ c["W4"]) * (c["h3"] > 0)
    gW4, gb4 = dO.T @ c["h3"], dO.sum(0)
    dz3b = bf16_round(dz3).astype(np.float64)
    gW3, gb3 = dz3b.T @ c["h2b"], dz3b.sum(0)
    dz2b = bf16_round((dz3b @ c["w3b"]) * (c["h2b"] > 0)).astype(np.float64)
    gW2, gb2 = dz2b.T @ c["h1b"], dz2b.sum(0)
    dz1 = (dz2b @ c["w2b"]) * (c["h1b"] > 0)
    inp = np.concatenate([np.asarray(t, np.float64)[:, None], np.asarray(xin, np.float64)], axis=1)
    gW1, gb1 = dz1.T @ inp, dz1.sum(0)
    return [gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4]


def cv_jump_multipliers(time, jumps, lam_kappa):
    """Per-row multipliers of the jump integrand g in the reference's adapted
    control variate (sde_mc/varred.py:118-128): the recorded mark J_k minus the
    compensator lambda E[J] h_k with h = diff(time) — the last row has no
    compensator because the reference sums g[:, :-1] against diff(time).
    time (n, S), jumps (n, S, d), lam_kappa scalar or (d,)."""
    t = np.asarray(time, np.float64)
    m = np.array(jumps, np.float64, copy=True)
    h = np.diff(t, axis=1)
    m[:, :-1, :] -= np.asarray(lam_kappa, np.float64) * h[..., None]
    return m


def cv2_loss_and_grads(pf, pg, time, paths, left, normals, mult_g, payoffs, r):
    """Var(Gamma) with Gamma = payoff + sum e^{-rt} f(t, X) . dW
    + sum e^{-rt} g(t, X-) . mult_g, and both networks' gradients (FP64)."""
    n, S, d = normals.shape
    t = np.asarray(time, np.float64).reshape(n, S)
    fin = np.concatenate([t.reshape(-1, 1), np.asarray(paths, np.float64).reshape(-1, d)], 1)
    gin = np.concatenate([t.reshape(-1, 1), np.asarray(left, np.float64).reshape(-1, d)], 1)
    disc = np.exp(-t * r)[..., None]
    fo = mlp_forward(pf, fin)[0].reshape(n, S, d)
    go = mlp_forward(pg, gin)[0].reshape(n, S, d)
    a_f = (np.asarray(normals, np.float64) * fo * disc).sum((1, 2))
    a_g = (mult_g * go * disc).sum((1, 2))
    pay = np.asarray(payoffs, np.float64)
    loss, gamma, gf = cv_loss_and_grads(pf, fin, np.asarray(normals, np.float64), t, pay + a_g, r)
    _, _, gg = cv_loss_and_grads(pg, gin, mult_g, t, pay + a_f, r)
    return loss, gamma, gf, gg


# ------------------------------------------------- served control variate ---
class CvWeights(ctypes.Structure):
    """Mirror of ``sdemc_cv_weights`` (include/sdemc.h)."""
    _fields_ = [("comp", ctypes.c_float * 8), ("inv_comp", ctypes.c_float * 8), ("scale_over_k", ctypes.c_float),
                ("inv_sig", ctypes.c_float), ("drift", ctypes.c_float), ("T", ctypes.c_float),
                ("comp_j2", ctypes.c_float), ("inv_comp_j2", ctypes.c_float), ("agg", ctypes.c_int32),
                ("wkind", ctypes.c_int32), ("jumps", ctypes.c_int32), ("reserved", ctypes.c_int32)]


def serve_cv_weights(inst):
    cw = CvWeights()
    rc = load().oracle_serve_cv_weights(ctypes.byref(inst), ctypes.byref(cw))
    assert rc == 0
    return cw


def serve_cv_from_export(inst, cw, z, jt=None, jm=None, jsel=None, wg=None):
    """Per-path payoffs and the 2d + 1 control-variate regressors re-run from a
    GPU run's exported draws.  With ``wg`` (n, wcap, 2) the GPU's weights are
    used and checked: returns (payoffs, reg, rc, (worst w ratio, worst g
    ratio, blocks)); the ratios are error / bound and must stay <= 1."""
    z = _c(z)
    n, S = z.shape[0], z.shape[1]
    R = 2 * inst.dim + 1
    jt, jm, jsel, wg = _c(jt), _c(jm), _c(jsel, np.int32), _c(wg)
    jcap = jt.shape[1] if jt is not None else 0
    wcap = wg.shape[1] if wg is not None else 0
    pay = np.zeros(n, np.float32)
    reg = np.zeros((n, R), np.float32)
    ws = np.zeros(3, np.float64)
    rc = load().oracle_serve_cv_from_export(ctypes.byref(inst), ctypes.byref(cw), n, S, _p(z), _p(jt), _p(jm),
                                            _p(jsel), jcap, _p(wg), wcap, _p(pay), _p(reg), _p(ws))
    return pay, reg, rc, tuple(ws)


def serve_rows(pv, y, beta=None):
    """The server kernels' per-chunk FP64 rows (see oracle_serve_rows)."""
    pv, y = _c(pv), _c(y)
    n, R = y.shape
    W = 3 if beta is not None else 3 + 2 * R + R * (R + 1) // 2
    nch = (n + 31) // 32
    rows = np.zeros((max(nch, 1), W), np.float64)
    b = None if beta is None else _c(np.asarray(beta, np.float32)[:R])
    load().oracle_serve_rows(R, n, _p(pv), _p(y), _p(b), _p(rows))
    return rows[:nch]


def serve_slices(rows, slice_paths):
    """A phase's running sums: the rows accumulated slice by slice."""
    rows = _c(rows, np.float64)
    nch, W = rows.shape
    acc = np.zeros(W, np.float64)
    load().oracle_serve_slices(_p(rows), nch, W, slice_paths // 32, _p(acc))
    return acc


def serve_slice_paths(inst, slice_work=1 << 28):
    """Paths per slice of a request: the slice work over the expected path
    cost (nominal steps plus expected jumps, times the dimension), clamped to
    [2^10, 2^18] and rounded up to whole 32-path chunks."""
    steps = float(inst.num_steps)
    if inst.grid == 0:
        steps += float(np.float32(inst.rate)) * float(np.float32(inst.T))
    cost = steps * float(inst.dim)
    sl = math.ceil(float(slice_work) / max(cost, 1.0))
    sl = min(max(sl, 1 << 10), 1 << 18)
    return (sl + 31) // 32 * 32


def _solve_spd(C, c):
    """Cholesky solve of C beta = c with a jitter of 1e-12 tr / d on the
    diagonal, in the server's operation order; None when C is degenerate."""
    d = len(c)
    tr = 0.0
    for i in range(d):
        tr += C[i][i]
    if not (tr > 0.0) or not math.isfinite(tr):
        return None
    jitter = 1e-12 * tr / d
    L = [[0.0] * d for _ in range(d)]
    for i in range(d):
        for j in range(i + 1):
            s = C[i][j] + (jitter if i == j else 0.0)
            for k in range(j):
                s -= L[i][k] * L[j][k]
            if i == j:
                if not (s > 0.0):
                    return None
                L[i][i] = math.sqrt(s)
            else:
                L[i][j] = s / L[j][j]
    z = [0.0] * d
    for i in range(d):
        s = c[i]
        for k in range(i):
            s -= L[i][k] * z[k]
        z[i] = s / L[i][i]
    beta = [0.0] * d
    for i in range(d - 1, -1, -1):
        s = z[i]
        for k in range(i + 1, d):
            s -= L[k][i] * beta[k]
        beta[i] = s / L[i][i]
    if not all(math.isfinite(b) for b in beta):
        return None
    return beta


def serve_fit(acc, R, rel_target, max_paths=0):
    """A finished pilot: its mean and standard error, the control variate's
    coefficients fitted by regression on the pilot sums (kept when they cut
    the variance by 5 % or more), and the main run's size for a 95 %
    half-width of rel_target x |price| (find_num_trials, sde_mc/mc.py:418-427).
    acc holds the pilot sums in the pilot-statistics layout (or 3 sums for a
    plain pilot, R = 0)."""
    n = acc[2]
    mean = acc[0] / n if n > 0 else 0.0
    var = max((acc[1] - acc[0] * acc[0] / n) / (n - 1.0), 0.0) if n > 1 else 0.0
    out = dict(pilot_mean=mean, pilot_se=math.sqrt(var / max(n, 1.0)), est=0, vrf=1.0,
               beta=np.zeros(17, np.float32))
    var_main = var
    if R > 0 and n > 2:
        ybar = [acc[3 + a] / n for a in range(R)]
        C = [[0.0] * R for _ in range(R)]
        q = 3 + R
        for a in range(R):
            for b in range(a, R):
                v = (acc[q] - n * ybar[a] * ybar[b]) / (n - 1.0)
                C[a][b] = v
                C[b][a] = v
                q += 1
        c = [(acc[q + a] - n * ybar[a] * mean) / (n - 1.0) for a in range(R)]
        beta = _solve_spd(C, c)
        if beta is not None:
            explained = 0.0
            for a in range(R):
                explained += beta[a] * c[a]
            resid = var - explained
            if 0.0 < resid < var / 1.05:
                var_main = resid
                out["est"] = 1
                out["vrf"] = var / resid
                out["beta"][:R] = np.asarray(beta, np.float64).astype(np.float32)
    out["var_main"] = var_main
    if var_main <= 0.0:
        out["main_paths"] = 0
        return out
    cap = max_paths if max_paths > 0 else (1 << 36)
    eps = rel_target * abs(mean)
    if eps > 0.0 and math.isfinite(eps):
        want = math.ceil(1.96 * 1.96 * var_main / (eps * eps))
        nmain = cap if want >= cap else int(want)
    else:
        nmain = cap
    out["main_paths"] = max(nmain, 64)
    return out


def serve_main(acc):
    """Mean and standard error of a finished main run from its 3 sums."""
    n = acc[2]
    mean = acc[0] / n if n > 0 else 0.0
    var = max((acc[1] - acc[0] * acc[0] / n) / (n - 1.0), 0.0) if n > 1 else 0.0
    return mean, math.sqrt(var / max(n, 1.0))
