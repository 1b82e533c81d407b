"""Problem set-ups shared by the tests: each matches a fixture recorded from the
reference by tests/golden/make_golden.py (same parameters, same classes)."""
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import _native as N
from sde_mc_gb300.lowering import lower


def merton1d(steps=100, seed=1):
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    return sm.JumpEulerSolver(m, 1.0, steps, seed=seed), sm.EuroCall(1.0), sm.ConstantShortRate(0.02)


def merton2d_corr(steps=50, exact=False, seed=1):
    corr = sm.get_corr_matrix([0.5])
    m = sm.Merton(0.02, torch.tensor([0.2, 0.3]), 1.5, -0.05, 0.15, torch.tensor([1., 1.]), dim=2,
                  corr_matrix=corr)
    return (sm.JumpEulerSolver(m, 1.0, steps, exact_jumps=exact, seed=seed), sm.Rainbow(1.0),
            sm.ConstantShortRate(0.02))


def indep2d(steps=64, seed=1):
    """The 2D rainbow model: per-asset independent jumps, rho = 0.5."""
    corr = sm.get_corr_matrix([0.5])
    m = sm.IndependentJumpsMerton(0.02, torch.tensor([0.2, 0.3]), [1.0, 1.0], -0.05, 0.15, torch.ones(2), 2,
                                  corr_matrix=corr)
    return sm.JumpEulerSolver(m, 1.0, steps, seed=seed), sm.Rainbow(1.0), sm.ConstantShortRate(0.02)


def levy2d(steps=16, seed=1):
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    sde = sm.LevySde(lev, torch.ones(2))
    return sm.JumpEulerSolver(sde, 1.0, steps, seed=seed), sm.Rainbow(1.0), sm.ConstantShortRate(0.02)


def levy2d_exact(steps=4, seed=1):
    """The LevyRainbowMLMC preset's model (sde_mc/problem.py:93-106): Levy
    'indep', exact_jumps=True."""
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    return (sm.JumpEulerSolver(sm.LevySde(lev, torch.ones(2)), 1.0, steps, exact_jumps=True, seed=seed),
            sm.Rainbow(1.0), sm.ConstantShortRate(0.02))


def gbm_uniform(steps=12, seed=1):
    g = sm.Gbm(0.02, torch.tensor([0.2, 0.25]), torch.tensor([1., 1.5]), 2, corr_matrix=sm.get_corr_matrix([-0.3]))
    return sm.EulerSolver(g, 1.0, steps, seed=seed), sm.EuroCall(1.0), sm.ConstantShortRate(0.02)


def heston(steps=24, seed=1):
    """Heston (price, variance), rho = -0.7, on the uniform grid."""
    h = sm.Heston(0.02, 2.0, 0.04, 0.3, -0.7, torch.tensor([1., 0.04]))
    return sm.HestonSolver(h, 1.0, steps, seed=seed), sm.EuroCall(1.0), sm.ConstantShortRate(0.02)


def asian_merton(steps=20, seed=1):
    """An Asian call on a 1-D Merton (AsianWrapper) on the jump-adapted grid."""
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    return (sm.JumpEulerSolver(sm.AsianWrapper(m), 1.0, steps, seed=seed), sm.AsianCall(1.0, 1.0),
            sm.ConstantShortRate(0.02))


def loggbm_uniform(steps=16, seed=1):
    """Log-price GBM (constant coefficients), call through Option.log."""
    lg = sm.LogGbm(0.02, 0.25, torch.tensor([0.0]))
    return sm.EulerSolver(lg, 1.0, steps, seed=seed), sm.EuroCall(1.0, log=True), sm.ConstantShortRate(0.02)


def doublegbm_uniform(steps=12, seed=1):
    """GBM driven by two independent 2-D Brownian motions ('indep')."""
    dg = sm.DoubleGbm(0.03, torch.tensor([0.15, 0.2]), torch.tensor([0.1, 0.05]), torch.tensor([1.0, 1.2]), 2)
    return sm.EulerSolver(dg, 1.0, steps, seed=seed), sm.Basket(1.0), sm.ConstantShortRate(0.02)


def basket(d, steps=64, seed=1):
    rho = 0.3
    corr = sm.get_corr_matrix([rho] * (d * (d - 1) // 2)) if d > 1 else None
    sig = torch.linspace(0.1, 0.4, d)
    m = sm.Merton(0.02, sig, 1.5, -0.1, 0.2, torch.ones(d), dim=d, corr_matrix=corr)
    return sm.JumpEulerSolver(m, 1.0, steps, seed=seed), sm.Basket(1.0), sm.ConstantShortRate(0.02)


def double_gbm(d=2, steps=10, seed=1):
    g = sm.DoubleGbm(0.03, 0.15, 0.1, torch.ones(d), d)
    return sm.EulerSolver(g, 1.0, steps, seed=seed), sm.Basket(1.0), sm.ConstantShortRate(0.02)


FIXTURE_CASES = {
    "replay_merton1d": lambda: merton1d(100),
    "replay_merton2d_corr": lambda: merton2d_corr(50),
    "replay_merton2d_exact": lambda: merton2d_corr(20, exact=True),
    "replay_indep2d": lambda: indep2d(64),
    "replay_levy2d": lambda: levy2d(16),
    "replay_gbm_uniform": lambda: gbm_uniform(12),
    "replay_heston": lambda: heston(24),
    "replay_asian_merton": lambda: asian_merton(20),
    "replay_loggbm_uniform": lambda: loggbm_uniform(16),
    "replay_doublegbm_uniform": lambda: doublegbm_uniform(12),
}


def inst_for(case, num_paths=0, seed=7, path_offset=0, steps=None):
    solver, payoff, disc = case
    return lower(solver, payoff, disc, num_paths=num_paths, path_offset=path_offset, seed=seed, num_steps=steps)


def zdim(inst):
    d = inst.dim
    return d if inst.noise == N.NOISE_DIAG else (d + 1 if inst.noise == N.NOISE_INDEP_SHARED else 2 * d)


def served_cv_cases():
    """Requests for the served control variate's parity tests: dimensions 1, 2,
    6 and 8, common and per-asset jumps, call, put, digital, rainbow and
    basket payoffs (every weight kind and aggregate the server uses)."""
    def merton(d, sig, rate, steps, payoff, strike=1.0):
        corr = sm.get_corr_matrix([0.3] * (d * (d - 1) // 2)) if d > 1 else None
        m = sm.Merton(0.02, torch.tensor(sig), rate, -0.1, 0.2, torch.ones(d), dim=d, corr_matrix=corr)
        return sm.JumpEulerSolver(m, 1.0, steps), payoff(strike), sm.ConstantShortRate(0.02)

    return {
        "call1d": merton(1, [0.2], 2.0, 50, sm.EuroCall),
        "put1d": merton(1, [0.25], 1.5, 40, sm.EuroPut),
        "digital1d": merton(1, [0.2], 2.0, 40, sm.Digital),
        "rainbow2d_per_asset": indep2d(64),
        "basket6": merton(6, [0.15, 0.2, 0.25, 0.3, 0.35, 0.4], 2.0, 48, sm.Basket, 1.05),
        "basket8": merton(8, [0.1 + 0.04 * i for i in range(8)], 1.0, 32, sm.Basket, 0.95),
        "bestof3_uniform": (sm.EulerSolver(sm.Gbm(0.02, torch.tensor([0.2, 0.25, 0.3]), torch.ones(3), 3,
                                                  corr_matrix=sm.get_corr_matrix([0.3] * 3)), 1.0, 24),
                            sm.BestOf(1.1), sm.ConstantShortRate(0.02)),
    }
