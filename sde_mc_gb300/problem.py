"""Pricing problems with the reference's presets (sde_mc/problem.py:10-165).

A problem bundles a solver, a discounter and a payoff; ``run_mc`` /
``run_mc_terminal_cv`` / ``run_cv_mc`` take one.  The presets build the same
models, solvers, options and default parameters as the reference's, on this
package's classes, so every call on them runs on the GPU kernels.
"""
from abc import ABC

import torch

from .helpers import get_corr_matrix
from .levy import ExampleLevy, ExpExampleLevy, LevySde
from .options import BestOf, ConstantShortRate, EuroCall, Rainbow
from .sde import Gbm, Heston, Merton
from .solvers import EulerSolver, HestonSolver, JumpEulerSolver


class Problem(ABC):
    """Solver + discounter + payoff (sde_mc/problem.py:10-20)."""

    def __init__(self, solver, discounter, payoff):
        self.solver = solver
        self.discounter = discounter
        self.payoff = payoff

    def dim(self):
        return self.solver.sde.dim

    def set_steps(self, steps):
        self.solver.num_steps = steps


def _spots(spot, dim):
    return spot if torch.is_tensor(spot) else torch.ones(dim) * spot


class BlackScholesEuroCall(Problem):
    """1-D GBM call on the uniform grid."""

    def __init__(self, r, sigma, spot, strike, maturity, steps, device):
        model = Gbm(r, sigma, torch.tensor([spot]), 1)
        super().__init__(EulerSolver(model, maturity, steps, device), ConstantShortRate(r), EuroCall(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(0.02, 0.3, 1, 1, 3, steps, device)


class BlackScholesRainbow(Problem):
    """Correlated d-dimensional GBM, call on the maximum."""

    def __init__(self, r, sigma, spot, strike, maturity, dim, corr_matrix, steps, device):
        model = Gbm(r, sigma, _spots(spot, dim), dim, corr_matrix=corr_matrix)
        super().__init__(EulerSolver(model, maturity, steps, device), ConstantShortRate(r), Rainbow(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(0.02, 0.3, 1, 1, 3, 3, get_corr_matrix([0.7, 0.2, -0.3]), steps, device)


class HestonEuroCall(Problem):
    """Heston call with the implicit variance scheme."""

    def __init__(self, r, kappa, theta, xi, rho, spot, v0, strike, maturity, steps, device):
        model = Heston(r, kappa, theta, xi, rho, torch.tensor([spot, v0]))
        super().__init__(HestonSolver(model, maturity, steps, device), ConstantShortRate(r), EuroCall(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(0.02, 0.25, 0.5, 0.3, -0.3, 1, 0.15, 1, 3, steps, device)


class MertonEuroCall(Problem):
    """1-D Merton jump-diffusion call on the jump-adapted grid."""

    def __init__(self, mu, sigma, rate, alpha, gamma, spot, strike, maturity, steps, device):
        model = Merton(mu, sigma, rate, alpha, gamma, torch.tensor([spot]), 1)
        super().__init__(JumpEulerSolver(model, maturity, steps, device), ConstantShortRate(mu), EuroCall(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(0.02, 0.2, 1, -0.05, 0.3, 1, 1, 3, steps, device)


class LevyRainbow(Problem):
    """Exponential Levy assets, call on the maximum."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim, spot, strike, maturity, steps,
                 device, exact_jumps=False):
        levy = ExpExampleLevy(c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim)
        model = LevySde(levy, _spots(spot, dim), device=device)
        solver = JumpEulerSolver(model, maturity, steps, device=device, exact_jumps=exact_jumps)
        super().__init__(solver, ConstantShortRate(r), Rainbow(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(1, 1, 0.5, 2, 0.02, 0.3, 0.2, 0.001, 2, 1, 1, 3, steps, device)


class LevyRainbowMLMC(LevyRainbow):
    """LevyRainbow with jumps scaled by the post-diffusion state (the MLMC preset)."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim, spot, strike, maturity, steps,
                 device):
        super().__init__(c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim, spot, strike, maturity, steps,
                         device, exact_jumps=True)

    @classmethod
    def default_params(cls, steps, device):
        # the reference's preset returns the plain LevyRainbow here
        return LevyRainbow.default_params(steps, device)


class LevyCall(Problem):
    """1-D additive Levy log-price, call on exp(x) discounted forward."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, spot, strike, maturity, steps, device):
        chol = torch.tensor([[1.]], device=device)
        levy = ExampleLevy(c_minus, c_plus, alpha, mu, r, torch.tensor([sigma], device=device),
                           torch.tensor([f], device=device), chol, epsilon, 1)
        model = LevySde(levy, torch.tensor([spot]), device=device)
        csr = ConstantShortRate(r)
        super().__init__(JumpEulerSolver(model, maturity, steps, device=device), csr,
                         EuroCall(strike, log=True, discount=csr(-maturity)))

    @classmethod
    def default_params(cls, steps, device):
        return cls(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.001, 0, 1, 3, steps, device)


class LevyBestOf(Problem):
    """Exponential Levy assets, best-of payoff."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim, spot, strike, maturity, steps,
                 device):
        levy = ExpExampleLevy(c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim)
        model = LevySde(levy, _spots(spot, dim), device=device)
        super().__init__(JumpEulerSolver(model, maturity, steps, device=device), ConstantShortRate(r),
                         BestOf(strike))

    @classmethod
    def default_params(cls, steps, device):
        return cls(1, 1, 0.2, 2, 0.02, 0.3, 0.2, 0.001, 4, 1, 1, 3, steps, device)


class LevyCallOnMax(Problem):
    """Correlated additive Levy log-prices, call on the maximum of exp(x)."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, chol_corr, epsilon, dim, spot, strike, maturity,
                 steps, device):
        # argument order of the reference's call (c_plus first in ExampleLevy)
        levy = ExampleLevy(c_plus, c_minus, alpha, mu, r, sigma, f, chol_corr, epsilon, dim)
        model = LevySde(levy, _spots(spot, dim), device=device)
        csr = ConstantShortRate(r)
        super().__init__(JumpEulerSolver(model, maturity, steps, device=device), csr,
                         Rainbow(strike, log=True, discount=csr(-maturity)))

    @classmethod
    def default_params(cls, dim, steps, device):
        presets = {2: ([0.4], [0.2, 0.2], [0.15, 0.15]),
                   4: ([0.87, 0.94, 0.86, 0.87, 0.93, 0.96], [0.2, 0.15, 0.15, 0.1], [0.1, 0.1, 0.1, 0.1])}
        if dim not in presets:
            return 'No default parameters for dimension {:}'.format(dim)
        rhos, fs, sigmas = presets[dim]
        chol = torch.linalg.cholesky(get_corr_matrix(rhos)).to(device)
        return cls(1, 1, 0.5, 2, 0.02, torch.tensor(sigmas, device=device), torch.tensor(fs, device=device), chol,
                   0.001, dim, 0, 1, 3, steps, device)
