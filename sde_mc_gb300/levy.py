"""Levy-driven SDEs with truncated small jumps (sde_mc/levy.py:1-192).

``LevySde`` presents a Levy model through the ``Sde`` interface: jumps larger
than epsilon come from a compound Poisson clock with marks drawn by the
piecewise inverse CDF of the truncated measure, small jumps are replaced by an
extra Brownian term ('indep' layout: one shared scalar Brownian motion).
"""
from abc import abstractmethod

import numpy as np
import torch

from .helpers import get_jump_comp
from .sde import Sde

UNIFORM_TOL = 5.960464477539063e-08


class InverseCdf:
    """Inverse CDF of the normalised jump measure restricted to |x| > epsilon:
    exponential tails beyond |x| = 1 and power-law parts on (epsilon, 1)."""

    def __init__(self, c_minus, c_plus, mu, alpha, epsilon):
        self.cm, self.cp, self.mu, self.alpha, self.eps = c_minus, c_plus, mu, alpha, epsilon
        ea = epsilon ** (-alpha)
        self.lda = (c_minus + c_plus) * (1 / mu + (ea - 1) / alpha)
        self.y1 = c_minus / (mu * self.lda)
        self.y2 = (c_minus / mu + c_minus * (ea - 1) / alpha) / self.lda
        self.y3 = 1 - c_plus / (mu * self.lda)

    def __call__(self, y):
        cm, cp, mu, al, lda = self.cm, self.cp, self.mu, self.alpha, self.lda
        ea = self.eps ** (-al)
        left_tail = torch.log(mu * lda * y / cm) / mu - 1
        left_body = -(al * (lda * y / cm - 1 / mu) + 1) ** (-1 / al)
        right_body = ((-al / cp) * (lda * y - cm / mu - cm * (ea - 1) / al) + ea) ** (-1 / al)
        right_tail = 1 - torch.log(mu * lda * (1 - y) / cp) / mu
        return torch.where(y <= self.y1, left_tail,
                           torch.where(y < self.y2, left_body, torch.where(y < self.y3, right_body, right_tail)))


class Levy:
    """Levy-driven dynamics: coefficients plus the small-jump drift (gamma) and
    small-jump volatility (beta) of the truncation."""

    def __init__(self, dim, icdf):
        self.dim = dim
        self.icdf = icdf

    @abstractmethod
    def drift(self, t, x):
        pass

    @abstractmethod
    def diffusion(self, t, x):
        pass

    @abstractmethod
    def jumps(self, t, x, jumps):
        pass

    @abstractmethod
    def gamma(self):
        pass

    @abstractmethod
    def beta(self):
        pass

    @abstractmethod
    def jump_mean(self):
        pass


def _trunc_gamma(cp, cm, alpha, eps):
    return (cp - cm) * (1 - eps ** (1 - alpha)) / (1 - alpha)


def _trunc_beta(cp, cm, alpha, eps):
    return np.sqrt((cp + cm) * eps ** (2 - alpha) / (2 - alpha))


class LevySde(Sde):
    """Sde view of a Levy model: small jumps become a second Brownian term."""

    def __init__(self, levy, init_value, corr_matrix=None, scale_jump_rate=False, device='cpu', seed=1):
        super().__init__(init_value, levy.dim, 2 * levy.dim, 'indep', corr_matrix)
        self.levy = levy
        self.scale_rate = scale_jump_rate

    def drift(self, t, x):
        return self.levy.drift(t, x) - self.levy.jumps(t, x, 1) * self.levy.gamma()

    def diffusion(self, t, x):
        return torch.stack([self.levy.diffusion(t, x), self.levy.jumps(t, x, 1) * self.levy.beta()], dim=-1)

    def jumps(self, t, x, jumps):
        return self.levy.jumps(t, x, jumps)

    def sample_jumps(self, size, device):
        return self.levy.icdf(torch.rand(size, device=device) + UNIFORM_TOL / 3)

    def jump_rate(self):
        lda = self.levy.icdf.lda
        return torch.tensor(lda * self.levy.dim if self.scale_rate else lda)

    def jump_mean(self):
        return self.levy.jump_mean()


class ExampleLevy(Levy):
    """Exponential-Levy log-price model with correlated diffusion (additive form)."""

    def __init__(self, c_plus, c_minus, alpha, mu, r, sigma, f, chol_corr, epsilon, dim):
        super().__init__(dim, InverseCdf(c_minus, c_plus, mu, alpha, epsilon))
        self.cm, self.cp, self.alpha, self.mu = c_minus, c_plus, alpha, mu
        self.f, self.sigma, self.epsilon = f, sigma, epsilon
        self.jump_comp = torch.tensor([get_jump_comp(c_plus, c_minus, alpha, mu, f[i].item()) for i in range(dim)],
                                      device=f.device)
        self.sigma_matrix = torch.matmul(torch.diag(sigma), chol_corr)
        self.row_sum_sq = (self.sigma_matrix ** 2).sum(-1)

    def drift(self, t, x):
        return -0.5 * self.row_sum_sq - self.jump_comp

    def diffusion(self, t, x):
        return self.sigma * torch.ones_like(x)

    def jumps(self, t, x, jumps):
        return self.f * jumps * torch.ones_like(x)

    def gamma(self):
        return _trunc_gamma(self.cp, self.cm, self.alpha, self.epsilon)

    def beta(self):
        return _trunc_beta(self.cp, self.cm, self.alpha, self.epsilon)

    def jump_mean(self):
        return 0


class ExpExampleLevy(Levy):
    """Multiplicative Levy model dX = r X dt + sigma X dW + f X dL."""

    def __init__(self, c_minus, c_plus, alpha, mu, r, sigma, f, epsilon, dim=1):
        super().__init__(dim, InverseCdf(c_minus, c_plus, mu, alpha, epsilon))
        self.cm, self.cp, self.alpha, self.mu = c_minus, c_plus, alpha, mu
        self.r, self.sigma, self.f, self.epsilon = r, sigma, f, epsilon

    def drift(self, t, x):
        return self.r * x

    def diffusion(self, t, x):
        return x * self.sigma

    def jumps(self, t, x, jumps):
        return self.f * x * jumps

    def gamma(self):
        return _trunc_gamma(self.cp, self.cm, self.alpha, self.epsilon)

    def beta(self):
        return _trunc_beta(self.cp, self.cm, self.alpha, self.epsilon)

    def jump_mean(self):
        return 0


class Levy2d(Levy):
    """Two-dimensional additive Levy example with unit diffusion."""

    def __init__(self, c_plus, c_minus, alpha, mu, f, epsilon):
        super().__init__(2, InverseCdf(c_minus, c_plus, mu, alpha, epsilon))
        self.cp, self.cm, self.alpha, self.mu, self.f, self.epsilon = c_plus, c_minus, alpha, mu, f, epsilon

    def drift(self, t, x):
        return torch.ones_like(x) * (-self.f * (self.cp - self.cm) * (1 / self.mu + 1 / self.mu ** 2))

    def diffusion(self, t, x):
        return torch.ones_like(x)

    def jumps(self, t, x, jumps):
        return self.f * jumps * torch.ones_like(x)

    def gamma(self):
        return _trunc_gamma(self.cp, self.cm, self.alpha, self.epsilon)

    def beta(self):
        return _trunc_beta(self.cp, self.cm, self.alpha, self.epsilon)

    def jump_mean(self):
        if self.cp == self.cm:
            return 0
        mass = (self.cp + self.cm) * (1 / self.mu + (self.epsilon ** (-self.alpha) - 1) / self.alpha)
        return (self.cp - self.cm) * ((1 / self.mu + 1 / self.mu ** 2)
                                      + (1 - self.epsilon ** (1 - self.alpha)) / (1 - self.alpha)) / mass
