"""SDE model plug-ins with the reference's interface (sde_mc/sde.py:6-406).

Each class keeps the reference's constructor signature, attributes
(``init_value, dim, brown_dim, diffusion_struct, corr_matrix``) and methods
(``drift, diffusion, jumps, sample_jumps, jump_mean, jump_rate``) so user code
and presets run unchanged.  The methods are plain torch and are only called by
user code or by the descriptor lowering; the solvers never step paths through
them — the GPU kernels use the lowered affine coefficients instead.
"""
from abc import ABC, abstractmethod
import math

import numpy as np
import torch


class Sde(ABC):
    """Abstract SDE driven by a Brownian motion and a Poisson random measure.

    ``diffusion_struct`` is 'diag' (diffusion (bs, dim), brown_dim == dim),
    'indep' (several independent dim-dimensional Brownian motions, diffusion
    (bs, dim, brown_dim/dim)) or 'general' (sde_mc/sde.py:20-32).
    """

    def __init__(self, init_value, dim, brown_dim, diffusion_struct, corr_matrix=None, method='euler'):
        self.init_value = init_value
        self.dim = dim
        self.brown_dim = brown_dim
        self.diffusion_struct = diffusion_struct
        self.simulation_method = method
        self.corr_matrix = corr_matrix if corr_matrix is not None else torch.eye(dim)

    @abstractmethod
    def drift(self, t, x):
        """Drift vector at (t, x): (bs, dim)."""

    @abstractmethod
    def diffusion(self, t, x):
        """Diffusion at (t, x); shape set by diffusion_struct."""

    @abstractmethod
    def jumps(self, t, x, jumps):
        """Jump coefficient at (t, x) for marks ``jumps``: (bs, dim)."""

    @abstractmethod
    def sample_jumps(self, size, device):
        """Draw marks of the given shape."""

    @abstractmethod
    def jump_mean(self):
        """Mean of a mark."""

    @abstractmethod
    def jump_rate(self):
        """Intensity of the driving Poisson process (scalar or per component)."""


class DiffusionSde(Sde):
    """SDE without jumps (sde_mc/sde.py:155-176)."""

    def jumps(self, t, x, jumps):
        return None

    def sample_jumps(self, size, device):
        return None

    def jump_mean(self):
        return None

    def jump_rate(self):
        return torch.tensor(0)


class Gbm(DiffusionSde):
    """Correlated geometric Brownian motion: dX = mu X dt + sigma X dW."""

    def __init__(self, mu, sigma, init_value, dim, corr_matrix=None, method='euler'):
        super().__init__(init_value, dim, dim, 'diag', corr_matrix, method)
        self.mu = mu
        self.sigma = sigma

    def drift(self, t, x):
        return self.mu * x

    def diffusion(self, t, x):
        return self.sigma * x


class LogGbm(Gbm):
    """log of a one-dimensional GBM: dY = (mu - sigma^2/2) dt + sigma dW."""

    def __init__(self, mu, sigma, init_value):
        super().__init__(mu, sigma, init_value, 1)

    def drift(self, t, x):
        return (self.mu - 0.5 * self.sigma * self.sigma) * torch.ones_like(x)

    def diffusion(self, t, x):
        return self.sigma * torch.ones_like(x)


class DoubleGbm(DiffusionSde):
    """GBM driven by two independent dim-dimensional Brownian motions ('indep')."""

    def __init__(self, mu, sigma1, sigma2, init_value, dim, corr_matrix=None, method='euler'):
        super().__init__(init_value, dim, 2 * dim, 'indep', corr_matrix, method)
        self.mu = mu
        self.sigma1 = sigma1
        self.sigma2 = sigma2

    def drift(self, t, x):
        return self.mu * x

    def diffusion(self, t, x):
        return torch.stack([self.sigma1 * x, self.sigma2 * x], dim=-1)


class Heston(DiffusionSde):
    """Heston stochastic volatility (price, variance) with an implicit variance step."""

    def __init__(self, r, kappa, theta, xi, rho, init_value):
        assert 2 * kappa * theta > xi ** 2, "Feller condition 2*kappa*theta > xi^2 violated"
        super().__init__(init_value, 2, 2, 'diag', torch.tensor([[1., rho], [rho, 1.]]))
        self.simulation_method = 'heston'
        self.r = r
        self.kappa = kappa
        self.theta = theta
        self.xi = xi

    def drift(self, t, x):
        return torch.stack([self.r * x[:, 0], torch.zeros_like(x[:, 1])], dim=1)

    def diffusion(self, t, x):
        return torch.stack([torch.sqrt(x[:, 1]) * x[:, 0], torch.zeros_like(x[:, 1])], dim=1)

    def quadratic_parameters(self, x, h, normals):
        a = -torch.ones_like(x) - self.kappa * h
        b = self.xi * normals
        c = x + self.kappa * self.theta * h - 0.5 * h * self.xi ** 2
        return a, b, c


class LogNormalJumpsSde(Sde):
    """SDE whose marks are exp(N(alpha, gamma)) - 1."""

    def __init__(self, rate, alpha, gamma, init_value, dim, brown_dim, diffusion_struct, corr_matrix=None,
                 method='euler'):
        super().__init__(init_value, dim, brown_dim, diffusion_struct, corr_matrix, method)
        self.rate = rate if torch.is_tensor(rate) else torch.tensor(rate)
        self.alpha = alpha
        self.gamma = gamma

    def sample_jumps(self, size, device):
        return torch.exp(torch.randn(size=size, device=device) * self.gamma + self.alpha) - 1

    def jump_mean(self):
        return np.exp(self.alpha + 0.5 * self.gamma * self.gamma) - 1

    def jump_rate(self):
        return self.rate


class Merton(LogNormalJumpsSde):
    """Merton jump diffusion: GBM with common shifted-lognormal jumps, compensated drift."""

    def __init__(self, mu, sigma, rate, alpha, gamma, init_value, dim, corr_matrix=None, method='euler'):
        self.mu = mu
        self.sigma = sigma
        super().__init__(rate, alpha, gamma, init_value, dim, dim, 'diag', corr_matrix, method)

    def drift(self, t, x):
        return (self.mu - self.rate * self.jump_mean()) * x

    def diffusion(self, t, x):
        return self.sigma * x

    def jumps(self, t, x, jumps):
        return x * jumps


class IndependentJumpsMerton(Sde):
    """Merton basket whose assets jump independently (no counterpart class in the
    reference; its tests express the same law through a superposition adapter).

    Asset k has its own compound Poisson process of intensity ``rates[k]`` with
    marks exp(N(alpha, gamma)) - 1 and drift compensator mu - rates[k]*kappa.
    ``jump_rate()`` returns the per-asset intensities; their sum drives the
    solver's single jump clock and each event moves one asset, picked with
    probability rates[k] / sum(rates) — a superposition equal in law to
    independent per-asset jumps.  Marks are encoded as ``asset + (1 + J)``
    scaled into one float by :meth:`sample_jumps` only for host-side use.
    """

    def __init__(self, mu, sigma, rates, alpha, gamma, init_value, dim, corr_matrix=None, method='euler'):
        super().__init__(init_value, dim, dim, 'diag', corr_matrix, method)
        self.mu = mu
        self.sigma = sigma
        self.rates = torch.as_tensor(rates, dtype=torch.float32).reshape(-1).expand(dim).clone()
        self.alpha = alpha
        self.gamma = gamma

    def jump_mean(self):
        return math.exp(self.alpha + 0.5 * self.gamma * self.gamma) - 1

    def jump_rate(self):
        return self.rates

    def drift(self, t, x):
        return (self.mu - self.rates * self.jump_mean()) * x

    def diffusion(self, t, x):
        return self.sigma * x

    def jumps(self, t, x, jumps):
        # jumps: (bs, dim) with the mark in the picked asset's column, 0 elsewhere
        return x * jumps

    def sample_jumps(self, size, device):
        """Draw (bs, dim) marks: one picked asset per row carries exp(N)-1."""
        bs = int(size[0])
        pick = torch.multinomial(self.rates / self.rates.sum(), bs, replacement=True).to(device)
        marks = torch.exp(torch.randn(bs, device=device) * self.gamma + self.alpha) - 1
        out = torch.zeros((bs, self.dim), device=device)
        out[torch.arange(bs, device=device), pick] = marks
        return out


class AsianWrapper(Sde):
    """Wraps a 1-D SDE and carries the running integral of the path (Asian options)."""

    def __init__(self, base_sde):
        super().__init__(torch.cat([base_sde.init_value, torch.tensor([0.])]), 2, 2, 'diag', None,
                         base_sde.simulation_method)
        self.base_sde = base_sde

    def drift(self, t, x):
        return torch.stack([self.base_sde.drift(t, x[:, 0]), x[:, 0]], dim=1)

    def diffusion(self, t, x):
        return torch.stack([self.base_sde.diffusion(t, x[:, 0]), torch.zeros_like(x[:, 0])], dim=1)

    def jumps(self, t, x, jumps):
        return torch.stack([self.base_sde.jumps(t, x[:, 0], jumps[:, 0]), torch.zeros_like(x[:, 0])], dim=1)

    def sample_jumps(self, size, device):
        return self.base_sde.sample_jumps(size, device)

    def jump_mean(self):
        return self.base_sde.jump_mean()

    def jump_rate(self):
        return self.base_sde.jump_rate()
