"""Payoffs, discounting and closed-form prices (sde_mc/options.py:1-337).

Option classes keep the reference's interface — ``Option.__call__(x)`` =
``payoff(transform(x))`` on (bs, dim) terminal states — for host-side use and
for lowering into the kernels' fused payoff epilogue.  The closed forms are
FP64 host functions used as pricing oracles.
"""
from abc import ABC, abstractmethod
import math

import numpy as np
import torch
from scipy.stats import lognorm, norm


def bs_binary_aon(spot, strike, expiry, r, sigma):
    """Black-Scholes value of the asset-or-nothing quantity N(d1) the reference
    integrates numerically (sde_mc/options.py:8-32)."""
    d1 = (np.log(spot / strike) + (r + 0.5 * sigma * sigma) * expiry) / (np.sqrt(expiry) * sigma)
    return float(norm.cdf(d1))


def bs_call(spot, strike, expiry, r, sigma):
    """Black-Scholes European call."""
    sd = sigma * np.sqrt(expiry)
    d1 = (np.log(spot / strike) + (r + 0.5 * sigma ** 2) * expiry) / sd
    return spot * norm.cdf(d1) - strike * np.exp(-r * expiry) * norm.cdf(d1 - sd)


def merton_call(spot, strike, expiry, r, sigma, alpha, gamma, rate):
    """Merton jump-diffusion call as the Poisson mixture of Black-Scholes prices
    (40 terms): term k uses r_k = r - rate*beta + k log(1+beta)/T and
    sigma_k^2 = sigma^2 + k gamma^2/T, weighted by Poisson((1+beta) rate T)."""
    beta = np.exp(alpha + 0.5 * gamma * gamma) - 1
    lam = (beta + 1) * rate * expiry
    total = 0.0
    for k in range(40):
        r_k = r - rate * beta + k * np.log(beta + 1) / expiry
        sigma_k = np.sqrt(sigma ** 2 + k * gamma ** 2 / expiry)
        total += np.exp(-lam) * lam ** k / math.factorial(k) * bs_call(spot, strike, expiry, r_k, sigma_k)
    return total


def bs_digital_call(spot, strike, expiry, r, sigma):
    """Black-Scholes cash-or-nothing call (lognormal terminal law)."""
    mn = np.log(spot) + (r - 0.5 * sigma * sigma) * expiry
    sd = sigma * np.sqrt(expiry)
    return (1 - lognorm.cdf(strike, s=sd, scale=np.exp(mn))) * np.exp(-r * expiry)


def bs_asian_call(spot, strike, expiry, r, sigma):
    """Geometric-average Asian call under Black-Scholes."""
    sig_g = sigma / np.sqrt(3)
    b = 0.5 * (r - 0.5 * sig_g ** 2)
    sd = sig_g * np.sqrt(expiry)
    d1 = (np.log(spot / strike) + (b + sig_g ** 2 / 2) * expiry) / sd
    return spot * np.exp((b - r) * expiry) * norm.cdf(d1) - strike * np.exp(-r * expiry) * norm.cdf(d1 - sd)


class Option(ABC):
    """Payoff of the terminal state; ``log`` exponentiates the state first and
    ``discount`` scales it before the payoff is applied."""

    def __init__(self, log=False, discount=1):
        self.log = log
        self.discount = discount

    def transform(self, x):
        return self.discount * (torch.exp(x) if self.log else x)

    @abstractmethod
    def payoff(self, x):
        pass

    def __call__(self, x):
        return self.payoff(self.transform(x))


def _zero_like(v):
    return torch.tensor(0., dtype=v.dtype, device=v.device)


class EuroCall(Option):
    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x[:, 0]
        return torch.where(s > self.strike, s - self.strike, _zero_like(s))


class EuroPut(Option):
    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x[:, 0]
        return torch.where(s < self.strike, self.strike - s, _zero_like(s))


class BinaryAoN(Option):
    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x[:, 0]
        return torch.where(s >= self.strike, s, torch.tensor(0, dtype=s.dtype, device=s.device))


class Basket(Option):
    """Call on the arithmetic or geometric average of the components."""

    def __init__(self, strike, average_type='arithmetic', log=False, discount=1):
        assert average_type in ['arithmetic', 'geometric']
        super().__init__(log, discount)
        self.strike = strike
        self.average_type = average_type

    def payoff(self, x):
        s = x.mean(1) if self.average_type == 'arithmetic' else torch.exp(torch.log(x).mean(1))
        return torch.where(s > self.strike, s - self.strike, _zero_like(s))


class Rainbow(Option):
    """Call on the maximum of the components."""

    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x.max(1).values
        return torch.where(s > self.strike, s - self.strike, _zero_like(s))


class Digital(Option):
    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x[:, 0]
        return torch.where(s > self.strike, torch.ones_like(s), torch.zeros_like(s))


class AsianCall(Option):
    """Call on the time average carried in component 1 (see AsianWrapper)."""

    def __init__(self, time_interval, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.time_interval = time_interval
        self.strike = strike

    def payoff(self, x):
        a = x[:, 1] / self.time_interval
        s = torch.exp(a) if self.log else a
        return torch.where(s > self.strike, s - self.strike, _zero_like(s))


class HestonRainbow(Option):
    """Call on the maximum of the even (price) components of stacked Heston states."""

    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        s = x[:, 0::2].max(1).values
        return torch.where(s > self.strike, s - self.strike, _zero_like(s))


class BestOf(Option):
    def __init__(self, strike, log=False, discount=1):
        super().__init__(log, discount)
        self.strike = strike

    def payoff(self, x):
        best = torch.max(x, dim=1).values
        return torch.maximum(best, self.strike * torch.ones_like(best))


class ConstantShortRate:
    """Discount factor exp(-r t)."""

    def __init__(self, r):
        self.r = r

    def __call__(self, t):
        if not torch.is_tensor(t):
            t = torch.tensor(t)
        return torch.exp(-t * self.r)
