"""Host-side helpers with the reference's names (sde_mc/helpers.py:1-138)."""
import math

import numpy as np
import torch
from scipy.integrate import quad


def partition(interval, steps, ends='right', device='cpu'):
    """Grid interval*i/steps; ``ends`` picks which end points are kept."""
    assert ends in ['right', 'left', 'both', 'none']
    lo = 0 if ends in ('left', 'both') else 1
    hi = steps + 1 if ends in ('right', 'both') else steps
    return torch.tensor([interval * i / steps for i in range(lo, hi)], device=device)


def solve_quadratic(coefficients):
    """Larger root of a x^2 + b x + c, batched over tensors (a, b, c)."""
    a, b, c = coefficients
    disc = torch.sqrt(b * b - 4 * a * c)
    return torch.maximum((-b + disc) / (2 * a), (-b - disc) / (2 * a))


def mc_estimates(run_sum, run_sum_squares, n):
    """Sample mean and unbiased sample variance from running sums."""
    mean = run_sum / n
    var = (run_sum_squares - run_sum * run_sum / n) / (n - 1)
    return mean, var


def remove_steps(time_tol, steps, time_interval):
    """Index of the last step once ``time_tol`` is cut from the end of the interval."""
    return int(np.floor(steps - time_tol / (time_interval / steps)))


def get_corr_matrix(rhos):
    """Correlation matrix from its strict upper triangle (row-major); checks it is PD."""
    rhos_t = torch.tensor(rhos)
    m = len(rhos)
    n = int(round((1 + math.sqrt(1 + 8 * m)) / 2))
    if n * (n - 1) // 2 != m:
        raise AssertionError("Length of correlation vector is not triangular")
    corr = torch.eye(n)
    iu = torch.triu_indices(row=n, col=n, offset=1)
    corr[iu[0], iu[1]] = rhos_t
    corr = corr + torch.triu(corr, 1).t()
    try:
        torch.linalg.cholesky(corr)
    except Exception:
        raise RuntimeError('Matrix is not positive semidefinite')
    return corr


def ceil_mult(x, n):
    """Smallest multiple of n not below x."""
    return int(np.ceil(float(x) / n) * n)


def get_jump_comp(c_plus, c_minus, alpha, mu, f):
    """Compensator integral of exp(f x) - 1 (- f x near 0) against the tempered
    stable Levy measure used by the Levy examples."""
    def near(x):
        return np.exp(f * x) - 1 - f * x

    def far(x):
        return np.exp(f * x) - 1

    def tail(x):
        return np.exp(-mu * (np.abs(x) - 1))

    def power(x):
        return np.abs(x) ** (-alpha - 1)

    return (quad(lambda x: c_minus * far(x) * tail(x), -np.inf, -1)[0]
            + quad(lambda x: c_minus * near(x) * power(x), -1, 0)[0]
            + quad(lambda x: c_plus * near(x) * power(x), 0, 1)[0]
            + quad(lambda x: c_plus * far(x) * tail(x), 1, np.inf)[0])


def sample_cov(x, y):
    return torch.sum((x - x.mean()) * (y - y.mean())) / (len(x) - 1)
