"""Time-stepping schemes with the reference's interface (sde_mc/schemes.py:1-22).

``step(t, x, h, corr_normals)`` is kept for user code that steps a batch by
hand; the GPU kernels implement the same Euler update in registers.
"""
import torch

from .helpers import solve_quadratic


class EulerScheme:
    def step(self, t, x, h, corr_normals):
        struct = self.sde.diffusion_struct
        if struct == 'diag':
            return x + self.sde.drift(t, x) * h + self.sde.diffusion(t, x) * corr_normals
        if struct == 'indep':
            return x + self.sde.drift(t, x) * h + (self.sde.diffusion(t, x) * corr_normals).sum(dim=-1)
        # 'general': diffusion (bs, dim, brown_dim) applied to the (bs, brown_dim) increments
        return x + self.sde.drift(t, x) * h + torch.matmul(self.sde.diffusion(t, x),
                                                           corr_normals.unsqueeze(-1)).squeeze(-1)


class HestonScheme:
    """Euler price step with an implicit variance step: sqrt(v_{k+1}) is the
    larger root of a quadratic (full truncation free)."""

    def step(self, t, x, h, corr_normals):
        new = x + self.sde.drift(t, x) * h + self.sde.diffusion(t, x) * corr_normals
        root = solve_quadratic(self.sde.quadratic_parameters(x[:, 1], h, corr_normals[:, 1]))
        new[:, 1] = root * root
        return new
