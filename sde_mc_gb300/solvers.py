"""Solvers with the reference's interface (sde_mc/solvers.py:9-341).

``solve`` and ``multilevel_solve`` keep the reference's signatures and return
layouts but run on the GPU: the descriptor is lowered once per call and the
materialising kernel (K4) or the coupled MLMC kernel (K2) writes the result.
Each call takes a fresh, disjoint range of path indices from the solver's
counter-based RNG stream (seeded by ``seed``), so repeated calls draw new
paths as the reference's stateful generator does, and a new solver with the
same seed reproduces them exactly.
"""
from abc import ABC, abstractmethod

import torch

from . import _native as N
from . import kernels as K
from .lowering import lower, max_jumps_for
from .schemes import EulerScheme, HestonScheme


class SdeSolver(ABC):
    def __init__(self, sde, time_interval, num_steps, device='cpu', seed=1):
        self.sde = sde
        self.time_interval = time_interval
        self.num_steps = num_steps
        self.device = device
        self.has_jumps = bool(torch.as_tensor(self.sde.jump_rate()).any())
        if len(self.sde.corr_matrix) > 1:
            self.lower_cholesky = torch.linalg.cholesky(self.sde.corr_matrix.to('cpu'))
        else:
            self.lower_cholesky = torch.tensor([[1.]])
        self.seed = int(seed)
        self.path_cursor = 0
        torch.manual_seed(seed)  # the reference seeds torch's global generator here

    def take_paths(self, n):
        """Reserve the next n global path indices of this solver's stream."""
        off = self.path_cursor
        self.path_cursor += int(n)
        return off

    def lower(self, payoff=None, discounter=None, num_paths=0, num_steps=None, path_offset=None):
        off = self.take_paths(num_paths) if path_offset is None else path_offset
        return lower(self, payoff, discounter, num_paths=num_paths, path_offset=off, num_steps=num_steps)

    @abstractmethod
    def solve(self, bs=1, return_normals=False):
        pass

    def multilevel_terminals(self, bs, levels):
        """((paths_fine, paths_coarse), None) with only the initial and terminal
        columns of multilevel_solve's coupled paths (no column storage)."""
        return _multilevel_terminals(self, bs, levels)

    @abstractmethod
    def init_storage(self, bs, steps):
        pass

    def step(self, t, x, h, corr_normals):
        """One scheme step on a host batch (the scheme mixed into a concrete
        solver provides it, as in sde_mc/solvers.py:48, 61, 137)."""
        raise NotImplementedError("a solver's step comes from its scheme (EulerScheme, HestonScheme)")

    def sample_corr_normals(self, size, h, corr=True):
        """Host helper kept for API compatibility: L @ (randn(size) * sqrt(h))."""
        normals = torch.randn(size=size, device=self.device) * torch.sqrt(torch.as_tensor(h))
        if corr:
            return torch.matmul(self.lower_cholesky.to(normals.device), normals).squeeze(-1)
        return normals.squeeze(-1)

    def _out(self, t):
        dev = torch.device(self.device)
        return t if dev.type == 'cuda' else t.to(dev)


class DiffusionSolver(SdeSolver):
    """Uniform grid, exactly num_steps Euler steps (sde_mc/solvers.py:59-119)."""

    def init_storage(self, bs, steps):
        return torch.empty(size=(bs, steps + 1, self.sde.dim), device=self.device)

    def solve(self, bs=1, return_normals=False):
        bs = int(bs)
        inst = self.lower(num_paths=bs)
        out = K.materialise(inst, self.num_steps, want=("paths", "normals", "steps"))
        N.status_error(out["status"].item(), "solve")
        return self._out(out["paths"]), self._out(out["normals"])

    def multilevel_solve(self, bs, levels, return_normals=False):
        """Coupled fine/coarse paths (sde_mc/solvers.py:90-119): ((paths_fine
        (bs, fine + 1, dim), paths_coarse (bs, coarse + 1, dim)), the fine
        increments (bs, fine, dim[, 2]))."""
        bs = int(bs)
        fine, coarse = int(levels[0]), int(levels[1])
        inst = self.lower(num_paths=bs, num_steps=coarse)
        hf, hc = level_steps(self, fine, coarse)
        out = K.mlmc_paths(inst, fine, coarse, hf, hc, (fine + 1, coarse + 1), normals=True)
        N.status_error(out["status"].item(), "multilevel_solve")
        return (self._out(out["paths_fine"]), self._out(out["paths_coarse"])), self._out(out["normals"])


class EulerSolver(EulerScheme, DiffusionSolver):
    pass


class HestonSolver(HestonScheme, DiffusionSolver):
    """Uniform grid with Heston's implicit variance step (sde_mc/solvers.py:126-127);
    the kernels run it as the Heston model kind of the descriptor."""


class JumpDiffusionSolver(SdeSolver):
    """Jump-adapted grid (sde_mc/solvers.py:130-307): the step restarts at every
    jump time; all steps of a batch are stored up to the slowest path."""

    def __init__(self, sde, time_interval, num_steps, device='cpu', seed=1, exact_jumps=False):
        super().__init__(sde, time_interval, num_steps, device, seed)
        self.max_jumps = max_jumps_for(float(torch.as_tensor(self.sde.jump_rate()).float().sum()),
                                       self.time_interval)
        self.exact_jumps = exact_jumps

    def add_jumps(self, t, old_x, x, jumps):
        return x + self.sde.jumps(t, old_x, jumps)

    # Host helpers kept for callers that draw by hand (sde_mc/solvers.py:143-148);
    # the kernels draw the same laws from their own Philox streams.
    def sample_jump_times(self, size):
        """Jump times: cumulative sums along dim 1 of exponential gaps at the
        total jump rate."""
        rate = float(torch.as_tensor(self.sde.jump_rate()).sum())
        return torch.empty(size, device=self.device).exponential_(rate).cumsum(dim=1)

    def sample_one_jump(self, size):
        """One mark per path, repeated over the dimensions: (size, dim)."""
        return self.sde.sample_jumps([size, 1], self.device).repeat(1, self.sde.dim)

    def init_storage(self, bs, steps, low_storage=False):
        paths = torch.zeros(size=(bs, steps + 1, self.sde.dim), device=self.device)
        if low_storage:
            return paths, None, None, None, None
        left = torch.zeros_like(paths)
        jumps = torch.zeros_like(paths)
        time = torch.zeros(size=(bs, steps + 1, 1), device=self.device) + self.time_interval
        if self.sde.diffusion_struct == 'diag':
            normals = torch.zeros(size=(bs, steps, self.sde.dim), device=self.device)
        else:
            normals = torch.zeros(size=(bs, steps, self.sde.dim, int(self.sde.brown_dim / self.sde.dim)),
                                  device=self.device)
        return paths, left, time, jumps, normals

    def solve(self, bs=1, return_normals=False, low_storage=False):
        """Returns (paths[:, :S+1], (normals, time_paths, left_paths, S, jump_paths))
        with S the batch's step count, aux tensors at steps + max_jumps columns."""
        bs = int(bs)
        cap = self.num_steps + self.max_jumps
        inst = self.lower(num_paths=bs)
        want = ("paths", "steps") if low_storage else ("paths", "left", "time", "jumps", "normals", "steps")
        out = K.materialise(inst, cap, want=want)
        st = int(out["status"].item())
        if st:
            N.status_error(st, "JumpDiffusionSolver.solve")
        total = int(out["steps"].max().item()) if bs > 0 else 0
        paths = out["paths"][:, :total + 1]
        if low_storage:
            return self._out(paths), (None, None, None, total, None)
        time = out["time"].unsqueeze(-1)
        # beyond the batch's last step the reference's storage keeps its initial values
        time[:, total + 1:] = float(self.time_interval)
        out["left"][:, total + 1:] = 0.0
        out["jumps"][:, total + 1:] = 0.0
        out["normals"][:, total:] = 0.0
        return self._out(paths), (self._out(out["normals"]), self._out(time), self._out(out["left"]), total,
                                  self._out(out["jumps"]))

    def multilevel_solve(self, bs, levels, return_normals=False):
        """Coupled fine/coarse jump-adapted paths (sde_mc/solvers.py:228-307):
        ((paths_fine, paths_coarse), None), each (bs, total_steps_coarse + 1,
        dim) with the states after every coarse step (a finished path keeps its
        final state).  The estimators (mc_multilevel, get_optimal_trials) read
        only terminal states and run the level kernels directly."""
        bs = int(bs)
        fine, coarse = int(levels[0]), int(levels[1])
        inst = self.lower(num_paths=bs, num_steps=coarse)
        hf, hc = level_steps(self, fine, coarse)
        cols = coarse + int(self.max_jumps) + 1
        out = K.mlmc_paths(inst, fine, coarse, hf, hc, (cols, cols))
        N.status_error(out["status"].item(), "multilevel_solve")
        total = int(out["steps"].max().item()) if bs > 0 else 0
        return (self._out(out["paths_fine"][:, :total + 1]), self._out(out["paths_coarse"][:, :total + 1])), None



def level_steps(solver, fine, coarse):
    """h_fine = fl32(T / fine) and h_coarse = fl32(factor * h_fine) as the
    reference forms them (sde_mc/solvers.py:233-234)."""
    hf = torch.tensor(solver.time_interval / fine)
    hc = (fine // coarse) * hf
    return float(hf), float(hc)


def _multilevel_terminals(solver, bs, levels):
    bs = int(bs)
    fine, coarse = int(levels[0]), int(levels[1])
    dev = N.require_cuda()
    inst = solver.lower(num_paths=bs, num_steps=coarse)
    hf, hc = level_steps(solver, fine, coarse)
    d = inst.dim
    xf = torch.empty((bs, d), dtype=torch.float32, device=dev)
    xc = torch.empty((bs, d), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    import ctypes
    rc = N.load().sdemc_mlmc_terminals(ctypes.byref(inst), fine, coarse, hf, hc, N.ptr(xf), N.ptr(xc),
                                       N.ptr(status), N.stream_handle(dev))
    N.check(rc, "sdemc_mlmc_terminals")
    N.status_error(status.item(), "multilevel_solve")
    x0 = torch.as_tensor(solver.sde.init_value, dtype=torch.float32, device=dev).reshape(1, 1, d).expand(bs, 1, d)
    pf = torch.cat([x0, xf.unsqueeze(1)], 1)
    pc = torch.cat([x0, xc.unsqueeze(1)], 1)
    return (solver._out(pf), solver._out(pc)), None


class JumpEulerSolver(EulerScheme, JumpDiffusionSolver):
    pass


class Grid(ABC):
    def __init__(self, start, end):
        self.start = start
        self.end = end
        self.time_interval = end - start
        self.t = start

    def __iter__(self):
        return self

    @abstractmethod
    def __next__(self):
        pass


class UniformGrid(Grid):
    def __init__(self, start, end, num_steps):
        super().__init__(start, end)
        self.num_steps = num_steps
        self.h = (end - start) / num_steps
        assert self.h > 1e-8

    def __next__(self):
        if self.t > self.end - 1e-8:
            raise StopIteration
        t = self.t
        self.t += self.h
        return t
