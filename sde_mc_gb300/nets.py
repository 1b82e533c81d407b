"""Control-variate networks and path datasets (sde_mc/nets.py:1-228).

``Mlp`` keeps the reference's constructor and ``nn.Module`` behaviour.  When its
architecture is the one the GPU kernels implement — ReLU hidden layers of 64,
64, 64, no batch norm, no final activation, 1 + d inputs and d outputs with
d in {1, 2} — the control-variate functions in :mod:`sde_mc_gb300.varred`
train and evaluate it with the library's tensor-core kernels; its parameters
are packed into one FP32 device vector (:meth:`Mlp.flat_params`) and written
back after training (:meth:`Mlp.load_flat_params`).
"""
import torch
import torch.nn as nn
import torch.optim as optim
from torch.utils.data import Dataset


class ControlVariate(nn.Module):
    """Base class of control-variate models; ``sequential`` models take whole paths."""

    def __init__(self, sequential, device):
        super().__init__()
        self.sequential = sequential
        self.device = device


class ZeroFunction(ControlVariate):
    """Maps any input to zeros of width ``output_dim`` (switches a CV term off)."""

    def __init__(self, output_dim):
        super().__init__(sequential=False, device=None)
        self.output_dim = output_dim

    def forward(self, x):
        return torch.zeros((x.shape[0], self.output_dim), device=x.device)


class Mlp(ControlVariate):
    """Multilayer perceptron with optional batch norm (reference defaults)."""

    def __init__(self, input_size, layer_sizes, output_size, activation=nn.ReLU, final_activation=None,
                 batch_norm=True, batch_norm_init=True, device='cpu'):
        assert len(layer_sizes) > 0, "At least one hidden layer required."
        super().__init__(sequential=False, device=device)
        self.num_layers = len(layer_sizes)
        self.input_size, self.layer_sizes, self.output_size = input_size, list(layer_sizes), output_size
        self.activation, self.final_activation = activation, final_activation
        self.batch_norm, self.batch_norm_init = batch_norm, batch_norm_init
        layers = []
        if batch_norm_init:
            layers.append(nn.BatchNorm1d(input_size, device=device))
        layers.append(nn.Linear(input_size, layer_sizes[0], device=device))
        if batch_norm:
            layers.append(nn.BatchNorm1d(layer_sizes[0], device=device))
        layers.append(activation())
        for i in range(self.num_layers - 1):
            layers.append(nn.Linear(layer_sizes[i], layer_sizes[i + 1], device=device))
            if batch_norm:
                layers.append(nn.BatchNorm1d(layer_sizes[i + 1], device=device))
            layers.append(activation())
        layers.append(nn.Linear(layer_sizes[-1], output_size, device=device))
        if final_activation is not None:
            layers.append(final_activation())
        self.net = nn.Sequential(*layers)

    def forward(self, x):
        return self.net(x)

    # ------------------------------------------------ GPU kernel support ----
    def kernel_dim(self):
        """d if the kernels implement this network (else None)."""
        ok = (not self.batch_norm and not self.batch_norm_init and self.layer_sizes == [64, 64, 64]
              and self.activation is nn.ReLU and self.final_activation is None
              and self.output_size in (1, 2) and self.input_size == self.output_size + 1)
        return self.output_size if ok else None

    def linears(self):
        return [m for m in self.net if isinstance(m, nn.Linear)]

    def flat_params(self, device):
        """Parameters as one FP32 vector in (W1, b1, W2, b2, W3, b3, W4, b4) order."""
        parts = []
        for lin in self.linears():
            parts += [lin.weight.detach().reshape(-1), lin.bias.detach().reshape(-1)]
        return torch.cat(parts).to(device=device, dtype=torch.float32).contiguous()

    def load_flat_params(self, vec):
        off = 0
        with torch.no_grad():
            for lin in self.linears():
                for p in (lin.weight, lin.bias):
                    n = p.numel()
                    p.copy_(vec[off:off + n].view_as(p).to(p.device, p.dtype))
                    off += n


class Lstm(ControlVariate):
    """Sequential LSTM control variate (host torch module; no GPU kernel)."""

    def __init__(self, in_dim, hidden_dim, out_dim, device='cpu'):
        super().__init__(sequential=True, device=device)
        self.in_dim, self.hidden_dim, self.out_dim = in_dim, hidden_dim, out_dim
        self.lstm = nn.LSTM(in_dim, hidden_dim, batch_first=True).to(device)
        self.lin = nn.Linear(hidden_dim, out_dim).to(device)

    def forward(self, x):
        out, _ = self.lstm(x, self.init_hidden(x.shape[0]))
        return self.lin(out)

    def init_hidden(self, bs):
        z = torch.zeros((1, bs, self.hidden_dim), device=self.device)
        return z, z.clone()


class Gru(ControlVariate):
    """Sequential GRU control variate (host torch module; no GPU kernel)."""

    def __init__(self, in_dim, hidden_dim, out_dim, device='cpu'):
        super().__init__(sequential=True, device=device)
        self.in_dim, self.hidden_dim, self.out_dim = in_dim, hidden_dim, out_dim
        self.gru = nn.GRU(in_dim, hidden_dim, batch_first=True).to(device)
        self.lin = nn.Linear(hidden_dim, out_dim).to(device)

    def forward(self, x):
        out, _ = self.gru(x, self.init_hidden(x.shape[0]))
        return self.lin(out)

    def init_hidden(self, bs):
        return torch.zeros((1, bs, self.hidden_dim), device=self.device)


class NormalPathData(Dataset):
    """(paths without the last column, normals), payoffs — diffusion solvers."""

    def __init__(self, paths, payoffs, normals):
        self.paths = paths[:, :-1]
        self.payoffs = payoffs
        self.normals = normals
        self.full_paths = paths

    def __len__(self):
        return len(self.payoffs)

    def __getitem__(self, idx):
        return (self.paths[idx], self.normals[idx]), self.payoffs[idx]


class NormalJumpsPathData(Dataset):
    def __init__(self, paths, payoffs, normals, jumps):
        self.paths = paths[:, :-1]
        self.payoffs = payoffs
        self.normals = normals
        self.jumps = jumps

    def __len__(self):
        return len(self.payoffs)

    def __getitem__(self, idx):
        return (self.paths[idx], self.normals[idx], self.jumps[idx]), self.payoffs[idx]


class AdaptedPathData(Dataset):
    """Jump-adapted paths, normals, left limits, time grid and marks without the
    last column (sde_mc/nets.py:192-207).  ``full_paths``/``full_time`` keep the
    (N, S+1, ...) tensors the kernels read."""

    def __init__(self, paths, payoffs, normals, left_paths, time_paths, jump_paths, total_steps):
        self.paths = paths[:, :-1]
        self.payoffs = payoffs
        self.normals = normals
        self.left_paths = left_paths[:, :-1]
        self.time_paths = time_paths[:, :-1]
        self.jump_paths = jump_paths[:, :-1]
        self.total_steps = total_steps
        self.full_paths = paths
        self.full_time = time_paths
        self._full_left = left_paths
        self._full_jumps = jump_paths

    def __len__(self):
        return len(self.payoffs)

    def __getitem__(self, idx):
        return (self.paths[idx], self.normals[idx], self.left_paths[idx],
                self.time_paths[idx], self.jump_paths[idx]), self.payoffs[idx]

    # ------------------------------------------------------- export/import --
    def tensors(self):
        """The full tensors (paths, payoffs, normals, left, time, jumps) as
        materialised, last column included; on the device they were made on
        (a DataLoader over this dataset hands them out without a copy)."""
        return dict(paths=self.full_paths, payoffs=self.payoffs, normals=self.normals,
                    left_paths=self._full_left, time_paths=self.full_time, jump_paths=self._full_jumps,
                    total_steps=int(self.total_steps))

    def save(self, path):
        """Write the dataset to a ``.pt`` file (CPU tensors)."""
        torch.save({k: (v.detach().cpu() if torch.is_tensor(v) else v) for k, v in self.tensors().items()}, path)

    @classmethod
    def load(cls, path, device="cpu"):
        """Read a dataset written by :meth:`save` (onto ``device``)."""
        d = torch.load(path, map_location=device, weights_only=True)
        return cls(d["paths"], d["payoffs"], d["normals"], d["left_paths"], d["time_paths"], d["jump_paths"],
                   d["total_steps"])


def get_mlps(problem, num_layers, hidden_size, device):
    d = problem.dim() + 1
    brown_dim = problem.solver.sde.brown_dim
    layers = [hidden_size + d for _ in range(num_layers)]
    f = Mlp(d, layers, brown_dim, batch_norm=False, device=device)
    if problem.solver.has_jumps:
        g = Mlp(d, layers, d - 1, batch_norm=False, device=device)
        return [f, g]
    return f


def get_opt(models):
    if isinstance(models, list):
        return optim.Adam(list(models[0].parameters()) + list(models[1].parameters()))
    return optim.Adam(models.parameters())
