"""Learned control variates with the reference's interface (sde_mc/varred.py).

The adapted control variate (sde_mc/varred.py:98-199)
    Gamma = payoff + sum_k e^{-r t_k} f(t_k, X_k) . dW_k
                   + sum_k e^{-r t_k} g(t_k, X_k-) . (J_k - lambda E[J] h_k)
is trained and evaluated on the GPU by the library's kernels (K5/K6): BF16
tensor-core forward and backward passes with FP32 accumulation, a
deterministic gradient reduction and a fused Adam step, all on paths the
solver itself generated.  Each network is one kernel pass over its own
(inputs, multipliers): f reads the path and the Brownian increments, g the
left limits and the recorded marks minus their compensator (the last row has
none, as in the reference).  Supported models: ``Mlp(1+d, [64, 64, 64], d)``
(ReLU, no batch norm, d in {1, 2}) for f and g, ``ZeroFunction`` for g.
"""
import math
import time

import numpy as np
import torch

from . import _native as N
from .helpers import partition, remove_steps
from .nets import ZeroFunction


class EarlyStopping:
    """Stop training once the loss gain of an epoch no longer pays for its cost."""

    def __init__(self, eps, quantile, cost_batch, alpha):
        self.eps = eps
        self.quantile = quantile
        self.cost_batch = cost_batch
        self.alpha = alpha
        self.cost_epoch = None
        self.batch_size = None

    def threshold(self):
        return self.alpha * (self.cost_epoch * self.eps ** 2 * self.batch_size) / (self.cost_batch * self.quantile ** 2)

    def stop(self, delta_gamma):
        return delta_gamma < self.threshold()


def integrate_cv(normals, f_out, discounts, diffusion_struct, tol=0, time_interval=None):
    """sum_k sum_i dW_{k,i} f_i discount_k (host torch helper, sde_mc/varred.py:202-214)."""
    if tol != 0:
        assert time_interval is not None
        steps = normals.shape[1]
        new_steps = remove_steps(tol, steps, time_interval)
        normals, f_out, discounts = normals[:, :new_steps], f_out[:, :new_steps], discounts[:, :new_steps]
    if diffusion_struct == 'diag':
        return (normals * f_out * discounts).sum(-1).sum(-1)
    return ((normals * f_out).sum(-1) * discounts).sum(-1).sum(-1)


# --------------------------------------------------------------- GPU side --
class CvData:
    """Contiguous device tensors the kernels read: time (N, S+1), paths
    (N, S+1, d), normals (N, S, d), discounted payoffs (N)."""

    def __init__(self, time_full, paths_full, normals, payoffs, device):
        self.time = time_full.to(device=device, dtype=torch.float32).contiguous()
        self.paths = paths_full.to(device=device, dtype=torch.float32).contiguous()
        self.normals = normals.to(device=device, dtype=torch.float32).contiguous()
        self.payoffs = payoffs.to(device=device, dtype=torch.float32).contiguous()
        self.n = int(self.payoffs.numel())
        self.steps = int(self.normals.shape[1])
        self.dim = int(self.normals.shape[2])
        assert self.time.shape == (self.n, self.steps + 1)
        assert self.paths.shape == (self.n, self.steps + 1, self.dim)

    @classmethod
    def from_dataset(cls, ds, solver, device):
        """Inputs of the Brownian integrand f."""
        if hasattr(ds, "full_time"):  # AdaptedPathData
            return cls(ds.full_time.reshape(ds.full_time.shape[0], -1), ds.full_paths, ds.normals, ds.payoffs, device)
        # NormalPathData (uniform grid): times from partition(T, steps, 'left')
        n, steps = ds.normals.shape[0], ds.normals.shape[1]
        tp = partition(solver.time_interval, steps, ends='left')
        row = torch.cat([tp, torch.tensor([float(solver.time_interval)])]).to(torch.float32)
        return cls(row.unsqueeze(0).expand(n, steps + 1), ds.full_paths, ds.normals, ds.payoffs, device)

    @classmethod
    def jumps_from_dataset(cls, ds, solver, device):
        """Inputs of the jump integrand g (AdaptedPathData): left limits, and
        per row the recorded marks minus lambda E[J] h_k with h = diff(time)
        (sde_mc/varred.py:118-128); no payoff term."""
        if not hasattr(ds, "jump_paths"):
            raise ValueError("the jump integrand needs AdaptedPathData")
        n, S, d = ds.normals.shape
        t = ds.time_paths.reshape(n, S).to(device=device, dtype=torch.float32)
        lam_kappa = torch.as_tensor(solver.sde.jump_rate() * solver.sde.jump_mean(), dtype=torch.float32,
                                    device=device)
        mult = ds.jump_paths.to(device=device, dtype=torch.float32).clone()
        mult[:, :-1, :] -= lam_kappa * torch.diff(t, dim=1).unsqueeze(-1)
        left = ds.left_paths.to(device=device, dtype=torch.float32)
        left_full = torch.cat([left, left[:, -1:]], 1)  # the kernels read rows 0..S-1 of (S+1)
        return cls(ds.full_time.reshape(n, -1), left_full, mult, torch.zeros(n, device=device), device)


def _kernel_dim(net):
    dim = net.kernel_dim() if hasattr(net, "kernel_dim") else None
    if dim is None:
        raise NotImplementedError("the GPU control-variate kernels implement Mlp(1+d, [64, 64, 64], d) with ReLU, "
                                  "no batch norm, d in {1, 2}")
    return dim


def kernel_models(models):
    """[(net, dim, 'f' | 'g')] for the networks the kernels run: f, and g
    unless it is a ZeroFunction.  Raises for architectures without a kernel."""
    if isinstance(models, (list, tuple)):
        f, g = models
    else:
        f, g = models, None
    out = [(f, _kernel_dim(f), "f")]
    if g is not None and not isinstance(g, ZeroFunction):
        out.append((g, _kernel_dim(g), "g"))
    return out


def disc_rate(discounter):
    r = getattr(discounter, "r", None)
    if r is None:
        raise NotImplementedError("control-variate kernels need a ConstantShortRate discounter")
    return float(r)


class GpuCv:
    """Device state of one control-variate network: FP32 parameters, Adam
    moments and the gradient workspace."""

    def __init__(self, f, dim, device):
        self.f, self.dim, self.device = f, dim, device
        self.nparam = N.load().sdemc_cv_nparams(dim)
        self.params = f.flat_params(device)
        assert self.params.numel() == self.nparam
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self.grad = torch.zeros_like(self.params)
        self.nparts = 2 * _sms()
        self.partials = torch.empty((self.nparts, self.nparam), dtype=torch.float32, device=device)
        self._tc_status = None
        self._bwd_status = torch.zeros(1, dtype=torch.int32, device=device)

    def forward(self, data, rate, idx=None, gamma=None, fout=None):
        n = data.n if idx is None else int(idx.numel())
        if gamma is None:
            gamma = torch.empty(n, dtype=torch.float32, device=self.device)
        rc = N.load().sdemc_cv_forward(self.dim, N.ptr(self.params), N.ptr(data.time), N.ptr(data.paths),
                                       N.ptr(data.normals), N.ptr(data.payoffs), N.ptr(idx), n, data.steps,
                                       float(rate), N.ptr(gamma), N.ptr(fout), N.stream_handle(self.device))
        N.check(rc, "sdemc_cv_forward")
        return gamma

    def forward_tc(self, data, rate, idx=None, gamma=None):
        """Gamma through the tcgen05 network kernel (large batches)."""
        n = data.n if idx is None else int(idx.numel())
        if gamma is None:
            gamma = torch.empty(n, dtype=torch.float32, device=self.device)
        lib = N.load()
        need = lib.sdemc_cv_forward_tc_scratch_bytes(n, data.steps)
        # own workspace: the shared scratch pool's header words belong to K1/K10
        if getattr(self, "_tc_scratch", None) is None or self._tc_scratch.numel() < need:
            self._tc_scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=self.device)
        scratch = self._tc_scratch
        status = torch.zeros(1, dtype=torch.int32, device=self.device)
        rc = lib.sdemc_cv_forward_tc(self.dim, N.ptr(self.params), N.ptr(data.time), N.ptr(data.paths),
                                     N.ptr(data.normals), N.ptr(data.payoffs), N.ptr(idx), n, data.steps,
                                     float(rate), N.ptr(gamma), N.ptr(scratch), scratch.numel(), N.ptr(status),
                                     N.stream_handle(self.device))
        N.check(rc, "sdemc_cv_forward_tc")
        self._tc_status = status
        return gamma

    def backward(self, data, rate, gamma, idx=None):
        n = data.n if idx is None else int(idx.numel())
        rc = N.load().sdemc_cv_backward(self.dim, N.ptr(self.params), N.ptr(data.time), N.ptr(data.paths),
                                        N.ptr(data.normals), N.ptr(idx), n, data.steps, float(rate), N.ptr(gamma),
                                        N.ptr(self.partials), self.nparts, N.ptr(self.grad),
                                        N.stream_handle(self.device))
        N.check(rc, "sdemc_cv_backward")
        return self.grad

    def backward_tc(self, data, rate, gamma, idx=None):
        """K6 on tcgen05: the same gradient, every product on the 5th-generation
        tensor cores (the weight gradients accumulated in tensor memory)."""
        n = data.n if idx is None else int(idx.numel())
        rc = N.load().sdemc_cv_backward_tc(self.dim, N.ptr(self.params), N.ptr(data.time), N.ptr(data.paths),
                                           N.ptr(data.normals), N.ptr(idx), n, data.steps, float(rate),
                                           N.ptr(gamma), N.ptr(self.partials), self.nparts, N.ptr(self.grad),
                                           N.ptr(self._bwd_status), N.stream_handle(self.device))
        N.check(rc, "sdemc_cv_backward_tc")
        return self.grad

    def adam(self, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.step_count += 1
        rc = N.load().sdemc_adam_step(N.ptr(self.params), N.ptr(self.grad), N.ptr(self.m), N.ptr(self.v),
                                      self.nparam, self.step_count, float(lr), float(betas[0]), float(betas[1]),
                                      float(eps), N.stream_handle(self.device))
        N.check(rc, "sdemc_adam_step")

    def adam_dev(self, bc, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        """The Adam step with its bias corrections read from device memory
        (``bc``: 2 floats); the caller advances ``step_count``."""
        rc = N.load().sdemc_adam_step_dev(N.ptr(self.params), N.ptr(self.grad), N.ptr(self.m), N.ptr(self.v),
                                          self.nparam, N.ptr(bc), float(lr), float(betas[0]), float(betas[1]),
                                          float(eps), N.stream_handle(self.device))
        N.check(rc, "sdemc_adam_step_dev")

    def write_back(self, opt=None):
        """Copy the trained weights (and Adam state) into the torch objects."""
        self.f.load_flat_params(self.params)
        if opt is not None:
            off = 0
            for lin in self.f.linears():
                for p in (lin.weight, lin.bias):
                    n = p.numel()
                    st = opt.state[p]
                    st["step"] = torch.tensor(float(self.step_count))
                    st["exp_avg"] = self.m[off:off + n].view_as(p).to(p.device).clone()
                    st["exp_avg_sq"] = self.v[off:off + n].view_as(p).to(p.device).clone()
                    off += n


def _sms():
    import ctypes
    v = ctypes.c_int(0)
    N.check(N.load().sdemc_device_sms(ctypes.byref(v)), "sdemc_device_sms")
    return v.value


def adam_hparams(opt):
    if opt is None:
        return 1e-3, (0.9, 0.999), 1e-8
    if not isinstance(opt, torch.optim.Adam):
        raise NotImplementedError("the GPU training step implements torch.optim.Adam")
    grp = opt.param_groups[0]
    if grp.get("weight_decay", 0) or grp.get("amsgrad", False) or grp.get("maximize", False):
        raise NotImplementedError("Adam with weight decay / amsgrad / maximize is not implemented")
    lr = grp["lr"]
    return float(lr if not torch.is_tensor(lr) else lr.item()), tuple(grp["betas"]), float(grp["eps"])


# K6 on tcgen05 for the training gradient (False: the mma.sync kernel)
BACKWARD_TC = True


# True: epochs after the first replay one CUDA graph of the epoch's minibatch
# steps (the same kernels with the same arguments, so the same bits).  Off by
# default: measured on one GB300, the 2^18-path, 10-epoch training took
# 0.313 s with the graph and 0.312 s launched step by step (the loop is bound
# by the gradient kernel, not by the host), and per-request training of 4
# epochs was 3.5 % slower with the capture.
TRAIN_GRAPH = False


def train_gpu(cvs, datas, rate, epochs, batch_size, lr, betas, eps, print_losses=False, early_stopping=None,
              generator=None):
    """Minibatch training of the networks ``cvs`` (one data set each, same
    paths) on Var(Gamma); returns the per-epoch mean losses.  With
    ``TRAIN_GRAPH`` the epochs after the first replay a graph of a whole epoch
    captured once, the permutation and Adam's bias corrections refilled in
    place before each replay; otherwise every step is launched from the host."""
    import ctypes
    n = datas[0].n
    nb = n // batch_size
    if nb < 1:
        raise ValueError("batch size %d larger than the %d training paths" % (batch_size, n))
    dev = cvs[0].device
    lib = N.load()
    perm = torch.empty(n, dtype=torch.int64, device=dev)
    losses = torch.zeros(nb, dtype=torch.float64, device=dev)
    gamma = torch.empty(batch_size, dtype=torch.float32, device=dev)
    use_graph = TRAIN_GRAPH and BACKWARD_TC and epochs > 1
    if use_graph:
        bc_dev = [torch.empty((nb, 2), dtype=torch.float32, device=dev) for _ in cvs]
        bc_host = [torch.empty((nb, 2), dtype=torch.float32, pin_memory=True) for _ in cvs]
    graph = None

    def minibatch(b, adam):
        idx = perm[b * batch_size:(b + 1) * batch_size]
        cvs[0].forward(datas[0], rate, idx, gamma)
        for cv, data in zip(cvs[1:], datas[1:]):
            gamma.add_(cv.forward(data, rate, idx))
        losses[b] = gamma.double().var()
        for cv, data in zip(cvs, datas):
            if BACKWARD_TC:
                cv.backward_tc(data, rate, gamma, idx)
            else:
                cv.backward(data, rate, gamma, idx)
        for j, cv in enumerate(cvs):
            adam(j, cv, b)

    def eager_adam(j, cv, b):
        cv.adam(lr, betas, eps)

    def graph_adam(j, cv, b):
        cv.adam_dev(bc_dev[j][b], lr, betas, eps)

    loss_arr = []
    cost = 0.0
    for epoch in range(epochs):
        t0 = time.time()
        perm.copy_(torch.randperm(n, device=dev, generator=generator))
        if use_graph and epoch > 0:
            if graph is None:
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph):  # records the launches; nothing runs here
                    for b in range(nb):
                        minibatch(b, graph_adam)
            for j, cv in enumerate(cvs):
                base = bc_host[j].data_ptr()
                for b in range(nb):
                    N.check(lib.sdemc_adam_bias(cv.step_count + b + 1, float(betas[0]), float(betas[1]),
                                                ctypes.c_void_p(base + 8 * b)), "sdemc_adam_bias")
                bc_dev[j].copy_(bc_host[j], non_blocking=True)
                cv.step_count += nb
            graph.replay()
        else:
            for b in range(nb):
                minibatch(b, eager_adam)
        loss_arr.append(float(losses.mean()))  # waits for the epoch (and its table copies)
        if BACKWARD_TC:
            for cv in cvs:
                N.status_error(int(cv._bwd_status.item()), "control-variate gradient (tensor cores)")
        if print_losses:
            print('{}: Train loss: {:.5f}     95% confidence interval: {:.5f}'.format(
                epoch, loss_arr[-1], np.sqrt(loss_arr[-1]) * 2 / np.sqrt(n)))
        cost += time.time() - t0
        if early_stopping is not None and epoch > 0:
            early_stopping.cost_epoch = cost / (epoch + 1)
            if early_stopping.stop(loss_arr[epoch - 1] - loss_arr[epoch]):
                break
    return loss_arr


def _gpu_state(f, dim, device):
    st = getattr(f, "_sdemc_gpu", None)
    if st is None or st.device != device:
        st = GpuCv(f, dim, device)
        f._sdemc_gpu = st
    else:
        st.params = f.flat_params(device)
    return st


def _setup(models, dl, solver, device):
    cvs, datas = [], []
    for net, dim, role in kernel_models(models):
        cvs.append(_gpu_state(net, dim, device))
        if role == "f":
            datas.append(CvData.from_dataset(dl.dataset, solver, device))
        else:
            datas.append(CvData.jumps_from_dataset(dl.dataset, solver, device))
    return cvs, datas


TC_MIN_PATHS = 1 << 14  # below this the warp-level mma.sync kernel fills the GPU better


def gamma_gpu(cvs, datas, rate):
    """Gamma of every path of the data sets (payoff + each network's term):
    the tcgen05 network kernel for large sets, the mma.sync one for small."""
    def fwd(cv, data):
        if data.n >= TC_MIN_PATHS:
            out = cv.forward_tc(data, rate)
            N.status_error(int(cv._tc_status.item()), "control-variate network (tensor cores)")
            return out
        return cv.forward(data, rate)
    g = fwd(cvs[0], datas[0]).clone()
    for cv, data in zip(cvs[1:], datas[1:]):
        g += fwd(cv, data)
    return g


def train_adapted_control_variates(models, opt, dl, solver, discounter, epochs=10, print_losses=True, tol=0,
                                   early_stopping=None):
    """Train f (and g) on the dataset of ``dl`` (AdaptedPathData) with Adam;
    returns the per-epoch losses (sde_mc/varred.py:134-199)."""
    if tol != 0:
        raise NotImplementedError("tol != 0 (dropping the last steps) is not implemented on the GPU")
    dev = N.require_cuda()
    cvs, datas = _setup(models, dl, solver, dev)
    lr, betas, eps = adam_hparams(opt)
    losses = train_gpu(cvs, datas, disc_rate(discounter), epochs, int(dl.batch_size), lr, betas, eps, print_losses,
                       early_stopping)
    for cv in cvs:
        cv.write_back(opt)
    return losses


def apply_adapted_control_variates(models, dl, solver, discounter, tol=0):
    """(sum Gamma, sum Gamma^2) over the dataset of ``dl`` (sde_mc/varred.py:98-131)."""
    if tol != 0:
        raise NotImplementedError("tol != 0 is not implemented on the GPU")
    dev = N.require_cuda()
    cvs, datas = _setup(models, dl, solver, dev)
    g = gamma_gpu(cvs, datas, disc_rate(discounter)).double()
    return g.sum(), (g * g).sum()


def train_diffusion_control_variate(model, opt, dl, solver, discounter, epochs, print_losses=True, tol=0,
                                    early_stopping=None):
    """Uniform-grid variant (sde_mc/varred.py:23-72); returns (time, losses)."""
    start = time.time()
    if tol != 0:
        raise NotImplementedError("tol != 0 is not implemented on the GPU")
    dev = N.require_cuda()
    cvs, datas = _setup(model, dl, solver, dev)
    lr, betas, eps = adam_hparams(opt)
    losses = train_gpu(cvs, datas, disc_rate(discounter), epochs, int(dl.batch_size), lr, betas, eps, print_losses,
                       early_stopping)
    for cv in cvs:
        cv.write_back(opt)
    return time.time() - start, losses


def apply_diffusion_control_variate(model, dl, solver, discounter, tol=0):
    if tol != 0:
        raise NotImplementedError("tol != 0 is not implemented on the GPU")
    dev = N.require_cuda()
    cvs, datas = _setup(model, dl, solver, dev)
    g = gamma_gpu(cvs, datas, disc_rate(discounter)).double()
    return g.sum(), (g * g).sum()


def fused_supported(models, solver, discounter, tol=0):
    """True when K7 (paths + payoff + f in one pass) can price the control
    variate: f a supported Mlp, g = ZeroFunction, diagonal noise, d in {1, 2},
    a constant short rate and no dropped steps."""
    if tol != 0 or getattr(discounter, "r", None) is None:
        return False
    try:
        nets = kernel_models(models)
    except NotImplementedError:
        return False
    if len(nets) != 1:
        return False
    from .lowering import lower
    try:
        inst = lower(solver, None, discounter, num_paths=1)
    except NotImplementedError:
        return False
    return inst.noise == N.NOISE_DIAG and inst.dim in (1, 2) and inst.dim == nets[0][1]


def fused_cv_stats(models, solver, payoff, discounter, trials, gamma=None):
    """K7 over ``trials`` fresh paths of the solver's stream: returns the
    float64 tensor (sum G, sum G^2, n, sum P, sum P^2, mean G, var G, status)."""
    from . import kernels as K
    (f, dim, _), = kernel_models(models)
    dev = N.require_cuda()
    cv = _gpu_state(f, dim, dev)
    inst = solver.lower(payoff, discounter, num_paths=int(trials))
    return K.price_cv(inst, cv.params, disc_rate(discounter), gamma=gamma)
