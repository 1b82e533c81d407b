"""Generate the golden fixtures in this folder from the reference itself.

Run in a container where the reference sde_mc package is importable (it is
NOT available where the GPU tests run; the fixtures are committed instead):

    python tests/golden/make_golden.py --ref /path/to/sde_mc_checkout

It records, by wrapping the solver's own methods, every draw the reference
feeds its time-stepping loop (scheme increments, per-step marks, cumulative
jump times) together with the outputs (paths, time grid, left limits, jump
marks, payoffs), so a replay on the GPU can be compared element by element.
It also stores known-answer values of the closed-form prices, payoffs and
helpers, small-sample estimator statistics and an MLP/variance-loss/Adam case.
Seeds are fixed; all arrays are float32 unless the reference computes FP64.
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(path):
    sys.dont_write_bytecode = True
    sys.path.insert(0, path)
    np.math = math  # the reference calls np.math.factorial (removed in NumPy 2)
    import sde_mc  # noqa: E402
    return sde_mc


# ----------------------------------------------------------------- recorder --
class Recorder:
    """Wraps solver.step / sample_one_jump / sample_jump_times on one solver."""

    def __init__(self, solver):
        self.solver = solver
        self.steps = []   # (h, corr_normals) per scheme call
        self.marks = []   # (bs, dim) per sample_one_jump call
        self.jump_times = None
        self._orig = (solver.step, getattr(solver, "sample_one_jump", None),
                      getattr(solver, "sample_jump_times", None))
        step, one, jt = self._orig

        def rec_step(t, x, h, corr_normals):
            self.steps.append((h.clone(), corr_normals.clone()))
            return step(t, x, h, corr_normals)
        solver.step = rec_step
        if one is not None:
            def rec_one(size):
                out = one(size)
                self.marks.append(out.clone())
                return out
            solver.sample_one_jump = rec_one
        if jt is not None:
            def rec_jt(size):
                out = jt(size)
                self.jump_times = out.clone()
                return out
            solver.sample_jump_times = rec_jt

    def restore(self):
        step, one, jt = self._orig
        self.solver.step = step
        if one is not None:
            self.solver.sample_one_jump = one
        if jt is not None:
            self.solver.sample_jump_times = jt


def make_indep_merton(sde_mc, torch, r, sig, lam, a, g, rho, dim=2):
    """Per-asset independent compound Poisson jumps as one superposed clock:
    the scalar mark encodes the asset k and the factor Y as 10k + (Y + 1)."""

    class IndepMerton(sde_mc.Sde):
        def __init__(s):
            corr = torch.full((dim, dim), rho)
            corr.fill_diagonal_(1.0)
            super().__init__(torch.ones(dim), dim, dim, 'diag', corr)
            s.r, s.sig, s.lam, s.a, s.g = r, torch.tensor(sig), torch.tensor(lam), a, g
            s.kappa = math.exp(a + 0.5 * g * g) - 1

        def drift(s, t, x):
            return (s.r - s.lam * s.kappa) * x

        def diffusion(s, t, x):
            return s.sig * x

        def jumps(s, t, x, m):
            k = torch.floor(m / 10.)
            y = m - 10. * k - 1.
            onehot = (k == torch.arange(float(dim))).float()
            return x * y * onehot * (m != 0)

        def sample_jumps(s, size, device):
            k = torch.multinomial(s.lam / s.lam.sum(), int(np.prod(size)), replacement=True).float().view(size)
            return 10. * k + (torch.randn(size) * s.g + s.a).exp()

        def jump_mean(s):
            return s.kappa

        def jump_rate(s):
            return s.lam

    return IndepMerton()


def decode_indep_mark(torch, m):
    """The adapter's own float32 decode of the encoded mark (asset, factor)."""
    m = torch.as_tensor(m)
    k = torch.floor(m / 10.)
    y = m - 10. * k - 1.
    return k.to(torch.int32), y


def jump_replay_case(sde_mc, torch, solver, bs, payoff, disc, seed, one_asset=False):
    torch.manual_seed(seed)
    rec = Recorder(solver)
    paths, (normals, time_paths, left_paths, total_steps, jump_paths) = solver.solve(bs)
    rec.restore()
    S = int(total_steps)
    dts = torch.stack([h.reshape(bs) for h, _ in rec.steps], 1)
    dws = torch.stack([cn for _, cn in rec.steps], 1)
    marks_full = torch.stack([m[:, 0] for m in rec.marks], 1)
    out = dict(
        S=np.int64(S), bs=np.int64(bs),
        dt=dts.numpy().astype(np.float32),
        dw=dws.numpy().astype(np.float32),
        jump_times=rec.jump_times[:, :, 0].numpy().astype(np.float32),
        paths=paths.numpy().astype(np.float32),
        time=time_paths[:, :S + 1, 0].numpy().astype(np.float32),
        left=left_paths[:, :S + 1].numpy().astype(np.float32),
        jumps=jump_paths[:, :S + 1].numpy().astype(np.float32),
        payoffs=(payoff(paths[:, S]) * disc(solver.time_interval)).numpy().astype(np.float32),
    )
    if one_asset:
        k, y = decode_indep_mark(torch, marks_full)
        out['marks'] = y.numpy().astype(np.float32)
        out['asset'] = k.numpy().astype(np.int32)
    else:
        out['marks'] = marks_full.numpy().astype(np.float32)
    if full:
        # every column multilevel_solve returns: (bs, total_steps_coarse + 1, dim) each
        out['paths_fine'] = pf.numpy().astype(np.float32)
        out['paths_coarse'] = pc.numpy().astype(np.float32)
    return out


def mlmc_replay_case(sde_mc, torch, solver, bs, levels, seed, one_asset=False, full=False):
    fine, coarse = levels
    factor = fine // coarse
    torch.manual_seed(seed)
    rec = Recorder(solver)
    (pf, pc), _ = solver.multilevel_solve(bs, levels)
    rec.restore()
    # scheme calls come as `factor` fine steps then one coarse step
    fine_calls = [c for i, c in enumerate(rec.steps) if i % (factor + 1) != factor]
    coarse_calls = [c for i, c in enumerate(rec.steps) if i % (factor + 1) == factor]
    marks_full = torch.stack([m[:, 0] for m in rec.marks], 1)
    out = dict(
        bs=np.int64(bs), fine=np.int64(fine), coarse=np.int64(coarse),
        dw=torch.stack([cn for _, cn in fine_calls], 1).numpy().astype(np.float32),
        dt_fine=torch.stack([h.reshape(bs) for h, _ in fine_calls], 1).numpy().astype(np.float32),
        dt_coarse=torch.stack([h.reshape(bs) for h, _ in coarse_calls], 1).numpy().astype(np.float32),
        jump_times=rec.jump_times[:, :, 0].numpy().astype(np.float32),
        xf=pf[:, -1].numpy().astype(np.float32), xc=pc[:, -1].numpy().astype(np.float32),
        h_fine=np.float32(torch.tensor(solver.time_interval / fine).item()),
        h_coarse=np.float32((factor * torch.tensor(solver.time_interval / fine)).item()),
    )
    if one_asset:
        k, y = decode_indep_mark(torch, marks_full)
        out['marks'] = y.numpy().astype(np.float32)
        out['asset'] = k.numpy().astype(np.int32)
    else:
        out['marks'] = marks_full.numpy().astype(np.float32)
    if full:
        # every column multilevel_solve returns: (bs, total_steps_coarse + 1, dim) each
        out['paths_fine'] = pf.numpy().astype(np.float32)
        out['paths_coarse'] = pc.numpy().astype(np.float32)
    return out


def f32(v):
    return float(np.float32(v))


def cv_jump_fixture(sm, torch):
    """The adapted control variate with both integrands (f on the Brownian
    increments, g on the compensated jumps) through the reference's own
    apply_adapted_control_variates and train_adapted_control_variates on one
    64-path batch: the sums of Gamma, the first epoch's loss, the gradients
    left on the parameters and the parameters after one Adam step."""
    from torch.utils.data import DataLoader
    torch.manual_seed(23)
    corr = sm.get_corr_matrix([0.5])
    m = sm.Merton(0.02, torch.tensor([0.2, 0.3]), 1.5, -0.05, 0.15, torch.tensor([1., 1.]), dim=2, corr_matrix=corr)
    sol = sm.JumpEulerSolver(m, 1.0, 16)
    csr = sm.ConstantShortRate(0.02)
    ds = sm.simulate_adapted_data(64, sol, sm.Rainbow(1.0), csr, bs=64).dataset
    dl = DataLoader(ds, batch_size=64, shuffle=False)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    g = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    nets = {'f': f, 'g': g}
    p0 = {k: [p.detach().clone() for p in v.parameters()] for k, v in nets.items()}
    s1, s2 = sm.apply_adapted_control_variates([f, g], dl, sol, csr)
    opt = torch.optim.Adam(list(f.parameters()) + list(g.parameters()), lr=1e-3)
    losses = sm.train_adapted_control_variates([f, g], opt, dl, sol, csr, epochs=1, print_losses=False)
    out = dict(time=ds.time_paths.numpy(), paths=ds.paths.numpy(), left=ds.left_paths.numpy(),
               jumps=ds.jump_paths.numpy(), normals=ds.normals.numpy(), payoffs=ds.payoffs.numpy(),
               sum=np.float64(float(s1)), sum_sq=np.float64(float(s2)), loss=np.float64(losses[0]),
               lam_kappa=np.asarray(float(sol.sde.jump_rate() * sol.sde.jump_mean()), np.float32),
               r=np.float32(0.02))
    for k, v in nets.items():
        for i, (a, p) in enumerate(zip(p0[k], v.parameters())):
            out['p0%s_%d' % (k, i)] = a.numpy()
            out['grad%s_%d' % (k, i)] = p.grad.detach().numpy()
            out['p1%s_%d' % (k, i)] = p.detach().numpy()
    np.savez_compressed(os.path.join(HERE, 'cv_mlp_jumps.npz'), **out)


def uniform_replay(sm, torch, sol, bs, seed, payoff, csr):
    """DiffusionSolver.solve (sde_mc/solvers.py:68-88) with every scheme call's
    increments recorded."""
    torch.manual_seed(seed)
    rec = Recorder(sol)
    paths, _ = sol.solve(bs=bs)
    rec.restore()
    return dict(bs=np.int64(bs), S=np.int64(sol.num_steps),
                dw=torch.stack([cn for _, cn in rec.steps], 1).numpy().astype(np.float32),
                paths=paths.numpy().astype(np.float32), chol=sol.lower_cholesky.numpy().astype(np.float32),
                payoffs=(payoff(paths[:, -1]) * csr(sol.time_interval)).numpy().astype(np.float32))


def diffusion_fixtures(sm, torch):
    """Replay cases for the log-price GBM (sde_mc/sde.py:210-219, constant
    coefficients, payoff through Option.log) and the two-Brownian 'indep'
    GBM (sde.py:222-255, EulerScheme's summed diffusion, schemes.py:9-10)."""
    csr = sm.ConstantShortRate(0.02)
    cases = {}
    lg = sm.LogGbm(0.02, 0.25, torch.tensor([0.0]))
    cases['replay_loggbm_uniform'] = uniform_replay(sm, torch, sm.EulerSolver(lg, 1.0, 16), 24, 41,
                                                    sm.EuroCall(1.0, log=True), csr)
    dg = sm.DoubleGbm(0.03, torch.tensor([0.15, 0.2]), torch.tensor([0.1, 0.05]), torch.tensor([1.0, 1.2]), 2)
    cases['replay_doublegbm_uniform'] = uniform_replay(sm, torch, sm.EulerSolver(dg, 1.0, 12), 24, 42,
                                                       sm.Basket(1.0), csr)
    for name, arrs in cases.items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **{k: np.asarray(v) for k, v in arrs.items()})


def levy_mlmc_fixture(sm, torch):
    """MLMC couplings beyond Merton, through JumpDiffusionSolver.multilevel_solve
    (sde_mc/solvers.py:228-307) with factor 2: the Levy rainbow preset's
    (LevyRainbowMLMC, sde_mc/problem.py:93-106; the 2-D ExpExampleLevy 'indep'
    model with exact_jumps=True, the jump reading the post-diffusion state)
    and the Asian wrapper's around a 1-D Merton."""
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    lsde = sm.LevySde(lev, torch.ones(2))
    sol = sm.JumpEulerSolver(lsde, 1.0, 4, exact_jumps=True)
    c = mlmc_replay_case(sm, torch, sol, 32, (8, 4), seed=19)
    c.update(max_jumps=np.int64(sol.max_jumps), exact_jumps=np.int64(1))
    np.savez_compressed(os.path.join(HERE, 'mlmc_levy2d_exact.npz'), **{k: np.asarray(v) for k, v in c.items()})
    # AsianWrapper (sde_mc/sde.py:378-406) around a 1-D Merton, same coupling
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    sol = sm.JumpEulerSolver(sm.AsianWrapper(m), 1.0, 4)
    c = mlmc_replay_case(sm, torch, sol, 32, (8, 4), seed=20)
    c.update(max_jumps=np.int64(sol.max_jumps), exact_jumps=np.int64(0))
    np.savez_compressed(os.path.join(HERE, 'mlmc_asian_merton.npz'), **{k: np.asarray(v) for k, v in c.items()})


def model_stats(sm, torch):
    """The reference's own plain estimates (mc_simple, sde_mc/mc.py:53-123)
    for the model kinds beyond Merton: Heston (HestonSolver), the Asian
    wrapper around a 1-D Merton, the 2-D Levy rainbow and the log-price GBM
    with its payoff through Option.log.  Added to stats.json."""
    path = os.path.join(HERE, 'stats.json')
    with open(path) as fh:
        stats = json.load(fh)
    csr = sm.ConstantShortRate(0.02)
    runs = {}
    h = sm.Heston(0.02, 2.0, 0.04, 0.3, -0.7, torch.tensor([1., 0.04]))
    runs['heston_64_2p16'] = (sm.HestonSolver(h, 1.0, 64, seed=41), sm.EuroCall(1.0), 'terminal')
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    runs['asian_merton_20_2p16'] = (sm.JumpEulerSolver(sm.AsianWrapper(m), 1.0, 20, seed=42), sm.AsianCall(1.0, 1.0),
                                    'adapted')
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    runs['levy2d_16_2p16'] = (sm.JumpEulerSolver(sm.LevySde(lev, torch.ones(2)), 1.0, 16, seed=43), sm.Rainbow(1.0),
                              'adapted')
    lg = sm.LogGbm(0.02, 0.25, torch.tensor([0.0]))
    runs['loggbm_16_2p16'] = (sm.EulerSolver(lg, 1.0, 16, seed=44), sm.EuroCall(1.0, log=True), 'terminal')
    for name, (sol, pay, pt) in runs.items():
        ts = time.time()
        st = sm.mc_simple(2 ** 16, sol, pay, csr, bs=2 ** 14, payoff_time=pt)
        stats[name] = dict(mean=float(st.sample_mean), se=float(st.sample_std), n=2 ** 16, seconds=time.time() - ts)
    with open(path, 'w') as fh:
        json.dump(stats, fh, indent=1, sort_keys=True)


def heston_asian_fixtures(sm, torch):
    """Replay cases for the two non-affine models: Heston with its implicit
    variance step (sde_mc/schemes.py:16-22, sde.py:258-279) on the uniform
    grid, and AsianWrapper (sde.py:378-406) around a 1-D Merton on the
    jump-adapted grid."""
    cases = {}
    csr = sm.ConstantShortRate(0.02)
    h = sm.Heston(0.02, 2.0, 0.04, 0.3, -0.7, torch.tensor([1., 0.04]))
    sol = sm.HestonSolver(h, 1.0, 24)
    torch.manual_seed(31)
    rec = Recorder(sol)
    hp, _ = sol.solve(bs=16)
    rec.restore()
    cases['replay_heston'] = dict(
        bs=np.int64(16), S=np.int64(24), dw=torch.stack([cn for _, cn in rec.steps], 1).numpy().astype(np.float32),
        paths=hp.numpy().astype(np.float32), chol=sol.lower_cholesky.numpy().astype(np.float32),
        payoffs=(sm.EuroCall(1.0)(hp[:, -1]) * csr(1.0)).numpy().astype(np.float32))
    # DiffusionSolver.multilevel_solve (sde_mc/solvers.py:90-119) through
    # the Heston scheme: `factor` fine steps, then one coarse step on the
    # summed increments
    for name, levels, seed in (('mlmc_heston', (8, 4), 33), ('mlmc_heston_f4', (16, 4), 34)):
        fine, coarse = levels
        factor = fine // coarse
        sol = sm.HestonSolver(h, 1.0, coarse)
        torch.manual_seed(seed)
        rec = Recorder(sol)
        (pf, pc), _ = sol.multilevel_solve(32, levels)
        rec.restore()
        fine_calls = [c for i, c in enumerate(rec.steps) if i % (factor + 1) != factor]
        h_fine = torch.tensor(1.0 / fine)
        cases[name] = dict(
            bs=np.int64(32), fine=np.int64(fine), coarse=np.int64(coarse),
            dw=torch.stack([cn for _, cn in fine_calls], 1).numpy().astype(np.float32),
            xf=pf[:, -1].numpy().astype(np.float32), xc=pc[:, -1].numpy().astype(np.float32),
            h_fine=np.float32(h_fine.item()), h_coarse=np.float32((factor * h_fine).item()))
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    aw = sm.AsianWrapper(m)
    sol2 = sm.JumpEulerSolver(aw, 1.0, 20)
    cases['replay_asian_merton'] = jump_replay_case(sm, torch, sol2, 32, sm.AsianCall(1.0, 1.0), csr, seed=32)
    cases['replay_asian_merton']['chol'] = sol2.lower_cholesky.numpy().astype(np.float32)
    for name, arrs in cases.items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **{k: np.asarray(v) for k, v in arrs.items()})


def mlmc_columns_fixture(sm, torch):
    """Every column of the coupled paths multilevel_solve returns, with the
    draws it used: JumpDiffusionSolver.multilevel_solve (sde_mc/solvers.py:
    228-307; columns at each coarse step, to the batch's last) for a 1-D
    Merton (common jumps) and the 2-D per-asset-jump model, and
    DiffusionSolver.multilevel_solve (:90-119; every fine and every coarse
    step, the normals it returns) for a correlated 2-D GBM."""
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    sol = sm.JumpEulerSolver(m, 1.0, 4)
    c = mlmc_replay_case(sm, torch, sol, 32, (8, 4), seed=41, full=True)
    c.update(max_jumps=np.int64(sol.max_jumps), exact_jumps=np.int64(0))
    np.savez_compressed(os.path.join(HERE, 'mlmc_cols_merton1d.npz'), **{k: np.asarray(v) for k, v in c.items()})
    ind = make_indep_merton(sm, torch, 0.02, [0.2, 0.3], [1.0, 1.0], -0.05, 0.15, 0.5)
    sol = sm.JumpEulerSolver(ind, 1.0, 8)
    c = mlmc_replay_case(sm, torch, sol, 32, (16, 8), seed=42, one_asset=True, full=True)
    c.update(max_jumps=np.int64(sol.max_jumps), exact_jumps=np.int64(0))
    np.savez_compressed(os.path.join(HERE, 'mlmc_cols_indep2d.npz'), **{k: np.asarray(v) for k, v in c.items()})
    g = sm.Gbm(0.02, torch.tensor([0.2, 0.25]), torch.tensor([1., 1.5]), 2, corr_matrix=sm.get_corr_matrix([-0.3]))
    sol = sm.EulerSolver(g, 1.0, 4)
    torch.manual_seed(43)
    (pf, pc), normals = sol.multilevel_solve(32, (8, 4))
    np.savez_compressed(os.path.join(HERE, 'mlmc_cols_gbm_uniform.npz'), bs=np.int64(32), fine=np.int64(8),
                        coarse=np.int64(4), normals=normals.numpy().astype(np.float32),
                        paths_fine=pf.numpy().astype(np.float32), paths_coarse=pc.numpy().astype(np.float32),
                        h_fine=np.float32(torch.tensor(1.0 / 8).item()),
                        h_coarse=np.float32((2 * torch.tensor(1.0 / 8)).item()))


def optimal_trials_fixture(sm, torch):
    """get_optimal_trials (sde_mc/mlmc.py:77-97) on prescribed level samples.
    A stand-in solver returns paths whose terminal values are the samples
    (the coarse paths are zero), the payoff is EuroCall(0) (the identity on
    positive values) and the discounter is 1, so the reference's own float32
    variance and allocation arithmetic runs on known inputs.  Also records
    that the call leaves solver.num_steps at levels[0]."""
    rng = np.random.default_rng(21)
    cases = []
    for levels, eps, nsamp, scale in [([4, 8, 16, 32, 64, 128, 256], 1e-3 * 0.2, 256, 0.3),
                                      ([2, 4, 8], 5e-3, 100, 1.0), ([16, 64, 256], 2e-4, 64, 0.05)]:
        samples = []
        for lvl in range(len(levels)):
            # level variances falling with the step size, as for a convergent scheme
            v = np.abs(rng.standard_normal(nsamp)) * scale * (0.5 ** lvl) + 1e-3
            samples.append(v.astype(np.float32))

        class FixedSolver:
            time_interval = 1.0
            num_steps = 999

            def solve(self, bs, low_storage=False):
                return torch.from_numpy(samples[0]).reshape(-1, 1, 1), None

            def multilevel_solve(self, bs, pair):
                i = levels.index(pair[0])
                fine = torch.from_numpy(samples[i]).reshape(-1, 1, 1)
                return (fine, torch.zeros_like(fine)), None

        solver = FixedSolver()
        trials = sm.get_optimal_trials(nsamp, levels, eps, solver, sm.EuroCall(0.0), lambda t: 1.0)
        cases.append(dict(levels=levels, eps=eps, T=1.0, samples=[a.tolist() for a in samples],
                          trials=[int(t) for t in trials], num_steps_after=int(solver.num_steps)))
    with open(os.path.join(HERE, 'optimal_trials.json'), 'w') as fh:
        json.dump(cases, fh)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True, help='checkout of the sde_mc reference to import')
    ap.add_argument('--skip-stats', action='store_true')
    ap.add_argument('--only', choices=['cv_jumps', 'heston_asian', 'diffusions', 'levy_mlmc', 'model_stats',
                                       'optimal_trials', 'mlmc_columns'],
                    default=None,
                    help='write only these fixtures')
    args = ap.parse_args()
    sm = load_reference(args.ref)
    import torch
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    t0 = time.time()
    if args.only == 'cv_jumps':
        cv_jump_fixture(sm, torch)
        return
    if args.only == 'heston_asian':
        heston_asian_fixtures(sm, torch)
        return
    if args.only == 'diffusions':
        diffusion_fixtures(sm, torch)
        return
    if args.only == 'levy_mlmc':
        levy_mlmc_fixture(sm, torch)
        return
    if args.only == 'model_stats':
        model_stats(sm, torch)
        return
    if args.only == 'optimal_trials':
        optimal_trials_fixture(sm, torch)
        return
    if args.only == 'mlmc_columns':
        mlmc_columns_fixture(sm, torch)
        return
    cv_jump_fixture(sm, torch)
    heston_asian_fixtures(sm, torch)
    diffusion_fixtures(sm, torch)
    levy_mlmc_fixture(sm, torch)
    optimal_trials_fixture(sm, torch)
    mlmc_columns_fixture(sm, torch)

    # ------------------------------------------------------------ KATs ----
    kat = {}
    kat['bs_binary_aon'] = [[1, 1, 3, 0.02, 0.2], float(sm.bs_binary_aon(1, 1, 3, 0.02, 0.2))]
    kat['bs_call'] = [[1, 1, 3, 0.02, 0.2], float(sm.bs_call(1, 1, 3, 0.02, 0.2))]
    kat['merton_call'] = [[[1, 1, 3, 0.02, 0.3, -0.05, 0.3, 2], float(sm.merton_call(1, 1, 3, 0.02, 0.3, -0.05, 0.3, 2))],
                          [[1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0], float(sm.merton_call(1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0))],
                          [[1.0, 0.9, 0.5, 0.03, 0.25, -0.05, 0.15, 1.0], float(sm.merton_call(1.0, 0.9, 0.5, 0.03, 0.25, -0.05, 0.15, 1.0))]]
    kat['bs_digital_call'] = [[1, 1.1, 2, 0.02, 0.3], float(sm.bs_digital_call(1, 1.1, 2, 0.02, 0.3))]
    kat['bs_asian_call'] = [[1, 1, 1, 0.02, 0.2], float(sm.bs_asian_call(1, 1, 1, 0.02, 0.2))]
    t1 = torch.tensor([[1.], [3.], [0.5], [0.]])
    t2 = torch.tensor([[1., 2.], [0., 0.5], [1.2, 0.9]])
    t4 = torch.tensor([[1., 2., 0.5, 1.5], [0.3, 0.5, 0.8, 0.9], [1.2, 0.9, 1.1, 1.0]])
    pay = {}
    for name, opt, x in [
        ('EuroCall', sm.EuroCall(1), t1), ('EuroPut', sm.EuroPut(1), t1), ('BinaryAoN', sm.BinaryAoN(1), t1),
        ('Digital', sm.Digital(1.), t1), ('Basket', sm.Basket(1), t2), ('BasketGeo', sm.Basket(0.8, 'geometric'), t2 + 0.1),
        ('Rainbow', sm.Rainbow(1), t2), ('BestOf', sm.BestOf(1), t2), ('HestonRainbow', sm.HestonRainbow(1.0), t4),
        ('AsianCall', sm.AsianCall(2.0, 0.5), t2), ('EuroCallLog', sm.EuroCall(1.0, log=True, discount=0.9), t1 - 0.5),
        ('RainbowLog', sm.Rainbow(1.0, log=True, discount=1.05), t2 - 0.3), ('Basket4', sm.Basket(1.0), t4)]:
        pay[name] = dict(x=x.tolist(), out=opt(x).tolist())
    kat['payoffs'] = pay
    kat['constant_short_rate'] = dict(t=[0., 1., 2.], r=0.02, out=sm.ConstantShortRate(0.02)(torch.tensor([0., 1., 2.])).tolist(),
                                      scalar=float(sm.ConstantShortRate(0.02)(1.0)))
    s = torch.tensor([1, 2, 3, 4, 5, 20, 100.])
    mn, var = sm.mc_estimates(s.sum(), (s * s).sum(), len(s))
    kat['mc_estimates'] = dict(sample=s.tolist(), mean=float(mn), var=float(var))
    kat['get_corr_matrix'] = dict(rhos=[0.7, 0.2, -0.3], out=sm.get_corr_matrix([0.7, 0.2, -0.3]).tolist())
    kat['partition'] = {e: sm.partition(3, 3, e).tolist() for e in ['both', 'left', 'right', 'none']}
    kat['solve_quadratic'] = dict(a=[1., 1., 1., 2.], b=[0., -2., -13., 32.], c=[-1., -15., 42., -5.],
                                  out=sm.solve_quadratic((torch.tensor([1., 1., 1., 2.]), torch.tensor([0., -2., -13., 32.]),
                                                          torch.tensor([-1., -15., 42., -5.]))).tolist())
    kat['remove_steps'] = [[0.1, 1000, 3], sm.remove_steps(0.1, 1000, 3)]
    kat['ceil_mult'] = [[1001, 100], sm.ceil_mult(1001, 100)]
    mj = {}
    for lam, T in [(2.0, 1.0), (1.0, 3.0), (0.5, 1.0), (3.0, 2.0), (8.0, 1.0)]:
        m = sm.Merton(0.02, 0.2, lam, -0.1, 0.2, torch.tensor([1.]), dim=1)
        mj['%g_%g' % (lam, T)] = int(sm.JumpEulerSolver(m, T, 10).max_jumps)
    kat['max_jumps'] = mj
    m1 = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    kat['merton_c1_drift_coef'] = float((m1.mu - m1.rate * m1.jump_mean()))
    kat['merton_c1_jump_mean'] = float(m1.jump_mean())
    icdf = sm.InverseCdf(1, 1, 2, 0.5, 0.01)
    ys = torch.tensor([1e-4, 0.003, 0.01, 0.2, 0.45, 0.5, 0.55, 0.8, 0.99, 0.9999])
    kat['inverse_cdf'] = dict(params=[1, 1, 2, 0.5, 0.01], y=ys.tolist(), out=icdf(ys).tolist(),
                              lda=float(icdf.lda), y1=float(icdf.y1), y2=float(icdf.y2), y3=float(icdf.y3))
    kat['get_jump_comp'] = [[1, 1, 0.5, 2, 0.2], float(sm.get_jump_comp(1, 1, 0.5, 2, 0.2))]
    ev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.1, 0.01)
    kat['exp_example_levy'] = dict(gamma=float(ev.gamma()), beta=float(ev.beta()))
    with open(os.path.join(HERE, 'kat.json'), 'w') as fh:
        json.dump(kat, fh, indent=1, sort_keys=True)

    # --------------------------------------------------------- replays ----
    csr = sm.ConstantShortRate(0.02)
    cases = {}
    # C1: Merton 1D European call, 100 jump-adapted steps
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
    sol = sm.JumpEulerSolver(m, 1.0, 100)
    c = jump_replay_case(sm, torch, sol, 64, sm.EuroCall(1.0), csr, seed=11)
    c.update(coef_b=np.array([float(m.mu - m.rate * m.jump_mean())], np.float32), sigma=np.array([0.2], np.float32),
             x0=np.array([1.], np.float32), T=np.float32(1.0), steps=np.int64(100), rate=np.float32(2.0),
             max_jumps=np.int64(sol.max_jumps), exact_jumps=np.int64(0), disc=np.float32(csr(1.0).item()),
             chol=np.array([[1.]], np.float32), strike=np.float32(1.0))
    cases['replay_merton1d'] = c
    # 2D correlated Merton (common jumps), tensor sigma, EuroCall on asset 0 and Rainbow payoffs
    corr = sm.get_corr_matrix([0.5])
    m2 = sm.Merton(0.02, torch.tensor([0.2, 0.3]), 1.5, -0.05, 0.15, torch.tensor([1., 1.]), dim=2, corr_matrix=corr)
    sol2 = sm.JumpEulerSolver(m2, 1.0, 50)
    c = jump_replay_case(sm, torch, sol2, 32, sm.Rainbow(1.0), csr, seed=12)
    c.update(coef_b=(m2.mu - m2.rate * m2.jump_mean()) * torch.ones(2), sigma=np.array([0.2, 0.3], np.float32),
             x0=np.array([1., 1.], np.float32), T=np.float32(1.0), steps=np.int64(50), rate=np.float32(1.5),
             max_jumps=np.int64(sol2.max_jumps), exact_jumps=np.int64(0), disc=np.float32(csr(1.0).item()),
             chol=sol2.lower_cholesky.numpy().astype(np.float32), strike=np.float32(1.0))
    c['coef_b'] = np.asarray(c['coef_b'], np.float32)
    cases['replay_merton2d_corr'] = c
    # exact_jumps=True variant
    sol3 = sm.JumpEulerSolver(m2, 1.0, 20, exact_jumps=True)
    c = jump_replay_case(sm, torch, sol3, 32, sm.Rainbow(1.0), csr, seed=13)
    c.update(coef_b=np.asarray((m2.mu - m2.rate * m2.jump_mean()) * torch.ones(2), np.float32),
             sigma=np.array([0.2, 0.3], np.float32), x0=np.array([1., 1.], np.float32), T=np.float32(1.0),
             steps=np.int64(20), rate=np.float32(1.5), max_jumps=np.int64(sol3.max_jumps), exact_jumps=np.int64(1),
             disc=np.float32(csr(1.0).item()), chol=sol3.lower_cholesky.numpy().astype(np.float32), strike=np.float32(1.0))
    cases['replay_merton2d_exact'] = c
    # C2 model: per-asset independent jumps through the superposition adapter
    ind = make_indep_merton(sm, torch, 0.02, [0.2, 0.3], [1.0, 1.0], -0.05, 0.15, 0.5)
    sol4 = sm.JumpEulerSolver(ind, 1.0, 64)
    c = jump_replay_case(sm, torch, sol4, 32, sm.Rainbow(1.0), csr, seed=14, one_asset=True)
    c.update(coef_b=np.asarray(ind.r - ind.lam * ind.kappa, np.float32), sigma=np.array([0.2, 0.3], np.float32),
             x0=np.array([1., 1.], np.float32), T=np.float32(1.0), steps=np.int64(64), rate=np.float32(2.0),
             max_jumps=np.int64(sol4.max_jumps), exact_jumps=np.int64(0), disc=np.float32(csr(1.0).item()),
             chol=sol4.lower_cholesky.numpy().astype(np.float32), strike=np.float32(1.0))
    cases['replay_indep2d'] = c
    # Levy 'indep' layout: ExpExampleLevy in 2D with a coarse truncation
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    lsde = sm.LevySde(lev, torch.ones(2))
    sol5 = sm.JumpEulerSolver(lsde, 1.0, 16)
    c = jump_replay_case(sm, torch, sol5, 16, sm.Rainbow(1.0), csr, seed=15)
    c.update(x0=np.array([1., 1.], np.float32), T=np.float32(1.0), steps=np.int64(16), rate=np.float32(lsde.jump_rate().item()),
             max_jumps=np.int64(sol5.max_jumps), exact_jumps=np.int64(0), disc=np.float32(csr(1.0).item()),
             chol=sol5.lower_cholesky.numpy().astype(np.float32), strike=np.float32(1.0),
             levy_r=np.float32(0.02), levy_sigma=np.float32(0.2), levy_f=np.float32(0.2),
             levy_gamma=np.float32(lev.gamma()), levy_beta=np.float32(lev.beta()))
    cases['replay_levy2d'] = c
    # Uniform grid (EulerSolver): correlated 2D Gbm
    g2 = sm.Gbm(0.02, torch.tensor([0.2, 0.25]), torch.tensor([1., 1.5]), 2, corr_matrix=sm.get_corr_matrix([-0.3]))
    sol6 = sm.EulerSolver(g2, 1.0, 12)
    torch.manual_seed(16)
    rec = Recorder(sol6)
    gp, _ = sol6.solve(bs=16)
    rec.restore()
    cases['replay_gbm_uniform'] = dict(
        bs=np.int64(16), S=np.int64(12), dw=torch.stack([cn for _, cn in rec.steps], 1).numpy().astype(np.float32),
        paths=gp.numpy().astype(np.float32), x0=np.array([1., 1.5], np.float32), mu=np.float32(0.02),
        sigma=np.array([0.2, 0.25], np.float32), T=np.float32(1.0), steps=np.int64(12),
        h=np.float32(torch.tensor(1.0 / 12).item()), chol=sol6.lower_cholesky.numpy().astype(np.float32))
    # MLMC couplings
    sol7 = sm.JumpEulerSolver(m, 1.0, 4)
    c = mlmc_replay_case(sm, torch, sol7, 32, (8, 4), seed=17)
    c.update(coef_b=np.array([float(m.mu - m.rate * m.jump_mean())], np.float32), sigma=np.array([0.2], np.float32),
             x0=np.array([1.], np.float32), T=np.float32(1.0), rate=np.float32(2.0), max_jumps=np.int64(sol7.max_jumps),
             exact_jumps=np.int64(0), chol=np.array([[1.]], np.float32))
    cases['mlmc_merton1d'] = c
    sol8 = sm.JumpEulerSolver(ind, 1.0, 8)
    c = mlmc_replay_case(sm, torch, sol8, 32, (16, 8), seed=18, one_asset=True)
    c.update(coef_b=np.asarray(ind.r - ind.lam * ind.kappa, np.float32), sigma=np.array([0.2, 0.3], np.float32),
             x0=np.array([1., 1.], np.float32), T=np.float32(1.0), rate=np.float32(2.0), max_jumps=np.int64(sol8.max_jumps),
             exact_jumps=np.int64(0), chol=sol8.lower_cholesky.numpy().astype(np.float32))
    cases['mlmc_indep2d'] = c
    for name, arrs in cases.items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **{k: np.asarray(v) for k, v in arrs.items()})

    # ------------------------------------------------------ MLP / CV ------
    torch.manual_seed(21)
    sol9 = sm.JumpEulerSolver(ind, 1.0, 16)
    dl = sm.simulate_adapted_data(64, sol9, sm.Rainbow(1.0), csr, bs=64, inference=True)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    g = sm.ZeroFunction(2)
    opt = torch.optim.Adam(f.parameters(), lr=1e-3)
    (paths, normals, left_paths, time_paths, jump_paths), payoffs = next(iter(dl))
    n, steps, dim = paths.shape
    params0 = [p.detach().clone() for p in f.parameters()]
    discounts = csr(time_paths)
    f_in = torch.cat([time_paths.reshape(n * steps, 1), paths.reshape(n * steps, dim)], -1)
    f_out = f(f_in).view(normals.shape)
    bcv = sm.integrate_cv(normals, f_out, discounts, 'diag')
    gam = payoffs + bcv
    loss = gam.var()
    opt.zero_grad()
    loss.backward()
    grads = [p.grad.detach().clone() for p in f.parameters()]
    opt.step()
    params1 = [p.detach().clone() for p in f.parameters()]
    cv = dict(f_in=f_in.detach().numpy(), f_out=f_out.detach().numpy().reshape(n * steps, 2), normals=normals.numpy(),
              time=time_paths.numpy(), paths=paths.numpy(), payoffs=payoffs.numpy(), gamma=gam.detach().numpy(),
              loss=np.float32(loss.item()), r=np.float32(0.02))
    for i, (p0, gr, p1) in enumerate(zip(params0, grads, params1)):
        cv['p0_%d' % i] = p0.numpy()
        cv['grad_%d' % i] = gr.numpy()
        cv['p1_%d' % i] = p1.numpy()
    np.savez_compressed(os.path.join(HERE, 'cv_mlp.npz'), **cv)

    # ------------------------------------------------------- stats --------
    if not args.skip_stats:
        stats = {}
        oracle_c1 = float(sm.merton_call(1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0))
        m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
        sol = sm.JumpEulerSolver(m, 1.0, 100, seed=1)
        ts = time.time()
        st = sm.mc_simple(2 ** 16, sol, sm.EuroCall(1.0), csr, payoff_time='adapted')
        stats['c1_fp32_2p16'] = dict(mean=st.sample_mean, se=st.sample_std, n=2 ** 16, seconds=time.time() - ts,
                                     oracle=oracle_c1)
        sol = sm.JumpEulerSolver(m, 1.0, 100, seed=2)
        st = sm.mc_simple(2 ** 18, sol, sm.EuroCall(1.0), csr, bs=2 ** 16, payoff_time='adapted')
        stats['c1_fp32_2p18'] = dict(mean=st.sample_mean, se=st.sample_std, n=2 ** 18)
        sol4 = sm.JumpEulerSolver(ind, 1.0, 256, seed=3)
        ts = time.time()
        st = sm.mc_simple(2 ** 16, sol4, sm.Rainbow(1.0), csr, bs=2 ** 15, payoff_time='adapted')
        stats['c2_plain_2p16'] = dict(mean=st.sample_mean, se=st.sample_std, n=2 ** 16, seconds=time.time() - ts)
        sol4 = sm.JumpEulerSolver(ind, 1.0, 256, seed=4)
        levels = [2 ** (l + 2) for l in range(5)]
        ts = time.time()
        ml = sm.mc_multilevel([2 ** 14] * 5, levels, sol4, sm.Rainbow(1.0), csr)
        stats['c2_mlmc_l0_4'] = dict(mean=ml.sample_mean, se=ml.sample_std, levels=levels, trials=[2 ** 14] * 5,
                                     seconds=time.time() - ts)
        # per-level means/variances of the coupled differences
        lvl = []
        torch.manual_seed(5)
        for fi, co in zip(levels[1:], levels[:-1]):
            (pf, pc), _ = sol4.multilevel_solve(2 ** 14, (fi, co))
            y = csr(1.0) * (sm.Rainbow(1.0)(pf[:, -1]) - sm.Rainbow(1.0)(pc[:, -1]))
            lvl.append(dict(levels=[fi, co], mean=float(y.mean()), var=float(y.var()), n=2 ** 14))
        stats['c2_mlmc_level_stats'] = lvl
        g2 = sm.Gbm(0.02, 0.2, torch.tensor([1.]), 1)
        sol6 = sm.EulerSolver(g2, 1.0, 50, seed=6)
        st = sm.mc_simple(2 ** 16, sol6, sm.EuroCall(1.0), csr)
        stats['gbm1d_uniform_2p16'] = dict(mean=st.sample_mean, se=st.sample_std, n=2 ** 16,
                                           oracle=float(sm.bs_call(1, 1, 1, 0.02, 0.2)))
        with open(os.path.join(HERE, 'stats.json'), 'w') as fh:
            json.dump(stats, fh, indent=1, sort_keys=True)
        model_stats(sm, torch)
    print('golden fixtures written in %.1f s' % (time.time() - t0))


if __name__ == '__main__':
    main()
