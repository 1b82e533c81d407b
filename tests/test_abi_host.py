"""CPU-side checks: the C-ABI library loads and exports every declared symbol,
the ctypes descriptor matches the C layout, and the host-side API (lowering,
payoffs, helpers, closed forms) matches the reference's known answers."""
import math
import os
import re

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import _native as N
from sde_mc_gb300.lowering import lower, max_jumps_for
from tests.cases import FIXTURE_CASES, inst_for, indep2d, levy2d, merton1d
from tests.conftest import ROOT, load_npz


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sdemc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|size_t)\s+(sdemc_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = N.load()
    decl = declared_symbols()
    assert len(decl) >= 14
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) == set(N.EXPORTED)


def test_library_exports_nothing_undeclared():
    """The shared library's dynamic symbol table holds the header's entry
    points and no other public name (the CUDA runtime is linked statically
    and stays hidden)."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    N.load()
    out = subprocess.run([nm, "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True, check=True)
    names = {ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()}
    public = {n for n in names if not n.startswith("_")}
    assert public == set(declared_symbols()), sorted(public ^ set(declared_symbols()))


def test_adam_bias_corrections():
    """The host-side bias corrections that a graph of Adam steps reads from
    device memory: 1 - b1^t and sqrt(1 - b2^t) in float32; t < 1 refused."""
    import ctypes
    lib = N.load()
    buf = (ctypes.c_float * 2)()
    b1, b2 = float(np.float32(0.9)), float(np.float32(0.999))  # the float32 betas the call receives
    for t in (1, 7, 640):
        assert lib.sdemc_adam_bias(t, 0.9, 0.999, buf) == N.OK
        assert buf[0] == pytest.approx(1 - b1 ** t, rel=2e-6)
        assert buf[1] == pytest.approx(math.sqrt(1 - b2 ** t), rel=2e-5)
    assert lib.sdemc_adam_bias(0, 0.9, 0.999, buf) == N.EINVAL


def test_descriptor_layout_matches_header():
    lib = N.load()
    assert lib.sdemc_abi_version() == 1
    assert lib.sdemc_inst_size() == __import__("ctypes").sizeof(N.SdemcInst)
    assert N.abi_offsets() == N.ctypes_offsets()


def test_scratch_sizes():
    import ctypes
    inst = inst_for(merton1d(), num_paths=1000)
    lib = N.load()
    nch = (1000 + 31) // 32          # chunks of one warp round
    ngroups = (nch + 255) // 256     # first-level reduction groups
    assert lib.sdemc_price_scratch_bytes(ctypes.byref(inst)) == 256 + (nch + ngroups) * 3 * 8
    assert lib.sdemc_mlmc_scratch_bytes(ctypes.byref(inst)) == 256 + (nch + ngroups) * 5 * 8


def test_lowering_uses_reference_float32_coefficients(kat):
    inst = inst_for(merton1d(), num_paths=10)
    assert inst.drift_b[0] == np.float32(kat["merton_c1_drift_coef"])
    assert inst.diff_q[0] == np.float32(0.2)
    assert inst.h == np.float32(1.0 / 100)
    assert inst.rate == 2.0 and inst.mark == N.MARK_LOGNORMAL
    for name, factory in FIXTURE_CASES.items():
        fx = load_npz(name)
        ins = inst_for(factory(), num_paths=4)
        if "coef_b" in fx:
            np.testing.assert_array_equal(np.array(ins.drift_b[:ins.dim], np.float32), fx["coef_b"].reshape(-1))
        L = fx["chol"]
        packed = [L[i, j] for i in range(ins.dim) for j in range(i + 1)]
        np.testing.assert_array_equal(np.array(ins.chol[:len(packed)], np.float32), np.array(packed, np.float32))


def test_max_jumps_matches_reference(kat):
    for key, v in kat["max_jumps"].items():
        lam, T = map(float, key.split("_"))
        assert max_jumps_for(lam, T) == v
        m = sm.Merton(0.02, 0.2, lam, -0.1, 0.2, torch.tensor([1.]), dim=1)
        assert sm.JumpEulerSolver(m, T, 10).max_jumps == v


def test_payoffs_match_reference(kat):
    make = {"EuroCall": lambda: sm.EuroCall(1), "EuroPut": lambda: sm.EuroPut(1),
            "BinaryAoN": lambda: sm.BinaryAoN(1), "Digital": lambda: sm.Digital(1.), "Basket": lambda: sm.Basket(1),
            "BasketGeo": lambda: sm.Basket(0.8, 'geometric'), "Rainbow": lambda: sm.Rainbow(1),
            "BestOf": lambda: sm.BestOf(1), "HestonRainbow": lambda: sm.HestonRainbow(1.0),
            "AsianCall": lambda: sm.AsianCall(2.0, 0.5),
            "EuroCallLog": lambda: sm.EuroCall(1.0, log=True, discount=0.9),
            "RainbowLog": lambda: sm.Rainbow(1.0, log=True, discount=1.05), "Basket4": lambda: sm.Basket(1.0)}
    for name, case in kat["payoffs"].items():
        got = make[name]()(torch.tensor(case["x"]))
        np.testing.assert_allclose(got.numpy(), np.array(case["out"]), rtol=1e-6, atol=1e-7, err_msg=name)


def test_helpers_match_reference(kat):
    for e, v in kat["partition"].items():
        np.testing.assert_allclose(sm.partition(3, 3, e).numpy(), v)
    q = kat["solve_quadratic"]
    got = sm.solve_quadratic((torch.tensor(q["a"]), torch.tensor(q["b"]), torch.tensor(q["c"])))
    np.testing.assert_allclose(got.numpy(), q["out"], rtol=1e-6)
    s = torch.tensor(kat["mc_estimates"]["sample"])
    m, v = sm.mc_estimates(s.sum(), (s * s).sum(), len(s))
    assert float(m) == pytest.approx(kat["mc_estimates"]["mean"], rel=1e-6)
    assert float(v) == pytest.approx(kat["mc_estimates"]["var"], rel=1e-6)
    np.testing.assert_allclose(sm.get_corr_matrix(kat["get_corr_matrix"]["rhos"]).numpy(),
                               kat["get_corr_matrix"]["out"], rtol=1e-6)
    args, v = kat["remove_steps"]
    assert sm.remove_steps(*args) == v
    args, v = kat["ceil_mult"]
    assert sm.ceil_mult(*args) == v
    with pytest.raises(AssertionError):
        sm.get_corr_matrix([0.1, 0.2])
    with pytest.raises(RuntimeError):
        sm.get_corr_matrix([0.99, 0.99, -0.99])


def test_closed_forms_match_reference(kat):
    for args, v in kat["merton_call"]:
        assert sm.merton_call(*args) == pytest.approx(v, rel=1e-12)
    assert sm.bs_call(*kat["bs_call"][0]) == pytest.approx(kat["bs_call"][1], rel=1e-12)
    assert sm.bs_binary_aon(*kat["bs_binary_aon"][0]) == pytest.approx(kat["bs_binary_aon"][1], rel=1e-9)
    assert sm.bs_digital_call(*kat["bs_digital_call"][0]) == pytest.approx(kat["bs_digital_call"][1], rel=1e-10)
    assert sm.bs_asian_call(*kat["bs_asian_call"][0]) == pytest.approx(kat["bs_asian_call"][1], rel=1e-12)
    c = kat["constant_short_rate"]
    np.testing.assert_allclose(sm.ConstantShortRate(c["r"])(torch.tensor(c["t"])).numpy(), c["out"])
    assert float(sm.ConstantShortRate(c["r"])(1.0)) == pytest.approx(c["scalar"])


def test_levy_objects_match_reference(kat):
    ic = kat["inverse_cdf"]
    icdf = sm.InverseCdf(*ic["params"][:2], ic["params"][2], ic["params"][3], ic["params"][4])
    assert icdf.lda == pytest.approx(ic["lda"]) and icdf.y2 == pytest.approx(ic["y2"])
    np.testing.assert_allclose(icdf(torch.tensor(ic["y"])).numpy(), ic["out"], rtol=1e-5, atol=1e-6)
    assert sm.get_jump_comp(*kat["get_jump_comp"][0]) == pytest.approx(kat["get_jump_comp"][1], rel=1e-9)
    ev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.1, 0.01)
    assert ev.gamma() == pytest.approx(kat["exp_example_levy"]["gamma"])
    assert ev.beta() == pytest.approx(kat["exp_example_levy"]["beta"])


def test_sde_interfaces():
    g = sm.Gbm(0.02, 0.2, torch.tensor([1., 2.]), dim=2)
    assert g.diffusion_struct == 'diag' and g.brown_dim == 2 and g.jump_rate() == 0
    x0 = g.init_value
    assert torch.allclose(g.drift(0, x0), 0.02 * x0)
    m = sm.Merton(0.02, 0.3, 2, -0.05, 0.3, torch.tensor([1., 1.]), dim=2)
    assert torch.allclose(m.drift(0, x0), (0.02 - m.jump_mean() * 2) * x0)
    assert m.sample_jumps((3, 4, 2), 'cpu').shape == (3, 4, 2)
    h = sm.Heston(0.02, 0.5, 0.1, 0.15, -0.5, torch.tensor([1., 2.]))
    assert torch.allclose(h.corr_matrix, torch.tensor([[1, -0.5], [-0.5, 1]]))
    ind = indep2d()[0].sde
    assert torch.allclose(ind.jump_rate(), torch.tensor([1., 1.]))
    assert ind.sample_jumps((5, 1), 'cpu').shape == (5, 2)


def test_unknown_model_is_not_lowered():
    class Custom(sm.DiffusionSde):
        def drift(self, t, x):
            return x * x

        def diffusion(self, t, x):
            return x

    s = sm.EulerSolver(Custom(torch.ones(1), 1, 1, 'diag'), 1.0, 10)
    with pytest.raises(NotImplementedError):
        lower(s, sm.EuroCall(1.0), None, num_paths=10)
    with pytest.raises(NotImplementedError):
        lower(sm.JumpEulerSolver(sm.Gbm(0.1, 0.2, torch.ones(9), 9), 1.0, 10), sm.Basket(1.0), None, 10)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback():
    solver, payoff, disc = merton1d()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sm.mc_simple(1000, solver, payoff, disc, bs=1000)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        solver.solve(8)
    from sde_mc_gb300 import serve
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        serve.Server()


def test_server_struct_layouts_match_header():
    """The ctypes mirrors of the server's request/result structs have the C
    sizes, and an invalid server configuration is refused before any device
    work (no GPU needed)."""
    import ctypes
    from sde_mc_gb300 import serve
    assert serve.struct_sizes() == (ctypes.sizeof(serve.ServerCfg), ctypes.sizeof(serve.Request),
                                    ctypes.sizeof(serve.Result), ctypes.sizeof(serve.ServerStats))
    assert serve.Request.inst.offset == 0 and ctypes.sizeof(serve.Request) == ctypes.sizeof(N.SdemcInst) + 32
    lib = N.load()
    h = ctypes.c_void_p()
    bad = serve.ServerCfg(device=0, max_slots=0, mem_budget=1 << 30)
    assert lib.sdemc_server_create(ctypes.byref(bad), ctypes.byref(h)) == N.EINVAL
    assert h.value is None
    bad = serve.ServerCfg(device=0, max_slots=4, mem_budget=1 << 30, block_threads=48)
    assert lib.sdemc_server_create(ctypes.byref(bad), ctypes.byref(h)) == N.EINVAL


def test_batch_plan_groups_and_orders():
    """The host planner (no GPU needed): classes of equal (dim, noise, mode),
    contiguous chunk runs, descending cost inside a class, a permutation back
    to the caller's order, chunk/group prefix sums."""
    import ctypes
    from sde_mc_gb300 import batch as B
    from sde_mc_gb300 import workloads
    mix = workloads.basket_mix(64, device="cpu")
    insts = B.lower_mix(mix)
    n = len(insts)
    lib = N.load()
    nbytes = lib.sdemc_batch_plan_bytes(n)
    buf = ctypes.create_string_buffer(nbytes)
    arr = (N.SdemcInst * n)(*insts)
    assert lib.sdemc_batch_plan(ctypes.cast(arr, ctypes.c_void_p), n, buf, nbytes) == 0
    base = ctypes.addressof(buf)
    H = B.BatchHeader.from_address(base)
    assert H.n_inst == n
    classes = (B.BatchClass * H.n_class).from_address(base + H.off_classes)
    order = list((ctypes.c_int32 * n).from_address(base + H.off_order))
    cp = list((ctypes.c_int64 * (n + 1)).from_address(base + H.off_chunk_prefix))
    gp = list((ctypes.c_int64 * (n + 1)).from_address(base + H.off_group_prefix))
    plan = (N.SdemcInst * n).from_address(base + H.off_insts)
    assert sorted(order) == list(range(n))
    keys = set()
    for c in classes:
        assert (c.dim, c.noise, c.mode) not in keys
        keys.add((c.dim, c.noise, c.mode))
        costs = [plan[j].num_steps + plan[j].rate for j in range(c.first, c.first + c.count)]
        assert costs == sorted(costs, reverse=True)
        assert all(plan[j].dim == c.dim for j in range(c.first, c.first + c.count))
        assert c.chunk_begin == cp[c.first] and c.chunk_end == cp[c.first + c.count]
    assert sum(c.count for c in classes) == n
    for j in range(n):
        assert plan[j].num_paths == insts[order[j]].num_paths
        assert cp[j + 1] - cp[j] == (insts[order[j]].num_paths + 31) // 32
        assert gp[j + 1] - gp[j] == max(1, (cp[j + 1] - cp[j] + 255) // 256)
    assert H.total_chunks == cp[n] and H.total_groups == gp[n]
    assert lib.sdemc_batch_plan(ctypes.cast(arr, ctypes.c_void_p), n, buf, nbytes - 1) == N.ENOMEM


def test_basket_mix_law():
    """The basket-mix instance law: ranges and the stated draw order."""
    from sde_mc_gb300 import workloads
    mix = workloads.basket_mix(512, device="cpu")
    dims = [m.dim for m in mix]
    steps = [m.solver.num_steps for m in mix]
    paths = [m.paths for m in mix]
    assert set(dims) == set(range(1, 9))
    assert 32 <= min(steps) and max(steps) <= 512
    assert 2 ** 12 <= min(paths) and max(paths) <= 2 ** 18
    assert all(0.8 <= m.payoff.strike <= 1.2 for m in mix)
    assert [m.stream_id for m in mix] == list(range(512))


def test_torch_ops_registered_with_schemas():
    """Every C-ABI compute entry point the estimators use is a torch op with a
    typed schema (registration needs no GPU)."""
    from sde_mc_gb300 import torch_ops
    for name in torch_ops.OPS:
        op = getattr(torch.ops.sdemc, name)
        assert str(op.default._schema).startswith("sdemc::" + name + "(")
    assert "Tensor(a0!) params" in str(torch.ops.sdemc.adam_step.default._schema)
    solver, payoff, disc = merton1d()
    t = torch_ops.inst_tensor(lower(solver, payoff, disc, num_paths=64))
    assert t.dtype == torch.uint8 and t.numel() == N.load().sdemc_inst_size()
    with pytest.raises(ValueError):
        torch_ops._inst(t[:-1])


def test_adapted_path_data_round_trip(tmp_path):
    """AdaptedPathData written to a .pt file and read back gives the same
    tensors and the same DataLoader items (no GPU needed)."""
    n, S, d = 8, 5, 2
    g = torch.Generator().manual_seed(0)
    paths = torch.rand((n, S + 1, d), generator=g)
    normals = torch.randn((n, S, d), generator=g)
    left = torch.rand((n, S + 1, d), generator=g)
    time_p = torch.linspace(0, 1, S + 1).repeat(n, 1).unsqueeze(-1)
    jumps = torch.zeros((n, S + 1, d))
    payoffs = torch.rand(n, generator=g)
    ds = sm.AdaptedPathData(paths, payoffs, normals, left, time_p, jumps, S)
    f = tmp_path / "data.pt"
    ds.save(str(f))
    back = sm.AdaptedPathData.load(str(f))
    for k, v in ds.tensors().items():
        w = back.tensors()[k]
        assert (torch.equal(v, w) if torch.is_tensor(v) else v == w), k
    a, b = ds[3], back[3]
    for x, y in zip(a[0], b[0]):
        assert torch.equal(x, y)
    assert torch.equal(a[1], b[1])


def test_heston_and_asian_lowering():
    from tests.cases import asian_merton, heston
    f = np.float32
    inst = inst_for(heston(24), num_paths=4)
    assert inst.model == N.MODEL_HESTON and inst.grid == N.GRID_UNIFORM and inst.rate == 0.0
    assert inst.drift_b[0] == f(0.02)
    assert list(inst.mark_p[:4]) == [f(2.0), f(2.0 * 0.04), f(0.3), f(0.3 ** 2)]
    a = inst_for(asian_merton(20), num_paths=4)
    assert a.model == N.MODEL_ASIAN and a.dim == 2 and a.grid == N.GRID_ADAPTED
    assert list(a.x0[:2]) == [1.0, 0.0] and list(a.jump_k[:2]) == [1.0, 0.0]
    assert a.drift_b[1] == 0.0 and a.diff_q[1] == 0.0 and a.rate == 2.0 and a.mark == N.MARK_LOGNORMAL
    assert a.payoff == N.PAYOFF_ASIANCALL
    # EulerScheme on a Heston model: the variance never moves, the price is a
    # GBM with volatility sqrt(v0)
    h = sm.Heston(0.02, 2.0, 0.04, 0.3, -0.7, torch.tensor([1., 0.04]))
    e = lower(sm.EulerSolver(h, 1.0, 10), sm.EuroCall(1.0), None, num_paths=4)
    assert e.model == N.MODEL_AFFINE and e.diff_q[0] == np.sqrt(f(0.04)) and e.diff_q[1] == 0.0
    with pytest.raises(NotImplementedError):
        lower(sm.HestonSolver(sm.Gbm(0.02, 0.2, torch.ones(2), 2), 1.0, 10), sm.EuroCall(1.0), None)


def test_descriptor_and_launch_validation_on_the_host():
    """Bad descriptors and launch shapes are refused before any device work
    (no GPU needed): model kinds outside their shapes, interleave values."""
    import ctypes
    from tests.cases import asian_merton, heston
    lib = N.load()
    fake = ctypes.c_void_p(256)  # never dereferenced: validation fails first
    out = ctypes.c_void_p(512)

    def price_rc(inst, cfg=None):
        return lib.sdemc_price_chunks(ctypes.byref(inst), N.byref(cfg), fake, 1 << 30, None, None)

    h = inst_for(heston(24), num_paths=64)
    h.grid = N.GRID_ADAPTED
    assert price_rc(h) == N.EUNSUPPORTED            # Heston steps on the uniform grid only
    a = inst_for(asian_merton(20), num_paths=64)
    a.dim = 3
    assert price_rc(a) == N.EUNSUPPORTED            # the Asian wrapper is 2-D
    a = inst_for(asian_merton(20), num_paths=64)
    a.model = 7
    assert price_rc(a) == N.EINVAL                  # unknown model kind
    ok = inst_for(merton1d(10), num_paths=64)
    assert price_rc(ok, N.SdemcCfg(interleave=3)) == N.EINVAL
    assert price_rc(ok, N.SdemcCfg(block_threads=48)) == N.EINVAL
    f = inst_for(merton1d(10), num_paths=64)
    assert lib.sdemc_price_f64(ctypes.byref(f), fake, 0, out, None) == N.ENOMEM
    lv = inst_for(levy2d(8), num_paths=64)
    assert lib.sdemc_price_f64(ctypes.byref(lv), fake, 1 << 30, out, None) == N.EUNSUPPORTED
    # the wait probe's poll limit is the kernels' own bound, 1 .. 2^22
    assert lib.sdemc_wait_probe(0, fake, None) == N.EINVAL
    assert lib.sdemc_wait_probe((1 << 22) + 1, fake, None) == N.EINVAL
    assert lib.sdemc_wait_probe(16, None, None) == N.EINVAL



def test_problem_presets_lower():
    """The reference's problem presets (sde_mc/problem.py) build on this
    package's classes and lower to descriptors (host only)."""
    presets = [sm.BlackScholesEuroCall.default_params(8, "cpu"), sm.BlackScholesRainbow.default_params(8, "cpu"),
               sm.HestonEuroCall.default_params(8, "cpu"), sm.MertonEuroCall.default_params(8, "cpu"),
               sm.LevyRainbow.default_params(8, "cpu"), sm.LevyRainbowMLMC(1, 1, 0.5, 2, 0.02, 0.3, 0.2, 0.001, 2,
                                                                            1, 1, 3, 8, "cpu"),
               sm.LevyCall.default_params(8, "cpu"), sm.LevyBestOf.default_params(8, "cpu"),
               sm.LevyCallOnMax.default_params(2, 8, "cpu"), sm.LevyCallOnMax.default_params(4, 8, "cpu")]
    dims = [1, 3, 2, 1, 2, 2, 1, 4, 2, 4]
    for prob, d in zip(presets, dims):
        assert prob.dim() == d
        inst = lower(prob.solver, prob.payoff, prob.discounter, num_paths=16)
        assert inst.dim == d and inst.num_steps == 8
    assert presets[2].solver.__class__.__name__ == "HestonSolver" and \
        lower(presets[2].solver, presets[2].payoff, presets[2].discounter).model == N.MODEL_HESTON
    assert presets[5].solver.exact_jumps
    assert isinstance(sm.LevyCallOnMax.default_params(3, 8, "cpu"), str)
    presets[0].set_steps(20)
    assert presets[0].solver.num_steps == 20


def test_c_client_compiles_and_runs(tmp_path):
    """include/sdemc.h is plain C: a C99 program fills a descriptor, sizes the
    scratch, plans a batch and sees malformed calls refused, linked against the
    library (no GPU involved)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = os.path.join(ROOT, "sde_mc_gb300", "lib")
    exe = str(tmp_path / "abi_client")
    src = os.path.join(ROOT, "tests", "c_client", "abi_client.c")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", lib, "-lsdemc", "-Wl,-rpath," + lib], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "c abi client ok" in out.stdout


def test_served_stream_law():
    """The served stream: Poisson arrivals at 2,000/s (exponential gaps), the
    basket-mix instance law, targets drawn from {1e-2, 3e-3, 1e-3}, request
    i on RNG stream i; a window starting at t_begin is the same requests,
    shifted (host only)."""
    from sde_mc_gb300 import stream as S
    reqs = S.make_stream(2000.0, 0.5, seed=1)
    n = len(reqs)
    assert abs(n - 1000) < 4 * math.sqrt(1000)
    gaps = np.diff([r.t for r in reqs])
    assert (gaps > 0).all() and abs(gaps.mean() * 2000.0 - 1.0) < 0.1
    assert abs(np.std(gaps) / gaps.mean() - 1.0) < 0.15   # exponential: cv = 1
    targets = [r.target for r in reqs]
    assert set(targets) == {1e-2, 3e-3, 1e-3}
    assert all(abs(targets.count(t) / n - 1 / 3) < 0.06 for t in (1e-2, 3e-3, 1e-3))
    assert [r.inst.stream_id for r in reqs] == [r.idx for r in reqs]
    assert {r.dim for r in reqs} == set(range(1, 9))
    win = S.make_stream(2000.0, 0.5, seed=1, t_begin=0.25)
    late = [r for r in reqs if r.t >= 0.25]
    assert [r.idx for r in win] == [r.idx for r in late]
    assert all(abs(a.t - (b.t - 0.25)) < 1e-12 for a, b in zip(win, late))


def test_jump_solver_host_samplers():
    """sample_jump_times / sample_one_jump (sde_mc/solvers.py:143-148) for
    callers that draw by hand: increasing exponential-gap times at the total
    rate, one mark per path repeated over the dimensions."""
    torch.manual_seed(3)
    m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1., 1.]), dim=2)
    sol = sm.JumpEulerSolver(m, 1.0, 10)
    jt = sol.sample_jump_times((20000, 4, 1))
    assert jt.shape == (20000, 4, 1) and bool((jt[:, 1:] >= jt[:, :-1]).all())
    assert float(jt[:, 0].mean()) == pytest.approx(0.5, rel=0.03)
    j = sol.sample_one_jump(5000)
    assert j.shape == (5000, 2) and bool((j[:, 0] == j[:, 1]).all())
    assert float(torch.log1p(j[:, 0]).mean()) == pytest.approx(-0.1, abs=0.015)


def test_public_names_cover_the_reference():
    """Every public name of sde_mc's package namespace (as listed when the
    fixtures were recorded) exists here, and the solver classes carry the
    reference's public methods."""
    names = ["AdaptedPathData", "AsianCall", "AsianWrapper", "Basket", "BestOf", "BinaryAoN", "ConstantShortRate",
             "ControlVariate", "DataLoader", "Digital", "DiffusionSolver", "DoubleGbm", "EulerScheme",
             "EulerSolver", "EuroCall", "EuroPut", "ExampleLevy", "ExpExampleLevy", "Gbm", "Gru", "Heston",
             "HestonRainbow", "HestonScheme", "HestonSolver", "InverseCdf", "JumpDiffusionSolver",
             "JumpEulerSolver", "Levy", "Levy2d", "LevySde", "LogGbm", "Lstm", "MCStatistics", "Merton", "Mlp",
             "NormalJumpsPathData", "NormalPathData", "Option", "Rainbow", "Sde", "SdeSolver", "ZeroFunction",
             "bs_asian_call", "bs_binary_aon", "bs_call", "bs_digital_call", "get_corr_matrix", "get_jump_comp",
             "mc_multilevel", "mc_simple", "merton_call", "partition", "poisson", "remove_steps", "run_mc",
             "solve_quadratic", "get_optimal_trials", "mc_estimates", "Problem", "HestonEuroCall"]
    missing = [n for n in names if not hasattr(sm, n)]
    assert not missing, missing
    for cls in (sm.SdeSolver, sm.DiffusionSolver, sm.JumpDiffusionSolver):
        assert hasattr(cls, "step") and hasattr(cls, "sample_corr_normals")
    assert hasattr(sm.JumpDiffusionSolver, "sample_jump_times") and hasattr(sm.JumpDiffusionSolver, "sample_one_jump")
