"""Host tests of the benchmark's arithmetic: the per-path-step work counts
behind the roofline, the choice of the binding ceiling, the clock record's
parser and the peak fallbacks.  No GPU."""
import bench


def test_work_per_path_step():
    # Box-Muller, sqrt(dt), Euler: 15 flops at d = 1; the Cholesky product adds d (d + 1)
    assert bench.algorithmic_flops_per_path_step(1) == 15
    assert bench.algorithmic_flops_per_path_step(2) == 31
    assert bench.algorithmic_flops_per_path_step(8) == 5 + 80 + 72
    # two MUFU ops per normal and one for sqrt(dt), five per jump event
    assert bench.mufu_per_path_step(1) == 3
    assert bench.mufu_per_path_step(2, 0.5) == 7.5


def _roof(fp32_frac, mufu_frac):
    return {"bound": "fp32", "achieved": 10.0 * fp32_frac, "peak": 10.0, "unit": "TFLOP/s", "frac": fp32_frac,
            "peak_source": "ffma probe", "traffic": 123,
            "mufu": {"achieved": 2.0 * mufu_frac, "peak": 2.0, "unit": "Tops/s", "frac": mufu_frac,
                     "peak_source": "mufu probe"}}


def test_binding_ceiling_is_the_larger_fraction():
    r = bench.bind_roofline(_roof(0.3, 0.1))
    assert (r["bound"], r["frac"], r["unit"]) == ("fp32", 0.3, "TFLOP/s")
    assert r["fp32"]["frac"] == 0.3 and r["mufu"]["frac"] == 0.1 and r["traffic"] == 123
    r = bench.bind_roofline(_roof(0.06, 0.12))
    assert (r["bound"], r["frac"], r["unit"], r["peak"]) == ("mufu", 0.12, "Tops/s", 2.0)
    assert r["achieved"] / r["peak"] == r["frac"]
    assert r["fp32"]["frac"] == 0.06 and r["fp32"]["peak_source"] == "ffma probe"


def test_clock_record_parser():
    c = bench.ClockSampler(0)
    assert c.summary()["reasons"] == ["unsampled"]
    c.lines = ["0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 1200.5, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2010, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "garbage line", "0, [N/A], 2070, 0, 0x0, a, b, c, d"]
    s = c.summary()
    assert s["sm_mhz"] == 1980 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.lines.append("0, 1400, 2070, 1300, 0x8, Not Active, Active, Not Active, Not Active")
    assert bench.ClockSampler.summary(c)["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_peak_fallbacks_are_the_stated_measurements():
    assert bench.HBM_FALLBACK_GBS == 6800.0 and bench.BF16_FALLBACK_TFLOPS == 1900.0
    assert bench.load_json_file("no_such_file.json") is None


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm is rank 0's: another rank exits 0
    at once, with no output and no process group."""
    import os
    import subprocess
    import sys
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], env=env, cwd=root, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
