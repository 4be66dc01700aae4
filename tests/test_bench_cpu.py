"""The bench's whole-sweep roofline arithmetic (no GPU): per-sweep algorithmic FLOPs of the
16x16 Hubbard workload (about 1.20e11 plus 8 N^2 per accepted flip and flavour) and the
roofline time of each form."""
import bench
from alf_gb300 import model as mdl


def test_sweep_flops_of_the_16x16_workload():
    m = mdl.config("hubbard16x16")
    f = bench.sweep_flops(m, 0, 0)
    n3 = 256.0 ** 3
    assert abs(sum(f.values()) - 2 * (24 * 100 + 2 * 10 * 58.7) * n3) < 1e-3 * sum(f.values())
    assert abs(sum(f.values()) - 1.20e11) < 0.01e11
    assert bench.sweep_flops(m, 1000, 0)["rank1"] == 2 * 8.0 * 256 * 256 * 1000
    t = bench.sweep_flops(m, 0, 1)
    assert t["tau_wraps"] == 2 * 20.0 * 100 * n3 and "tau_cgr2_2" in t


def test_sweep_roofline_of_each_form():
    m = mdl.config("hubbard16x16")
    r64 = bench.sweep_roofline(m, 20000, 0, 16, 4000.0, "fp64", 1.0, 2000.0)
    assert abs(r64["t_roof_ms"] - r64["flops_per_step"] / 1e12 * 1e3) < 1e-9 * r64["t_roof_ms"]
    assert abs(r64["frac"] - r64["t_roof_ms"] / 4000.0) < 1e-15
    rmx = bench.sweep_roofline(m, 20000, 0, 16, 4000.0, "mixed", 1.0, 2000.0)
    fl = rmx["flops_by_phase"]
    expect = (fl["decompose"] + fl["cgr"]) / 1e12 + (fl["wraps"] + fl["propagate"] + fl["rank1"]) / 2e15
    assert abs(rmx["t_roof_ms"] - 1e3 * expect) < 1e-9 * rmx["t_roof_ms"]
    assert rmx["t_roof_ms"] < r64["t_roof_ms"]


def test_reference_arm_prints_one_contract_line():
    # the host-core arm runs without a GPU: one JSON line with the reference markers
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--config",
                          "hubbard4x4", "--steps", "2", "--warmup", "1"], capture_output=True, text=True,
                         timeout=300, check=True).stdout.strip().splitlines()
    d = json.loads(out[-1])
    assert d["impl"] == "reference" and d["unit"] == "sweeps/s" and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 1


def test_grouped_roofline_sums_the_groups():
    a = mdl.hubbard("square", 6, 6, beta=4.0)
    b = mdl.config("hubbard16x16")
    g = bench.sweep_roofline_groups([(a, 100.0, 0, 3), (b, 2000.0, 0, 2)], 1000.0, "mixed", 1.0, 2000.0)
    one = bench.sweep_roofline(a, 100.0, 0, 3, 1000.0, "mixed", 1.0, 2000.0)
    two = bench.sweep_roofline(b, 2000.0, 0, 2, 1000.0, "mixed", 1.0, 2000.0)
    assert abs(g["t_roof_ms"] - one["t_roof_ms"] - two["t_roof_ms"]) < 1e-9 * g["t_roof_ms"]
    assert abs(g["flops_per_step"] - one["flops_per_step"] - two["flops_per_step"]) < 1e-6 * g["flops_per_step"]


def test_clock_summary_reports_the_median_clock_and_active_reasons():
    c = bench.ClockSampler(0)
    assert c.summary()["reasons"] == ["unsampled"]
    row = lambda sm, hw, pc: [sm, "2070", "900.1", "0x0", hw, "Not Active", "Not Active", pc]
    c.samples = [row("2070", "Not Active", "Not Active"), row("1980", "Not Active", "Active"),
                 row("2040", "Active", "Not Active"), row("[N/A]", "Not Active", "Not Active")]
    s = c.summary()
    assert s["sm_mhz"] == 2040.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 4
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_both_arms_share_one_config_object():
    # the reference arm and the GPU arm describe the same workload with the same object; how
    # each arm runs it lives in its own `arm` object
    a = bench.parse(["--impl", "reference"])
    b = bench.parse([])
    m, lt = bench.workload_model(a.config)
    assert bench.bench_config(a, m, lt) == bench.bench_config(b, m, lt)
    assert b.chains == 16 and b.precision == "mixed" and a.config == b.config == "hubbard16x16"
    assert bench.parse(["--config", "kondo12x12"]).chains == 32
