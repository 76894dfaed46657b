"""bench.py host logic without a GPU: the seed plumbing of the synthetic
workloads and the reference arm's JSON line (the CPU oracle timed on the
host cores), including its `unavailable` line for workloads the reference
has no CPU form of."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_every_workload_takes_a_seed_without_touching_the_table(bench):
    for name, cfg in bench.CONFIGS.items():
        assert bench.cfg_seed(cfg) == bench.SEED == 1234, name
        c = bench.with_seed(cfg, 7)
        assert bench.cfg_seed(c) == 7, name
        assert bench.cfg_seed(bench.CONFIGS[name]) == 1234, name
        assert c["workload"] == cfg["workload"]


def run_ref(*extra):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3", *extra], cwd=ROOT,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_reference_arm_line_on_the_host_cores():
    d = run_ref("--config", "cfg1", "--seed", "5")
    assert d["impl"] == "reference" and d["unit"] == "Mrays/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["config"]["config"] == "cfg1" and d["config"]["seed"] == 5
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


@pytest.mark.parametrize("config", ["cfg4", "build"])
def test_reference_arm_unavailable_without_a_cpu_form(config):
    d = run_ref("--config", config)
    assert d["impl"] == "reference" and "unavailable" in d


@pytest.mark.parametrize("name", ["svo_frame_cfg2", "volume_forward_cfg3", "volume_backward_cfg4"])
def test_profile_figures_the_bench_line_cites(bench, name):
    """The committed ncu summaries carry the figures the bench line reports
    beside its roofline: DRAM and L2 bytes per launch and the issue side."""
    t = bench.profile_traffic(name)
    l2 = bench.profile_l2(name)
    iss = bench.profile_issue(name)
    assert t and t > 1e6
    assert l2 and l2["bytes_per_launch"] > t and 0 < l2["pct_of_peak_sector_rate"] < 100
    assert iss and 0 < iss["issue_active_pct"] <= 100 and 0 < iss["simd_efficiency_pct"] <= 100
    assert iss["thread_instructions_per_unit"] > 0 and iss["unit"]
    assert name in iss["source"] and name in l2["source"]
