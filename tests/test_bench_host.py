"""Host-side pieces of the benchmark that need no GPU: the clock record of
the timed region, the algorithmic byte table behind the roofline, the
workload description and the reference arm's rank rule under torchrun."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _row(sm, smax, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return f"0, {sm}, {smax}, 812.40, 0x0000000000000000, {hw}, {hwt}, {swt}, {cap}"


def test_clock_summary_median_max_and_reasons():
    lines = [_row(2070, 2070), _row(2055, 2070, cap="Active"), _row(1980, 2070),
             "garbage", _row("[N/A]", 2070), ""]
    c = bench.summarize_clocks(lines)
    assert c["samples"] == 3
    assert c["sm_mhz"] == 2055.0
    assert c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == ["sw_power_cap"]


def test_clock_summary_reports_every_slowdown_kind():
    lines = [_row(1500, 2070, hw="Active"), _row(1400, 2070, hwt="Active"), _row(1300, 2070, swt="Active")]
    c = bench.summarize_clocks(lines)
    assert c["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert c["sm_mhz"] == 1400.0


def test_clock_summary_without_samples():
    c = bench.summarize_clocks([])
    assert c["sm_mhz"] is None and c["sm_max_mhz"] is None
    assert c["reasons"] == [] and c["samples"] == 0


def test_clock_sampler_without_process():
    s = bench.ClockSampler(0)
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]


@pytest.mark.parametrize("kernel", ["grad_ip_f64", "recover_f64", "error_f64", "esize_f64", "average_f64",
                                    "measure_f64", "mark_bits", "prep_f32", "tet_f32", "recover_f32",
                                    "error_f32", "average_f32", "measure_f32", "prep_l", "mlp_l", "error_l",
                                    "average_l", "measure_l"])
def test_algorithmic_bytes_positive(kernel):
    V, T, E = (9 ** 3, 6 * 8 ** 3, 3 * 8 * 81 + 3 * 64 * 9 + 512)
    b = bench.algorithmic_bytes(kernel, V, T, E)
    assert b is not None and b > 0


def test_algorithmic_bytes_of_the_recovery_at_160():
    """The recovery's algorithmic bytes per launch on the 160^3 box: CSR
    offsets, the vertex-to-element list, its weights, the packed element
    gradients, and the recovered values out (1.26 GB)."""
    V, T, E = 4173281, 24576000, 28902880
    b = bench.algorithmic_bytes("recover_f32", V, T, E)
    assert b == 4 * (V + 1) + 16 * T + 16 * T + 16 * T + 16 * V
    assert 1.25e9 < b < 1.27e9
    assert bench.algorithmic_bytes("no_such_kernel", V, T, E) is None


def test_pass_bytes_formula():
    assert bench.pass_bytes(10, 20, 40) == 96 * 10 + 96 * 20 + 8.25 * 40


def test_workload_desc_counts():
    d = bench.workload_desc(160, "fp32")
    assert (d["n_verts"], d["n_elems"], d["n_edges"]) == (4173281, 24576000, 28902880)
    assert d["precision"] == "fp32"
    assert "24576000 tets" in d["workload"]
    assert "larger than L2" in d["l2"]


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun only rank 0 runs the CPU reference arm and prints its
    line; the other ranks exit 0 and print nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "3", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_tiling_option_parses_and_refuses():
    assert bench.parse_tiling("0,0,0,0:256:16") == ([0, 0, 0, 0], 256, 16)
    assert bench.parse_tiling("1,2,4,0:1024:4") == ([1, 2, 4, 0], 1024, 4)
    for bad in ("0,0,0:256:16", "3,0,0,0:256:16", "0,0,0,0:256", "0,0,0,0:0:16", "0,0,0,0:256:-1"):
        with pytest.raises(ValueError):
            bench.parse_tiling(bad)
