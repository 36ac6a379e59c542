"""Host-side pieces of bench.py that the JSON line depends on, on CPU:
recall, the clocks record (median SM clock under load, throttle reasons),
the DRAM-traffic record tied to its exact workload, the workload config and
the default step counts."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def args_for(**over):
    old = sys.argv
    sys.argv = ["bench.py"]
    try:
        a = bench.parse()
    finally:
        sys.argv = old
    for k, v in over.items():
        setattr(a, k, v)
    return a


def test_defaults_meet_the_timing_rules():
    a = args_for()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert (a.n, a.dim, a.nlist, a.m, a.pqk, a.nq, a.k) == (10_000_000, 96, 16384, 24, 256, 10_000, 10)


def test_recall_at():
    gt = np.array([[1, 2, 3], [4, 5, 6]])
    ids = np.array([[3, 2, 9, 1], [7, 8, 9, 4]])  # only the first k ids count
    assert bench.recall_at(ids, gt) == (2 / 3 + 0 / 3) / 2


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_record():
    c = bench.ClockSampler(0)
    c.proc = _FakeProc()
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1390.2, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 10, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    r = c.stop()
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    c.lines.append("0, 1200, 2070, 700, 0x8, Active, Not Active, Active, Not Active")
    assert bench.ClockSampler.stop(c)["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    none = bench.ClockSampler(0)
    assert none.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_traffic_record_only_for_its_workload():
    a = args_for()
    t = bench.scan_traffic(a, 32)
    assert t is not None and 2e9 < t < 2e10  # the captured launch's DRAM read + write bytes
    assert bench.scan_traffic(a, 128) is None  # another nprobe: another launch
    assert bench.scan_traffic(args_for(n=4_000_000), 32) is None
    assert bench.scan_traffic(args_for(m=16), 32) is None
    assert bench.scan_traffic(args_for(adc_tables="fp32"), 32) is None  # another kernel


def test_traffic_record_is_the_scan_stage():
    """The record's bytes are the scan stage's: the scan kernel and the
    selection kernel after it, the two kernels the roofline's time covers."""
    import json
    import os
    rec = json.load(open(os.path.join(os.path.dirname(bench.__file__), "profiles", "scan_adc_kernel_10Mx96_dram.json")))
    parts = rec["per_kernel"]
    assert set(parts) == {"scan_adc_kernel", "scan_select_kernel"}
    assert rec["dram_bytes_read_per_launch"] == sum(k["dram_bytes_read"] for k in parts.values())
    assert rec["dram_bytes_write_per_launch"] == sum(k["dram_bytes_write"] for k in parts.values())
    assert bench.scan_traffic(args_for(), 32) == rec["dram_bytes_read_per_launch"] + rec["dram_bytes_write_per_launch"]


def test_workload_config():
    """The config names the workload from the arguments alone, so both arms
    (and every rank) report the same one."""
    a = args_for()
    cfg = bench.workload_config(a, 32, 1)
    assert cfg["nprobe"] == 32 and cfg["mode"] == "exact_rerank"
    assert "240 MB of scan codes" in cfg["l2"] and "3.84 GB raw vectors" in cfg["l2"]
    assert "model" not in cfg
    assert bench.workload_config(a, 32, 1) == cfg


def test_compare_results_counts_only_real_mismatches():
    o_ids = np.array([[1, 2, 3], [4, 5, 6]])
    o_d = np.array([[0.1, 0.2, 0.3], [0.1, 0.2, 0.3]])
    o_n = np.array([3, 3])
    # a swap inside a tie of the reference distance is not a mismatch
    g_ids = np.array([[1, 3, 2], [4, 5, 6]])
    g_d = np.array([[0.1, 0.2, 0.2], [0.1, 0.2, 0.3]])
    o_d2 = np.array([[0.1, 0.2, 0.2], [0.1, 0.2, 0.3]])
    r = bench.compare_results(g_ids, g_d, o_n, o_ids, o_d2, o_n)
    assert r["id_mismatches_outside_ties"] == 0 and r["count_mismatches"] == 0 and r["max_rel_dist_err"] == 0
    # a different id at a different distance is one
    g_ids = np.array([[1, 2, 9], [4, 5, 6]])
    g_d = np.array([[0.1, 0.2, 0.25], [0.1, 0.2, 0.3]])
    r = bench.compare_results(g_ids, g_d, o_n, o_ids, o_d, o_n)
    assert r["id_mismatches_outside_ties"] == 1 and r["max_rel_dist_err"] > 0.1
    r = bench.compare_results(o_ids, o_d, np.array([3, 2]), o_ids, o_d, o_n)
    assert r["count_mismatches"] == 1


def test_rerank_depth_matches_the_library():
    assert bench.rerank_depth(10, 0) == 64 and bench.rerank_depth(10, 1) == 64
    assert bench.rerank_depth(100, 1) == 416 and bench.rerank_depth(1, 0) == 64


def test_serve_schedule_records():
    """The served stream's schedule: sorted arrivals at about the rate, 1% of
    each mutation kind, every record's range inside the array it indexes,
    kept searches' id slots disjoint and in order."""
    a = args_for()
    reqs, rows, add_ids, add_vecs, del_ids, kept, n_out = bench.serve_schedule(a, 2000.0, 3.0, 500, 16, 10_000, 5)
    assert abs(len(reqs) - 6000) < 400
    assert np.all(np.diff(reqs["at_ms"]) >= 0) and reqs["at_ms"].max() <= 3000.0
    kinds = reqs["kind"]
    assert 0.004 < np.mean(kinds == 1) < 0.02 and 0.004 < np.mean(kinds == 2) < 0.02
    s = kinds == 0
    assert (reqs["count"][s] >= 1).all() and (reqs["count"][s] <= 512).all()
    assert (reqs["k"][s] >= 1).all() and (reqs["k"][s] <= 100).all()
    assert (reqs["nprobe"][s] >= 8).all() and (reqs["nprobe"][s] <= 256).all()
    assert (reqs["first"][s] + reqs["count"][s]).max() == len(rows) and rows.max() < 500
    ad = kinds == 1
    assert (reqs["first"][ad] + reqs["count"][ad]).max() == len(add_ids) == len(add_vecs)
    np.testing.assert_allclose(np.linalg.norm(add_vecs, axis=1), 1.0, rtol=1e-5)
    de = kinds == 2
    assert (reqs["first"][de] + reqs["count"][de]).max() == len(del_ids) and del_ids.max() < 10_000
    end = 0
    for i, r, k, off in kept:
        assert reqs[i]["out_offset"] == off == end and k >= 10 and len(r) == reqs[i]["count"]
        end += len(r) * k
    assert end == n_out
    assert (reqs["out_offset"][~s] == 0).all()


def test_fp8_probe_study_on_cpu():
    """The FP8-against-BF16 probe study: each screen's band holds at least
    nprobe centroids, FP8's rounding error and band are the larger."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    c = rng.standard_normal((512, 32)).astype(np.float32)
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    q = torch.from_numpy((c[rng.integers(0, 512, 64)] + 0.3 * rng.standard_normal((64, 32))).astype(np.float32))
    r = bench.fp8_probe_study(torch, torch.device("cpu"), c, q, 8, nq=64)
    for kind in ("bf16", "fp8_e4m3"):
        assert r[kind]["band_mean"] >= 8 and r[kind]["band_max"] <= 512
    assert r["fp8_e4m3"]["operand_rel_err"] > 4 * r["bf16"]["operand_rel_err"]
    assert r["fp8_e4m3"]["band_mean"] > r["bf16"]["band_mean"]
