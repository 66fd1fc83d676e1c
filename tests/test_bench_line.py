"""The benchmark's result line (the last stdout line, the one a driver parses) stays a
compact, parseable JSON object with the contract keys, whatever the detail sections hold;
the oracle-comparison helpers count mismatches as the parity bar defines them."""
import argparse
import json

import numpy as np

import bench


def _fake_measurement():
    args = argparse.Namespace(workload="detector", tracks=1 << 22, seed=0xC0FFEE, schedule="mixed_sort_queue_learned",
                              steps=20, warmup=5, primaries=1 << 20)
    rows = []
    for shape in ("box", "tube", "cone", "tube_phi", "polycone", "polyhedron", "torus2", "trd", "box_minus_tube"):
        for prec in ("fp64", "mixed"):
            for q in bench.QUERY_BYTES:
                r = {"config": "cfg2", "shape": shape, "query": q, "precision": prec, "n": 1 << 22}
                if q in ("inside", "contains"):
                    r["mismatch_vs_oracle"] = 0
                else:
                    r.update(max_abs_err_vs_oracle=1.2e-12, beyond_tol_vs_oracle=0, bit_identical_to_oracle=1 << 22)
                rows.append(r)
    nav = {"state_mismatch": 0, "next_volume_mismatch": 0, "max_abs_err_vs_oracle": 0.0, "beyond_tol_vs_oracle": 0,
           "bit_identical_to_oracle": 1 << 22}
    parity = {"section": "parity_vs_oracle", "tracks": 1 << 22, "headline": nav, "plain_fp64": nav,
              "shapes": bench.shape_parity_summary(rows)}
    return {
        "value": 6.06e8, "ms_per_step": 6.92, "n": 1 << 22, "ws": 1, "args": args, "pool": 86_500_000,
        "ms_fp64": 182.0, "ms_fp64_sort": 25.9, "ids_equal": True, "step_err": 0.0, "e2e_value": 5.17e8,
        "e2e_calls": {"calls": 10, "min": 8.09, "median": 8.11, "max": 8.12}, "head": 15, "passes": 4,
        "roofline": {"bound": "hbm", "achieved": 58.0, "peak": 6668.5, "unit": "GB/s", "frac": 0.0087,
                     "traffic": 4.1e9, "kernel": "k_step_mixed_queue", "note": "x" * 200},
        "roofline_fp64": {"bound": "fp64", "achieved": 1.8e11, "peak": 6.2e11, "unit": "FP64 thread-ops/s",
                          "frac": 0.29, "ops_per_step": 302.6, "note": "y" * 80},
        "n_err": 0, "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 30},
        "parity": parity,
        "cpu_baseline": {"value": 1.6e7, "unit": "nav steps/s", "cores": 16, "kind": "port",
                         "single_thread_value": 1.1e6, "sample": "the first 131072 of the 4194304 step inputs"},
    }


def test_headline_line_is_compact_and_complete():
    line = bench.headline_line(_fake_measurement())
    text = json.dumps(line)
    assert len(text) < 4096, len(text)
    back = json.loads(text)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks",
                "gpu_launches", "ids_identical_to_fp64", "speedup_vs_plain_fp64", "speedup_vs_fp64_sort",
                "vs_oracle"):
        assert key in back, key
    assert back["value"] > 0 and back["e2e"]["value"] > 0
    assert back["e2e"]["h2d_bytes_per_step"] == (1 << 22) * 60
    assert back["vs_oracle"]["state_mismatch"] == 0
    assert back["vs_oracle"]["shape_queries"]["fp64"]["queries"] == 9 * 6 * (1 << 22)
    assert "\n" not in text


def test_compare_to_oracle_counts():
    ref = np.array([1.0, 2.0, bench.INF, 5.0, -1.0])
    gpu = np.array([1.0, 2.0 + 5e-10, bench.INF, 5.0 + 1e-8, -1.0])
    r = bench.compare_to_oracle(gpu, ref)
    assert r["beyond_tol_vs_oracle"] == 1
    assert r["bit_identical_to_oracle"] == 3
    assert abs(r["max_abs_err_vs_oracle"] - 1e-8) < 1e-12
    # a sentinel on one side only is a mismatch
    r = bench.compare_to_oracle(np.array([bench.INF]), np.array([3.0]))
    assert r["beyond_tol_vs_oracle"] == 1
    assert bench.compare_to_oracle(np.array([1, 3, 2], np.int32), np.array([1, 3, 3], np.int32)) == {
        "mismatch_vs_oracle": 1}


def test_nav_parity_compares_all_state_fields():
    o = np.zeros(3, bench.NAVSTATE_NP)
    o["nav_ind"] = [5, 6, 7]
    g = o.copy()
    g["on_boundary"][1] = 1
    g["pad"][2] = 9  # padding is not part of the state
    r = bench.nav_parity(g, np.zeros(3), o, np.zeros(3))
    assert r["state_mismatch"] == 1 and r["next_volume_mismatch"] == 0


def test_arguments_parse(monkeypatch):
    """The command lines the benchmark is run with parse (the driver's, the reference arm's,
    the profiling one), and every schedule the parser offers is defined."""
    import sys
    for argv in (["--gpus", "1", "--steps", "20", "--warmup", "5"], ["--impl", "reference"],
                 ["--tracks", "1048576", "--variants", "0", "--tune", "0", "--queue-blocks", "6"]):
        monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
        a = bench.parse()
        assert a.schedule in bench.SCHEDULES
    assert set(bench.SCHEDULES) >= {"fp64", "fp64_sort", "mixed_sort_queue", "mixed_sort_queue_learned"}
