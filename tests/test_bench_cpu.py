"""The benchmark's reference arm runs on the host cores alone (the CPU oracle
on a bounded particle sample): it prints one JSON line with the contract's
keys on rank 0, and other ranks of a torchrun launch exit 0 without work."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *args],
                          capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)


def test_reference_arm_prints_the_contract_line(oracle_lib):
    r = _run({}, "--steps", "1", "--warmup", "0", "--workload", "rk5-64")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "config", "cpu_baseline",
                "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def _full_line():
    """A result with every leg, shaped as bench.main() builds it."""
    acc = {"rows": {r: {"energy_rel_err_median": 1.23456789e-8, "energy_rel_err_p90": 4.5e-7,
                        "fraction_energy_err_le_1e-6": 0.93712345, "ks_energy": 0.0012345,
                        "mean_energy_rel_err": 1.234567e-5}
                    for r in ("1", "10", "50")}, "ks_bound": 0.010625}
    names = ("fp64", "fp64_fma", "fp32", "bf16", "fp32_learned", "bf16_learned",
             "fp64_fma_face", "fp32_face", "bf16_face", "fp32_learned_face", "bf16_learned_face")
    detail = {k: {"value": 1.2345678e8, "particle_gyroperiods_per_s": 12345.678901,
                  "launch": {"trial_ms": {"2": 1.0, "3": 2.0}}} for k in names}
    return {
        "metric": "accepted particle-steps/s (plain FP64 kernel)", "value": 4.8012345678e7,
        "unit": "particle-steps/s", "n_gpus": 1, "steps": 20, "warmup": 5,
        "ms_per_step": 970.123456, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded fields and particles)",
        "config": {"workload": "dop853-256", "method": "dop853", "grid": "256^3",
                   "spectrum": "kolmogorov", "particles": 1048576, "rtol": 1e-10,
                   "t_end_gyroperiods": 100, "window_gyroperiods": 0.05, "eta": 0.001,
                   "precision": "fp64", "l2": "x" * 80},
        "roofline": {"bound": "fp64", "achieved": 0.39012345, "peak": 1.2571234, "unit": "TFLOP/s",
                     "frac": 0.3101234, "traffic": 3.2e10, "frac_of_no_fma_peak": 0.7412345,
                     "peak_source": "y" * 200, "no_fma_note": "z" * 300},
        "e2e": {"value": 4.68e7, "unit": "particle-steps/s", "h2d_bytes_per_step": 226000000,
                "d2h_bytes_per_step": 164000000, "steps": 4, "api": "w" * 200},
        "cpu_baseline": {"value": 6.89e6, "unit": "particle-steps/s", "cores": 16, "kind": "port",
                         "sample": "s" * 90},
        "parity": {"bitwise": True, "particles": 603720, "mismatched": 0, "compared": "c" * 200},
        "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 100},
        "gpu_launches": 20, "rejected_fraction": 0.58712345, "stopped_particles": {},
        "plain_fma": {"roofline": {"frac": 0.4951234}},
        "mixed": {"accepted_steps_per_s": {k: v["value"] for k, v in detail.items()},
                  "detail": detail, "over_plain_exact": {k: 5.123456 for k in names},
                  "physics_rate_over_plain_exact": {k: 4.56789 for k in names},
                  "accuracy": {k: acc for k in names[1:]}},
        "learned": {"physics_rate_ratio": 0.95612345, "attempts_ratio": 0.812345,
                    "physics_rate_ratio_8_inputs": 0.9412345,
                    **{k: {"over_plain_exact": {"accepted": 5.123456, "simulated_time": 5.98765,
                                                "attempts": 0.5123},
                           "accuracy_1_gyroperiod": {"energy_rel_err_median": 2.6789e-9,
                                                     "fraction_energy_err_le_1e-6": 0.998123}}
                       for k in ("fp32_learned", "fp32_learned_face")}},
        "ensemble": {"a": "e" * 5000},
    }


def test_compact_line_is_small_and_complete():
    sys.path.insert(0, str(ROOT))
    import bench
    out = bench.compact_line(_full_line(), str(ROOT / "legs" / "bench_legs.json"))
    text = json.dumps(out)
    assert len(text) <= 1900, len(text)
    assert out["legs"] == "legs/bench_legs.json"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches", "parity", "targets"):
        assert key in out, key
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in out["roofline"], key
    assert len(out["targets"]) <= 10
    assert out["parity"]["bitwise"] is True
    assert "ensemble" not in out and "mixed" not in out
