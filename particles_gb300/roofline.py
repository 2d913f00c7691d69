"""Algorithmic floating-point work of the hot path, for roofline fractions.

Counting convention: every IEEE add, subtract, multiply, divide, square root
and real power is one flop (an FMA would be two).  The constants are the
counts measured by running the CPU oracle's own code on an op-counting number
type (``or_count_ops``); tests/test_oracle_kat.py checks that they still
agree.  They describe the minimal algorithm the GPU executes: the
reference's redundant evaluations (integrations.F90:156, :445-446, :576) are
not counted because they recompute values already held.
"""
from __future__ import annotations

import numpy as np

# key -> (method, what, with_eta) as understood by or_count_ops
COUNT_KEYS = {
    "eval": (1, 0, 0),          # one f(s): trilinear gather of U, B + Lorentz force
    "eval_j": (1, 0, 1),        # ... with the resistive eta J term (J gathered too)
    "rk5_stage": (1, 1, 0),     # RK5 attempt without its evaluations
    "dp853_stage": (2, 1, 0),   # DOP853 attempt without its evaluations
    "rk5_accept": (1, 2, 0),
    "rk5_reject": (1, 3, 0),
    "dp853_accept": (2, 2, 0),
    "dp853_reject": (2, 3, 0),
    "rk5_init": (1, 4, 0),      # dti_guess without its evaluation
    "dp853_init": (2, 4, 0),
    "rk5_sample": (1, 5, 0),    # one dense-output row
    "dp853_sample": (2, 5, 0),
}

FLOPS = {
    "eval": 161,
    "eval_j": 212,
    "rk5_stage": 385,
    "dp853_stage": 943,
    "rk5_accept": 4,
    "rk5_reject": 3,
    "dp853_accept": 6,
    "dp853_reject": 3,
    "rk5_init": 96,
    "dp853_init": 96,
    "rk5_sample": 82,
    "dp853_sample": 94,
}


def run_flops(method: str, cnt: np.ndarray, *, with_eta: bool = False, fresh: bool = True,
              resumed: int = 0, samples: int = 0) -> float:
    """Algorithmic flops of a run from its counters.

    ``cnt`` (np, 3) counter deltas of the run (all, accepted, rejected);
    ``fresh`` adds the initial-step guess per particle; ``resumed`` is the
    number of particles that re-derived f(si) on resume; ``samples`` the
    dense-output rows written.
    Evaluations: RK5 needs 5 per attempt plus 1 after each accept (stage 1 is
    kept across a rejection); DOP853 needs 11 per attempt plus f(sf) at each
    accept.  One evaluation per started or resumed particle gives f(si).
    """
    c = np.asarray(cnt, np.float64).reshape(-1, 3).sum(0)
    npart = np.asarray(cnt).reshape(-1, 3).shape[0]
    fe = FLOPS["eval_j" if with_eta else "eval"]
    if method in ("rk5", 1):
        evals = 5 * c[0] + c[1]
        f = c[0] * FLOPS["rk5_stage"] + c[1] * FLOPS["rk5_accept"] + c[2] * FLOPS["rk5_reject"]
        f += samples * FLOPS["rk5_sample"] + (npart * FLOPS["rk5_init"] if fresh else 0)
    else:
        evals = 11 * c[0] + c[1]
        f = c[0] * FLOPS["dp853_stage"] + c[1] * FLOPS["dp853_accept"] + c[2] * FLOPS["dp853_reject"]
        f += samples * FLOPS["dp853_sample"] + (npart * FLOPS["dp853_init"] if fresh else 0)
    evals += (npart if fresh else 0) + resumed
    return float(f + evals * fe)


def gather_bytes(method: str, cnt: np.ndarray, *, record_bytes: int) -> float:
    """Field bytes the gathers touch (8 corner records per evaluation)."""
    c = np.asarray(cnt, np.float64).reshape(-1, 3).sum(0)
    evals = (5 * c[0] + c[1]) if method in ("rk5", 1) else (11 * c[0] + c[1])
    return float(evals * 8 * record_bytes)


def split_work(method: str, cnt: np.ndarray, *, with_eta: bool = False) -> dict:
    """Work of a run split by where it executes in the mixed-precision kernels:
    the step machine (stage sums, error norm, controller: FP64), the
    evaluations (gather + force: FP64 in the FP64 builds, FP32 in the mixed
    ones) and their count.  Windows of a continuing run (no initial guess)."""
    c = np.asarray(cnt, np.float64).reshape(-1, 3).sum(0)
    if method in ("rk5", 1):
        evals = 5 * c[0] + c[1]
        machine = c[0] * FLOPS["rk5_stage"] + c[1] * FLOPS["rk5_accept"] + c[2] * FLOPS["rk5_reject"]
    else:
        evals = 11 * c[0] + c[1]
        machine = (c[0] * FLOPS["dp853_stage"] + c[1] * FLOPS["dp853_accept"]
                   + c[2] * FLOPS["dp853_reject"])
    return {"machine_flops": float(machine), "evals": float(evals),
            "eval_flops": float(evals * FLOPS["eval_j" if with_eta else "eval"])}


# bytes one evaluation gathers from each field store: 8 corners (FP64
# records 48 / 80 B; FP32 records 32 B, with J 32 + 4 B; BF16 brick records
# 16 / 32 B plus the brick's FP32 offset/scale pairs, 48 / 80 B)
EVAL_BYTES = {("fp64", False): 8 * 48, ("fp64", True): 8 * 80,
              ("fp64_fma", False): 8 * 48, ("fp64_fma", True): 8 * 80,
              ("fp32", False): 8 * 32, ("fp32", True): 8 * 36,
              ("bf16", False): 8 * 16 + 48, ("bf16", True): 8 * 32 + 80}


def mixed_roofline(method: str, precision: str, cnt: np.ndarray, seconds: float, *,
                   fp64_peak: float, hbm_peak: float, with_eta: bool = False) -> dict:
    """Roofline figures of one run of any build: FP64 flops per second and
    their fraction of the FP64 peak (for the mixed builds only the step
    machine's; their evaluations run in FP32), FP32 flops per second, and the
    gathered bytes per second against the HBM peak (an upper bound on the
    field traffic: most gathers hit L1/L2).  Peaks in flop/s and B/s."""
    w = split_work(method, cnt, with_eta=with_eta)
    mixed = precision in ("fp32", "bf16")
    f64 = w["machine_flops"] + (0.0 if mixed else w["eval_flops"])
    f32 = w["eval_flops"] if mixed else 0.0
    gb = w["evals"] * EVAL_BYTES[(precision, with_eta)]
    return {"bound": "fp64", "fp64_tflops": f64 / seconds / 1e12,
            "fp64_frac": f64 / seconds / fp64_peak, "fp32_tflops": f32 / seconds / 1e12,
            "gather_gbs": gb / seconds / 1e9, "gather_frac_of_hbm": gb / seconds / hbm_peak}
