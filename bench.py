#!/usr/bin/env python
"""Benchmark: accepted particle-steps/s of the fused GB300 integrator.

Workload (default, `dop853-256`): DOP853 FP64, rtol = atol = 1e-10, periodic
256^3 grid, B = x^ + Kolmogorov dB (dB_rms = 1, |n| in [1, 32]), V of the same
spectrum (V_rms = 0.2), E = -V x B + eta J with eta = 1e-3, 2^20 protons with
uniform positions, isotropic directions and gamma log-uniform in [1.001, 1e3],
t_end = 100 gyro-periods of B0 at gamma = 1 (qom = 200, c = 20, L = 1), dense
output at every gyro-period.  Inputs are seeded synthetic data.

A step is one window of that run: every particle advances from t to
t + window (default 0.05 gyro-periods) with its controller memory carried, so
successive steps continue the same trajectories the uninterrupted run
follows (bit for bit).  Warm-up steps run the first windows; the timed steps
the next ones.

Reported (one JSON line, rank 0):
  value      accepted particle-steps/s with everything resident in HBM,
             device time over the K timed steps (CUDA events + barrier)
  e2e        the same through the host-buffer C ABI (pt_integrate_fields):
             pinned host state/counters/carry copied in and out every step
  roofline   algorithmic FP64 flops of the timed kernel launches / their
             CUDA-event time, against the FP64 FMA peak measured live
  cpu_baseline  the CPU oracle (OpenMP, all host threads) on a seeded
             particle subsample of the same windows
  plain_fma  the same workload with the FMA build of the FP64 kernel (leg
             `fma`), with its roofline against the FMA-counted FP64 peak;
             plain_fma_face the same with face-capped trial steps, and
             plain_fma_accuracy both against the exact kernel
  mixed      the mixed-precision workload (RK5, 512^3, 2^22 particles) in
             every precision / controller variant, with per-particle
             energy and position errors against the exact kernel
  learned    the learned controller against the classical one (DOP853)
  ensemble   three snapshots in one persistent launch per window, as
             launches and as a CUDA graph, and with face-capped steps in
             the FMA build and in FP32 with the noise-floor norm
  targets    the plain kernel's roofline fractions and the mixed + learned
             ratios with their accuracy, gathered from the legs above

`--impl reference` times the reference algorithm on the host cores (the CPU
oracle, the restatement of sources/integrations.F90) on the same workload,
each step a bounded particle sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

QOM, VUN = 200.0, 1.0 / 20.0
T0 = 2.0 * math.pi / QOM

WORKLOADS = {
    # the headline FP64 workload (DOP853, 256^3, eta J, 2^20 particles)
    "dop853-256": dict(method="dop853", n=256, spectrum="kolmogorov", nmax=32, db_rms=1.0,
                       v_rms=0.2, eta=1e-3, npart=1 << 20, gamma=(1.001, 1e3), speed=None,
                       tol=1e-10, periods=100, seed=1, window=0.05),
    # the mixed-precision workload: RK5 rtol 1e-8, 512^3, 2^22 particles
    # windows of 0.1 gyro-periods: the slowest particles need ~100x the mean
    # attempts of a window, so shorter windows are set by their duration
    "rk5-512": dict(method="rk5", n=512, spectrum="kolmogorov", nmax=32, db_rms=1.0, v_rms=0.2,
                    eta=0.0, npart=1 << 22, gamma=(1.001, 1e2), speed=None, tol=1e-8,
                    periods=50, seed=2, window=0.1),
    # uneven batch in one persistent launch: three snapshots
    "ensemble-3": dict(method="dop853", n=(128, 192, 256), spectrum="kolmogorov", nmax=32,
                       db_rms=(0.5, 1.0, 2.0), v_rms=0.2, eta=0.0, npart=1 << 21,
                       split=(1, 2, 4), gamma=(1.0001, 1e4), speed=None,
                       tol=(1e-6, 1e-8, 1e-10), periods=10, seed=(1, 2, 3), window=0.02),
    # the CPU-runnable workload (reference RK5, 64^3, 1024 particles)
    "rk5-64": dict(method="rk5", n=64, spectrum="flat", nmax=4, db_rms=0.5, v_rms=0.1,
                   eta=0.0, npart=1024, gamma=None, speed=0.5, tol=1e-8, periods=10, seed=0,
                   window=1.0),
}


# Distance of the ensemble's open x faces outside the domain, in domain
# lengths (the field is periodic): particles stream along the guide field
# B0 x^ at up to c (20 domain lengths per unit time, 6.3 per 10 gyro-periods),
# so faces at the domain edge let 92 % of them out within the workload's 10
# gyro-periods.  Measured on a 2^17-particle sample of the three members
# (positions sampled every 0.1 gyro-period): 35 % leave at a margin of 3,
# 9.1 % at 5, 0.4 % at 6; 5.5 lets about 5 % leave.
ENSEMBLE_OPEN_X_MARGIN = 5.5


TRAIN_EPOCHS = 2


def train_controller(torch, records, method, face_feature=True):
    """Network + safety factor from accepted-step records: 90 % train
    (TRAIN_EPOCHS epochs of Adam on the GPU), the safety factor maximises
    the expected progress per attempt on the held-out 10 %
    (learned.choose_safety)."""
    from particles_gb300 import learned as LRN
    X, T = LRN.dataset(records, method, face_feature=face_feature)
    k = int(0.9 * X.shape[0])
    norm = LRN.normalisation(X[:k], T[:k])
    params, hist = LRN.train(torch, X[:k], T[:k], norm, epochs=TRAIN_EPOCHS, batch=16384,
                             lr=2e-3)
    safety, info = LRN.choose_safety(params, norm, X[k:], T[k:])
    model = LRN.Model(params, norm, safety=safety)
    return model, {"records": int(X.shape[0]), "mse_per_epoch": hist, "safety": safety,
                   "inputs": LRN.NIN if face_feature else LRN.NIN - 1, **info}

# Variants of the mixed-precision leg: (name, field precision).  "_learned":
# the learned controller proposes trial steps (trained on records of the
# exact classical run; with "_face", on records of the FP32 face-capped run);
# "_face": trial steps end just past the next cell face (PT_CTL_FACE);
# "_noise": the error norm with the FP32 evaluation's rounding floor
# (PT_CTL_NOISE).
MIXED_VARIANTS = (("fp64", "fp64"), ("fp64_fma", "fp64_fma"), ("fp32", "fp32"), ("bf16", "bf16"),
                  ("fp32_learned", "fp32"), ("bf16_learned", "bf16"), ("fp64_fma_face", "fp64_fma"),
                  ("fp32_face", "fp32"), ("bf16_face", "bf16"), ("fp32_learned_face", "fp32"),
                  ("bf16_learned_face", "bf16"), ("fp32_noise", "fp32"), ("bf16_noise", "bf16"),
                  ("fp32_learned_noise", "fp32"), ("bf16_learned_noise", "bf16"),
                  ("fp32_face_noise", "fp32"), ("bf16_face_noise", "bf16"),
                  ("fp32_learned_face_noise", "fp32"), ("bf16_learned_face_noise", "bf16"))

# DRAM bytes per attempt (dram__bytes_read.sum + dram__bytes_write.sum of one
# launch / the attempts it made), from a one-pass ncu capture of a small case
# of the same kernel and workload: 2^17 particles, the fourth window of the
# benchmark's window length (the bench's own first timed window).  A run's
# traffic per launch is this figure times the attempts of its launches.  The
# figure is an upper estimate at full size: with 8x fewer particles, fewer
# concurrently integrated particles share the field lines held in L2.
DRAM_BYTES_PER_ATTEMPT = {("dop853-256", "fp64"): (5439085056 + 1313298688) / 14067525}


def parse():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(k for k in WORKLOADS if k != "ensemble-3"),
                    default="dop853-256")
    ap.add_argument("--precision", choices=["fp64", "fp64_fma", "fp32", "bf16"], default="fp64")
    ap.add_argument("--controller", choices=["classical", "learned"], default="classical",
                    help="learned: the first warm-up window records accepted steps, a model "
                         "is trained on them and the later windows use it")
    ap.add_argument("--face", action="store_true",
                    help="face-capped trial steps (PT_CTL_FACE; not with --precision fp64)")
    ap.add_argument("--noise", action="store_true",
                    help="error norm with the FP32 evaluation's rounding floor (PT_CTL_NOISE)")
    ap.add_argument("--particles", type=int, default=0,
                    help="override the particle count (profiling of small cases only)")
    ap.add_argument("--window", type=float, default=0.0,
                    help="override the window in gyro-periods (profiling only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-controller leg")
    ap.add_argument("--no-order", action="store_true",
                    help="keep the natural queue order (default: longest first)")
    ap.add_argument("--order", choices=["work", "brick"], default="brick",
                    help="queue order: longest first (work), or longest-first classes "
                         "sorted inside by the Morton index of the particle's cell (brick; "
                         "+5-17 %% accepted steps/s for the mixed-precision kernels)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble leg")
    ap.add_argument("--ensemble-precision", choices=["fp64", "fp64_fma", "fp32"], default="fp64")
    ap.add_argument("--no-face-ensemble", action="store_true",
                    help="skip the ensemble's face-capped variants (FMA, and FP32 with the noise-floor norm)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="launch every kernel in its default variant (3 blocks per SM)")
    ap.add_argument("--records", type=int, default=10_000_000)
    ap.add_argument("--train-epochs", type=int, default=TRAIN_EPOCHS,
                    help="epochs of Adam for the learned controllers")
    ap.add_argument("--legs", default="headline,fma,mixed,learned,ensemble",
                    help="comma list of legs to run (headline always prints the line)")
    ap.add_argument("--mixed-steps", type=int, default=5)
    ap.add_argument("--accuracy-particles", type=int, default=32768)
    ap.add_argument("--accuracy-seconds", type=float, default=60.0,
                    help="time limit of the exact kernel's accuracy reference run")
    ap.add_argument("--legs-out",
                    default=os.path.join(tempfile.gettempdir(), "particles_gb300_bench_legs.json"),
                    help="file that receives the full result with every leg (stdout gets one "
                         "compact line)")
    return ap.parse_args()


def hbm_peak():
    """Measured HBM copy bandwidth (B/s) from the measured-peaks file when it
    is present, else the 6.8 TB/s fallback; returns (B/s, source)."""
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(f.read_text())["hbm_gbs"]) * 1e9, "measured"
    except (OSError, ValueError, KeyError):
        return 6.8e12, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_inputs(cfg, npart, rank, backend="numpy"):
    """Fields (reference layout), params, time grid and this rank's particles.
    backend "torch" synthesises the fields on the GPU (CUDA tensors)."""
    from particles_gb300 import fields, initial, params
    tmax = cfg["periods"] * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=cfg["tol"],
                             rtol=cfg["tol"], facmin=0.333, facmax=6.0, safe=0.9, beta=0.0)
    tg = params.time_grid(cfg["periods"], tmax)
    out = fields.snapshot(cfg["n"], db_rms=cfg["db_rms"], v_rms=cfg["v_rms"], vunit=VUN,
                          spectrum=cfg["spectrum"], nmin=1.0, nmax=cfg["nmax"],
                          seed=cfg["seed"], with_j=cfg["eta"] != 0.0, backend=backend)
    from particles_gb300.shard import particle_indices
    idx = particle_indices(rank, npart)
    s0 = initial.isotropic_state(npart, cfg["seed"], speed=cfg["speed"],
                                 gamma_range=cfg["gamma"], index=idx)
    return prm, tg, out, s0


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle_sample(cfg, s0_all, tg, nsub, seed=12345):
    import oracle
    idx = np.random.default_rng(seed).choice(s0_all.shape[0], nsub, replace=False)
    idx.sort()
    state = np.zeros((nsub, tg.size, 8))
    state[:, 0, :6] = s0_all[idx]
    return state, np.zeros((nsub, 3), np.int64), oracle.make_carry(nsub)


def _oracle_window(cfg, prm, tg, out, sample, t_stop, nthreads):
    import oracle
    uu, bb = out[:2]
    jj = out[2] if len(out) > 2 else None
    state, cnt, carry = sample
    oracle.integrate(cfg["method"], prm, tg, uu, bb, state, cnt, eta=cfg["eta"], jj=jj,
                     carry=carry, t_stop=t_stop, nthreads=nthreads)


def _calibrate(cfg, prm, tg, out, s0_all, window, nthreads, ncal=512):
    """Seconds per particle of the first window on the host (CPU oracle)."""
    sample = _oracle_sample(cfg, s0_all, tg, min(ncal, s0_all.shape[0]), seed=777)
    t = time.perf_counter()
    _oracle_window(cfg, prm, tg, out, sample, window * T0, nthreads)
    return (time.perf_counter() - t) / sample[0].shape[0]


def cpu_baseline(cfg, prm, tg, out, s0_all, window, warm, steps, seconds, gpu=None):
    """The CPU oracle (test infrastructure, here only the timed baseline) with
    all host threads on a seeded particle subsample, over exactly the windows
    the GPU timed (after the same warm-up windows); the subsample is sized so
    the timed part takes about ``seconds``.

    ``gpu`` (host copies of the GPU's counters, carry and first output rows
    after the same windows, from ``gpu_snapshot``) turns the same run into a
    parity check: the subsample's states from the oracle and from the kernel
    are compared bit for bit.  Returns (baseline, parity or None)."""
    nthreads = os.cpu_count() or 1
    per_particle = _calibrate(cfg, prm, tg, out, s0_all, window, nthreads)
    nsub = int(seconds / max(per_particle * steps, 1e-9))
    nsub = max(256, min(nsub, s0_all.shape[0]))
    sample = _oracle_sample(cfg, s0_all, tg, nsub)
    w = 0
    for _ in range(warm):
        w += 1
        _oracle_window(cfg, prm, tg, out, sample, w * window * T0, nthreads)
    cnt = sample[1]
    acc0 = cnt[:, 1].sum()
    t0 = time.perf_counter()
    for _ in range(steps):
        w += 1
        _oracle_window(cfg, prm, tg, out, sample, w * window * T0, nthreads)
    el = time.perf_counter() - t0
    acc = float(cnt[:, 1].sum() - acc0)
    base = {"value": acc / el, "unit": "particle-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{nsub} of {s0_all.shape[0]} particles, the same {steps} windows "
                      f"after {warm}: {int(acc)} accepted steps in {el:.1f} s"}
    return base, (parity_check(sample, gpu, s0_all.shape[0]) if gpu is not None else None)


def gpu_snapshot(torch, d_state, d_cnt, d_carry, npart, rows):
    """Host copies of what a window leaves behind for every particle: counters,
    the carry's t, dt, errold and current state si(6), and the first ``rows``
    output rows (the rows written so far)."""
    car = d_carry[: 15 * 8 * npart].view(torch.float64).view(15, npart)
    return {"cnt": d_cnt.cpu().numpy(), "t": car[0].cpu().numpy(), "dt": car[1].cpu().numpy(),
            "errold": car[2].cpu().numpy(), "si": car[3:9].t().cpu().numpy(),
            "state": d_state[:, :rows].cpu().numpy(), "rows": rows}


def parity_check(sample, gpu, npart, seed=12345):
    """Bit-for-bit comparison of the oracle's subsample (``_oracle_sample``'s
    seeded choice) with the GPU's snapshot of the same particles."""
    state, cnt, carry = sample
    nsub = state.shape[0]
    idx = np.random.default_rng(seed).choice(npart, nsub, replace=False)
    idx.sort()
    ca = np.ctypeslib.as_array(carry)
    o_t, o_dt, o_eo, o_si = ca["t"], ca["dt"], ca["errold"], ca["si"]
    r = gpu["rows"]
    bad = np.zeros(nsub, bool)
    bad |= (gpu["cnt"][idx] != cnt).any(1)
    for a, b in ((gpu["t"][idx], o_t), (gpu["dt"][idx], o_dt), (gpu["errold"][idx], o_eo)):
        bad |= a.view(np.int64) != np.ascontiguousarray(b, np.float64).view(np.int64)
    bad |= (gpu["si"][idx].view(np.int64)
            != np.ascontiguousarray(o_si, np.float64).view(np.int64)).any(1)
    bad |= (gpu["state"][idx].reshape(nsub, -1).view(np.int64)
            != np.ascontiguousarray(state[:, :r]).reshape(nsub, -1).view(np.int64)).any(1)
    return {"bitwise": bool(not bad.any()), "particles": int(nsub), "mismatched": int(bad.sum()),
            "compared": f"counters, t, dt, errold, x and u of every particle of the CPU sample "
                        f"and output rows 1..{r}, after the warm-up and timed windows"}


def run_reference(args, cfg, rank, world):
    """--impl reference: the reference algorithm (CPU oracle) on the host cores,
    each step one window of the workload over a seeded particle sample sized
    to about 6 s of host time."""
    if rank != 0:
        return 0
    npart = args.particles or cfg["npart"]
    window = args.window or cfg["window"]
    prm, tg, out, s0 = build_inputs(cfg, npart, 0)
    nthreads = os.cpu_count() or 1
    per_particle = _calibrate(cfg, prm, tg, out, s0, window, nthreads)
    nsub = max(256, min(int(6.0 / max(per_particle, 1e-9)), npart))
    sample = _oracle_sample(cfg, s0, tg, nsub)
    w = 0
    for _ in range(args.warmup):
        w += 1
        _oracle_window(cfg, prm, tg, out, sample, w * window * T0, nthreads)
    cnt = sample[1]
    acc0 = cnt[:, 1].sum()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w += 1
        _oracle_window(cfg, prm, tg, out, sample, w * window * T0, nthreads)
    el = time.perf_counter() - t0
    acc = float(cnt[:, 1].sum() - acc0)
    v = acc / el
    line = {
        "impl": "reference", "metric": "accepted particle-steps/s (plain FP64 kernel)", "value": v,
        "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(cfg, npart, window, args),
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": nthreads,
                         "kind": "port",
                         "sample": f"{nsub} seeded particles of the workload's {npart}, windows "
                                   f"of {window} gyro-periods ({args.warmup} warm-up, "
                                   f"{args.steps} timed)"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference is Fortran and cannot be built here (no Fortran compiler); its "
                "algorithm runs as the project's C++ restatement (oracle/), OpenMP over particles",
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(cfg, npart, window, args):
    return {
        "workload": args.workload, "method": cfg["method"], "grid": f"{cfg['n']}^3",
        "spectrum": cfg["spectrum"], "particles": npart, "rtol": cfg["tol"],
        "t_end_gyroperiods": cfg["periods"], "window_gyroperiods": window,
        "eta": cfg["eta"], "precision": args.precision,
        "l2": "field records exceed the 129 MB L2 (inputs larger than L2; no flush)",
    }


def stopped_particles(f, d_status, where):
    """Particles that ended with a negative status (reported, not fatal).

    The reference's trilinear gather computes the right-hand node from
    x + 1/dm separately from the left one (interpolations.F90:141-146); one
    ulp below some cell faces the two skip a node, so the interpolated field
    jumps there, adaptive steps shrink without bound and the reference loops
    forever (integrations.F90:361).  The exact kernel reproduces that
    arithmetic and stops such a particle with DT_UNDERFLOW."""
    from particles_gb300 import _native as N
    rc = f.run_check()
    if rc not in (N.PT_OK, N.PT_ERR_PARTICLE):
        raise RuntimeError(f"{where} failed: {N.last_error()}")
    st = d_status.cpu().numpy()
    names = {-2: "STEP_LIMIT", -3: "DT_UNDERFLOW", -4: "NONFINITE", -5: "TIMEOUT"}
    out = {}
    for code, name in names.items():
        k = int((st == code).sum())
        if k:
            out[name] = k
    return out


class QueueOrder:
    """Longest-first queue order for the persistent kernel: particles sorted
    by the attempts they needed in the previous window, so the slowest ones
    start first and the end-of-window tail stays short.  With ``cells`` (the
    grid's (dm1, dm2, dm3), unit domain) and the carry, the order is by work
    class (bit length of the attempts, longest first) and, inside a class, by
    the Morton index of the particle's cell, so the lanes of a warp start on
    neighbouring cells and share the 8^3 bricks they gather from.  The order
    changes which lane takes which particle, never a particle's result."""

    def __init__(self, torch, d_cnt, enabled=True, cells=None, d_carry=None):
        self.torch, self.cnt, self.enabled = torch, d_cnt, enabled
        self.prev = None
        self.order = None
        self.cells, self.carry = cells, d_carry
        if cells is not None:
            bits = max(int(d - 1).bit_length() for d in cells)
            v = torch.arange(1 << bits, device=d_cnt.device, dtype=torch.int64)
            spread = torch.zeros_like(v)
            for b in range(bits):
                spread |= ((v >> b) & 1) << (3 * b)
            self.spread = spread

    def before(self):
        if self.enabled:
            self.prev = self.cnt[:, 0].clone()
        return self.order

    def after(self):
        if not self.enabled:
            return
        torch = self.torch
        work = self.cnt[:, 0] - self.prev
        if self.cells is None:
            self.order = torch.argsort(work, descending=True).to(torch.int32)
            return
        n = work.shape[0]
        x = self.carry[: 9 * 8 * n].view(torch.float64)[3 * n: 6 * n].view(3, n)
        key = torch.zeros(n, dtype=torch.int64, device=work.device)
        for i in range(3):
            d = self.cells[i]
            c = torch.remainder(torch.floor(x[i] * d), d).to(torch.int64)
            key |= self.spread[c] << i
        cls = 63 - torch.bucketize(work, torch.tensor([1 << k for k in range(63)],
                                                      device=work.device), right=True)
        key |= cls << 40
        self.order = torch.argsort(key).to(torch.int32)


def tune(args, f, method, prm, d_time, d_state, stream, t_stop, **kw):
    """pt_autotune of the kernel the next runs launch (launch variant =
    register cap x threads per block); the choice becomes that kernel's
    default.  The trial is the first window itself, on all particles
    (scratch copies): per-particle work spreads over ~100x within a window, so
    short capped trials on a sample mispredict the full launch."""
    if args.no_autotune:
        return None
    (v, tpb), ms = f.autotune(method, prm, d_time, d_state, stream=stream.cuda_stream,
                              t_stop=t_stop, sample=-1, **kw)
    return {"blocks_per_sm": v, "threads_per_block": tpb, "trial": "first window, all particles",
            "trial_ms": {f"{b}x{t}": round(ms_, 3) for (b, t), ms_ in ms.items()}}


def plain_fma_leg(args, cfg, npart, window, prm, tg, out, s0, dev, stream, peak, rec_bytes,
                  face=False):
    """The headline workload again with the FMA build of the FP64 kernel (same
    algorithm and operand order, multiplies and adds contracted to FMAs):
    results within the FP64 tolerance of the CPU oracle instead of bit-identical,
    and its roofline against the FMA-counted FP64 peak.  face: with
    face-capped trial steps (PT_CTL_FACE)."""
    import torch
    from particles_gb300 import Fields, roofline
    from particles_gb300 import _native as N
    L = N.load()
    m = tg.size
    f = Fields(out[0], out[1], out[2] if len(out) > 2 else None, precision="fp64_fma")
    with torch.cuda.stream(stream):
        d_time = torch.tensor(tg, device=dev)
        d_state = torch.zeros((npart, m, 8), dtype=torch.float64, device=dev)
        d_state[:, 0, :6] = torch.tensor(s0, device=dev)
        d_cnt = torch.zeros((npart, 3), dtype=torch.int64, device=dev)
        d_status = torch.zeros(npart, dtype=torch.int32, device=dev)
        d_carry = torch.zeros(int(L.pt_carry_bytes(npart)), dtype=torch.uint8, device=dev)
    stream.synchronize()
    ordq = QueueOrder(torch, d_cnt, enabled=not args.no_order,
                      cells=(cfg["n"],) * 3 if args.order == "brick" else None, d_carry=d_carry)

    def run(w):
        order = ordq.before()
        f.run_device(cfg["method"], prm, d_time, d_state, d_cnt, d_status, d_carry,
                     eta=cfg["eta"], t_stop=w * window * T0, time_budget_s=900.0,
                     stream=stream.cuda_stream, order=order, face_steps=face)
        ordq.after()

    launch = tune(args, f, cfg["method"], prm, d_time, d_state, stream, window * T0, eta=cfg["eta"],
                  face_steps=face)
    w = 0
    for _ in range(args.warmup):
        w += 1
        run(w)
    stream.synchronize()
    acc0 = d_cnt.sum(0).cpu().numpy()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        w += 1
        ev[k][0].record(stream)
        run(w)
        ev[k][1].record(stream)
    stream.synchronize()
    dev_s = sum(a.elapsed_time(b) for a, b in ev) * 1e-3
    dcnt = d_cnt.cpu().numpy().sum(0) - acc0
    flops = roofline.run_flops(cfg["method"], np.array([dcnt]), with_eta=cfg["eta"] != 0.0,
                               fresh=False)
    res = {"value": float(dcnt[1]) / dev_s, "unit": "particle-steps/s", "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
           "rejected_fraction": float(dcnt[2] / max(dcnt[0], 1)),
           "particle_gyroperiods_per_s": npart * window * args.steps / dev_s,
           "controller": "classical, face-capped steps" if face else "classical",
           "roofline": {"bound": "fp64", "achieved": flops / dev_s / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / dev_s / peak,
                        "peak_source": "FP64 FMA peak measured live on this GPU (pt_probe_peak)"},
           "launch": launch, "precision": "fp64_fma",
           "parity": "within the FP64 tolerance of the CPU oracle (not bit-identical)"}
    f.close()
    del d_state, d_cnt, d_status, d_carry
    torch.cuda.empty_cache()
    return res


def headline_accuracy(cfg, prm, tg, out, s0, dev, na=16384):
    """Energy / position error of the FMA build, classical and with face-capped
    steps, against the exact kernel (bit-identical to the CPU oracle) on a
    subsample of the headline workload over one gyro-period."""
    import torch
    from particles_gb300 import Fields, errors
    from particles_gb300 import _native as N
    L = N.load()
    m = tg.size
    na = min(na, s0.shape[0])
    d_time = torch.tensor(tg, device=dev)
    res = {}
    for name, prec, face in (("fp64", "fp64", False), ("fp64_fma", "fp64_fma", False),
                             ("fp64_fma_face", "fp64_fma", True)):
        f = Fields(out[0], out[1], out[2] if len(out) > 2 else None, precision=prec)
        st = torch.zeros((na, m, 8), dtype=torch.float64, device=dev)
        st[:, 0, :6] = torch.tensor(s0[:na], device=dev)
        cnt = torch.zeros((na, 3), dtype=torch.int64, device=dev)
        status = torch.zeros(na, dtype=torch.int32, device=dev)
        carry = torch.zeros(int(L.pt_carry_bytes(na)), dtype=torch.uint8, device=dev)
        f.run_device(cfg["method"], prm, d_time, st, cnt, status, carry, eta=cfg["eta"],
                     t_stop=tg[1] * (1 + 1e-12), time_budget_s=900.0, face_steps=face,
                     stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.current_stream().synchronize()
        res[name] = st.cpu().numpy()
        f.close()
        del st, cnt, status, carry
    acc = {}
    for name in ("fp64_fma", "fp64_fma_face"):
        rep = errors.report(res["fp64"], res[name], rows=(1,), tgrid=tg / T0)
        rep["reference"] = "exact FP64 kernel (bit-identical to the CPU oracle)"
        rep["particles"] = na
        acc[name] = rep
    torch.cuda.empty_cache()
    return acc


def mixed_leg(args, dev, stream, peak):
    """The mixed-precision workload (RK5, rtol 1e-8, 512^3, 2^22 particles): accepted
    particle-steps/s of the exact FP64, FMA FP64 and mixed FP32 kernels on the
    same windows, and the mixed kernel's per-particle energy / position error
    against the exact kernel (bit-identical to the CPU oracle) at a common
    output time."""
    import torch
    from particles_gb300 import Fields, fields, initial, params, roofline
    cfg = WORKLOADS["rk5-512"]
    npart, window = cfg["npart"], cfg["window"]
    tmax = cfg["periods"] * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=cfg["tol"],
                             rtol=cfg["tol"], facmin=0.333, facmax=6.0, safe=0.9, beta=0.0)
    tg = params.time_grid(cfg["periods"], tmax)
    m = tg.size
    uu, bb = fields.snapshot(cfg["n"], db_rms=cfg["db_rms"], v_rms=cfg["v_rms"], vunit=VUN,
                             spectrum=cfg["spectrum"], nmin=1.0, nmax=cfg["nmax"],
                             seed=cfg["seed"], backend="torch")
    s0 = initial.isotropic_state(npart, cfg["seed"], gamma_range=cfg["gamma"])
    d_time = torch.tensor(tg, device=dev)
    out = {"workload": "rk5-512", "grid": "512^3", "particles": npart, "rtol": cfg["tol"],
           "window_gyroperiods": window, "steps": args.mixed_steps, "warmup": args.warmup}
    handles = {}
    for prec in ("fp64", "fp64_fma", "fp32", "bf16"):
        handles[prec] = Fields(uu, bb, precision=prec, stream=stream.cuda_stream)
    del uu, bb
    torch.cuda.empty_cache()

    def fresh(n):
        st = torch.zeros((n, m, 8), dtype=torch.float64, device=dev)
        st[:, 0, :6] = torch.tensor(s0[:n], device=dev)
        return (st, torch.zeros((n, 3), dtype=torch.int64, device=dev),
                torch.zeros(n, dtype=torch.int32, device=dev),
                torch.zeros(int(handles["fp64"]._L.pt_carry_bytes(n)), dtype=torch.uint8,
                            device=dev))

    from particles_gb300 import learned as LRN
    rates = {}
    model = model_face = None
    for name, prec in MIXED_VARIANTS:
        f = handles[prec]
        face = "_face" in name
        noise = "_noise" in name
        mdl = (model_face if face else model) if "_learned" in name else None
        st, cnt, status, carry = fresh(npart)
        launch = tune(args, f, "rk5", prm, d_time, st, stream, window * T0, model=mdl,
                      face_steps=face, noise_floor=noise)
        ordq = QueueOrder(torch, cnt, enabled=not args.no_order,
                          cells=(cfg["n"],) * 3 if args.order == "brick" else None, d_carry=carry)
        w = 0
        for _ in range(args.warmup):
            w += 1
            o = ordq.before()
            f.run_device("rk5", prm, d_time, st, cnt, status, carry, t_stop=w * window * T0,
                         time_budget_s=900.0, stream=stream.cuda_stream, order=o, model=mdl,
                         face_steps=face, noise_floor=noise)
            ordq.after()
        stream.synchronize()
        c0 = cnt.sum(0).cpu().numpy()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.mixed_steps):
            w += 1
            o = ordq.before()
            f.run_device("rk5", prm, d_time, st, cnt, status, carry, t_stop=w * window * T0,
                         time_budget_s=900.0, stream=stream.cuda_stream, order=o, model=mdl,
                         face_steps=face, noise_floor=noise)
            ordq.after()
        e1.record(stream)
        stream.synchronize()
        stopped = stopped_particles(f, status, f"mixed leg {name}")
        d = cnt.sum(0).cpu().numpy() - c0
        sec = e0.elapsed_time(e1) * 1e-3
        rates[name] = {"value": float(d[1]) / sec, "attempts_per_s": float(d[0]) / sec,
                       "rejected_fraction": float(d[2] / max(d[0], 1)),
                       "ms_per_step": 1e3 * sec / args.mixed_steps,
                       "particle_gyroperiods_per_s": npart * window * args.mixed_steps / sec,
                       "stopped_particles": stopped, "launch": launch,
                       "roofline": roofline.mixed_roofline("rk5", prec, d[None], sec,
                                                           fp64_peak=peak, hbm_peak=hbm_peak()[0])}
        if name == "fp64":
            # the plain integrator writes the learned controller's training records
            rec = LRN.record_buffer(torch, min(args.records, 4_000_000))
            w += 1
            f.run_device("rk5", prm, d_time, st, cnt, status, carry, t_stop=w * window * T0,
                         time_budget_s=900.0, stream=stream.cuda_stream, records=rec)
            stream.synchronize()
            model, out["learned_training"] = train_controller(
                torch, LRN.records_from_buffer(rec), "rk5")
            del rec
        if name == "fp32_face":
            # the face-capped controller's accepted steps train the network the
            # "_learned_face" variants use (steps that end just past a face)
            rec = LRN.record_buffer(torch, min(args.records, 4_000_000))
            w += 1
            f.run_device("rk5", prm, d_time, st, cnt, status, carry, t_stop=w * window * T0,
                         time_budget_s=900.0, stream=stream.cuda_stream, records=rec,
                         face_steps=True)
            stream.synchronize()
            model_face, out["learned_face_training"] = train_controller(
                torch, LRN.records_from_buffer(rec), "rk5")
            out["learned_face_training"]["recorded_in"] = "a window of the FP32 face-capped run"
            del rec
        del st, cnt, status, carry
        torch.cuda.empty_cache()
    out["accepted_steps_per_s"] = {k: v["value"] for k, v in rates.items()}
    out["detail"] = rates
    out["mixed_over_plain_exact"] = rates["fp32"]["value"] / rates["fp64"]["value"]
    out["bf16_over_plain_exact"] = rates["bf16"]["value"] / rates["fp64"]["value"]
    out["field_bytes"] = {k: h.nbytes for k, h in handles.items()}
    out["mixed_over_plain_fma"] = rates["fp32"]["value"] / rates["fp64_fma"]["value"]
    out["mixed_learned_over_plain_exact"] = rates["fp32_learned"]["value"] / rates["fp64"]["value"]
    out["physics_rate_mixed_learned_over_plain_exact"] = (
        rates["fp32_learned"]["particle_gyroperiods_per_s"]
        / rates["fp64"]["particle_gyroperiods_per_s"])
    out["over_plain_exact"] = {k: v["value"] / rates["fp64"]["value"] for k, v in rates.items()}
    out["physics_rate_over_plain_exact"] = {
        k: v["particle_gyroperiods_per_s"] / rates["fp64"]["particle_gyroperiods_per_s"]
        for k, v in rates.items()}
    out["bf16_learned_over_plain_exact"] = rates["bf16_learned"]["value"] / rates["fp64"]["value"]
    out["physics_rate_bf16_learned_over_plain_exact"] = (
        rates["bf16_learned"]["particle_gyroperiods_per_s"]
        / rates["fp64"]["particle_gyroperiods_per_s"])

    # accuracy of every variant on a seeded subsample at 1, 10 and 50
    # gyro-periods (the configuration's t_end): the exact kernel integrated
    # as far as the time budget allows (50 gyro-periods take ~25 s), every
    # other variant to the same output time.  Per-particle errors at late
    # times measure chaos; the energy histograms are compared by their
    # two-sample KS distance against the 95 % critical value 1.36 sqrt(2/n).
    na = min(args.accuracy_particles, npart)
    res = {}
    w_ref = cfg["periods"]
    t_acc = time.perf_counter()
    for name, prec in (MIXED_VARIANTS if na > 0 else ()):
        face = "_face" in name
        noise = "_noise" in name
        mdl = (model_face if face else model) if "_learned" in name else None
        st, cnt, status, carry = fresh(na)
        t_start = time.perf_counter()
        w = 0
        while True:
            w += 1
            handles[prec].run_device("rk5", prm, d_time, st, cnt, status, carry,
                                     t_stop=tg[min(w, m - 1)] * (1 + 1e-12), time_budget_s=900.0,
                                     stream=stream.cuda_stream, model=mdl, face_steps=face,
                                     noise_floor=noise)
            stream.synchronize()
            if w >= w_ref or (name == "fp64" and
                              time.perf_counter() - t_start > args.accuracy_seconds):
                break
        if name == "fp64":
            w_ref = w
        res[name] = (st.cpu().numpy(), w)
    from particles_gb300 import errors
    out["accuracy"] = {}
    ks_bound = 1.36 * math.sqrt(2.0 / max(na, 1))
    for prec, _ in (MIXED_VARIANTS[1:] if na > 0 else ()):
        nrow = min(res["fp64"][1], res[prec][1])       # sample index reached by both
        rep = errors.report(res["fp64"][0], res[prec][0], rows=(1, min(10, nrow), nrow),
                            tgrid=tg / T0)
        rep["reference"] = "exact FP64 kernel (bit-identical to the CPU oracle)"
        rep["particles"] = na
        rep["ks_bound"] = ks_bound
        rep["ks_within_bound"] = all(r["ks_energy"] < ks_bound for r in rep["rows"].values())
        out["accuracy"][prec] = rep
    out["accuracy_wall_seconds"] = time.perf_counter() - t_acc
    for mo in (model, model_face):
        if mo is not None:
            mo.close()
    for f in handles.values():
        f.close()
    return out


def ensemble_leg(args, dev, stream):
    """The ensemble workload: three snapshots (128^3, 192^3, 256^3; dB_rms 0.5, 1, 2;
    seeds 1-3) with 2^21 particles split 1:2:4, gamma log-uniform in
    [1.0001, 1e4], DOP853 at rtol 1e-6, 1e-8, 1e-10 and an open x boundary, in
    ONE persistent launch per window; finished and escaped particles are
    compacted out of the work lists between windows, which are reordered
    longest first.  Timed both as one launch sequence per window and as one
    captured CUDA graph of the same number of windows."""
    import torch
    from particles_gb300 import Ensemble, Fields, fields, initial, params
    cfg = WORKLOADS["ensemble-3"]
    prec = args.ensemble_precision
    tot = cfg["npart"]
    counts = [tot * w // sum(cfg["split"]) for w in cfg["split"]]
    counts[-1] = tot - sum(counts[:-1])
    tmax = cfg["periods"] * T0
    tg = params.time_grid(cfg["periods"], tmax)
    members, keep, fma_fields, f32_fields, s0s = [], [], [], [], []
    for k in range(3):
        prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=cfg["tol"][k],
                                 rtol=cfg["tol"][k], facmin=0.333, facmax=6.0, safe=0.9, beta=0.0)
        uu, bb = fields.snapshot(cfg["n"][k], db_rms=cfg["db_rms"][k], v_rms=cfg["v_rms"],
                                 vunit=VUN, spectrum=cfg["spectrum"], nmin=1.0, nmax=cfg["nmax"],
                                 seed=cfg["seed"][k], backend="torch")
        f = Fields(uu, bb, precision=prec, stream=stream.cuda_stream)
        if not args.no_face_ensemble:
            fma_fields.append(Fields(uu, bb, precision="fp64_fma", stream=stream.cuda_stream))
            f32_fields.append(Fields(uu, bb, precision="fp32", stream=stream.cuda_stream))
        del uu, bb
        torch.cuda.empty_cache()
        n = counts[k]
        s0 = initial.isotropic_state(n, cfg["seed"][k], gamma_range=cfg["gamma"])
        s0s.append(s0)
        st = torch.zeros((n, tg.size, 8), dtype=torch.float64, device=dev)
        st[:, 0, :6] = torch.tensor(s0, device=dev)
        members.append(dict(fields=f, params=prm, open_x=True,
                            open_x_margin=ENSEMBLE_OPEN_X_MARGIN,
                            time=torch.tensor(tg, device=dev), state=st,
                            cnt=torch.zeros((n, 3), dtype=torch.int64, device=dev),
                            status=torch.zeros(n, dtype=torch.int32, device=dev),
                            carry=torch.zeros(int(f._L.pt_carry_bytes(n)), dtype=torch.uint8,
                                              device=dev)))
        keep.append(f)
    launch = tune(args, members[2]["fields"], cfg["method"], members[2]["params"],
                  members[2]["time"], members[2]["state"], stream, cfg["window"] * T0)
    ens = Ensemble(cfg["method"], members, precision=prec)
    win = cfg["window"] * T0
    out = {"workload": "ensemble-3", "grids": ["128^3", "192^3", "256^3"],
           "particles": counts, "rtol": list(cfg["tol"]), "gamma": list(cfg["gamma"]),
           "precision": prec, "window_gyroperiods": cfg["window"], "open_x": True,
           "launch": launch}

    def accepted():
        return sum(int(m["cnt"][:, 1].sum()) for m in members)

    t = 0.0
    for _ in range(args.warmup):
        t += win
        ens.run(t, stream=stream.cuda_stream)
    stream.synchronize()
    res = {}
    for mode in ("launches", "graph"):
        a0 = accepted()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if mode == "graph":
            ens.capture(args.steps, win, stream=stream.cuda_stream)
            e0.record(stream)
            ens.replay(stream=stream.cuda_stream)
            e1.record(stream)
            t += args.steps * win
        else:
            e0.record(stream)
            for _ in range(args.steps):
                t += win
                ens.run(t, stream=stream.cuda_stream)
            e1.record(stream)
        stream.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3
        live, esc = ens.counts()
        res[mode] = {"accepted_steps_per_s": (accepted() - a0) / sec,
                     "ms_per_step": 1e3 * sec / args.steps,
                     "live": live.tolist(), "escaped": esc.tolist()}
    # launch-bound windows: a small ensemble (3 x 2048 particles on the same
    # snapshots) in windows short enough that the host's work per window --
    # seven launches and the Python call -- is comparable to the GPU's, run
    # as separate launches and as one captured graph of the same windows
    small = []
    for k in range(3):
        mb = members[k]
        n = 2048
        small.append(dict(fields=mb["fields"], params=mb["params"], open_x=True,
                          open_x_margin=ENSEMBLE_OPEN_X_MARGIN, time=mb["time"],
                          state=mb["state"][:n].clone(), cnt=torch.zeros((n, 3), dtype=torch.int64,
                                                                         device=dev),
                          status=torch.zeros(n, dtype=torch.int32, device=dev),
                          carry=torch.zeros(int(mb["fields"]._L.pt_carry_bytes(n)),
                                            dtype=torch.uint8, device=dev)))
    short = {}
    sw, k_short = win / 20.0, 100
    for mode in ("launches", "graph"):
        for mb in small:
            mb["cnt"].zero_(); mb["carry"].zero_()
        es = Ensemble(cfg["method"], small, precision=prec)
        ts = 0.0
        for _ in range(3):                               # warm-up windows
            ts += sw
            es.run(ts, stream=stream.cuda_stream)
        if mode == "graph":
            es.capture(k_short, sw, stream=stream.cuda_stream)
            es.run(ts, stream=stream.cuda_stream)        # the graph starts from this window end
        stream.synchronize()
        w0 = time.perf_counter()
        if mode == "graph":
            es.replay(stream=stream.cuda_stream)
        else:
            for _ in range(k_short):
                ts += sw
                es.run(ts, stream=stream.cuda_stream)
        stream.synchronize()
        wall = time.perf_counter() - w0
        es.close()
        short[mode] = {"windows": k_short, "particles": 3 * 2048,
                       "window_gyroperiods": cfg["window"] / 20.0,
                       "wall_us_per_window": 1e6 * wall / k_short}
    short["graph_speedup"] = (short["launches"]["wall_us_per_window"]
                              / short["graph"]["wall_us_per_window"])
    res["launch_bound_windows"] = short
    rc = ens.check()
    live, esc = ens.counts()
    out.update(res)
    out["escaped_fraction"] = float(esc.sum()) / tot
    out["t_gyroperiods"] = t / T0
    out["check"] = int(rc)
    ens.close()
    for f in keep:
        f.close()
    def fast_run(flds, fprec, noise):
        """The same ensemble from the same initial states with face-capped
        trial steps (and the noise-floor norm when `noise`): warm-up and
        timed windows as launches.  Returns (result, ensemble, members, t)."""
        fm = [dict(mb, fields=flds[k],
                   state=torch.zeros_like(mb["state"]), cnt=torch.zeros_like(mb["cnt"]),
                   status=torch.zeros_like(mb["status"]), carry=torch.zeros_like(mb["carry"]))
              for k, mb in enumerate(members)]
        for k, mb in enumerate(fm):
            mb["state"][:, 0, :6] = torch.tensor(s0s[k], device=dev)
        ef = Ensemble(cfg["method"], fm, precision=fprec, face_steps=True, noise_floor=noise)
        tf = 0.0
        for _ in range(args.warmup):
            tf += win
            ef.run(tf, stream=stream.cuda_stream)
        stream.synchronize()
        a0 = sum(int(m["cnt"][:, 1].sum()) for m in fm)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            tf += win
            ef.run(tf, stream=stream.cuda_stream)
        e1.record(stream)
        stream.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3
        c = sum(m["cnt"].sum(0).cpu().numpy() for m in fm)
        r = {"accepted_steps_per_s": (int(c[1]) - a0) / sec,
             "ms_per_step": 1e3 * sec / args.steps,
             "over_exact_launches": (int(c[1]) - a0) / sec
             / res["launches"]["accepted_steps_per_s"],
             "simulated_time_per_s_over_exact_launches":
             res["launches"]["ms_per_step"] / (1e3 * sec / args.steps),
             "rejected_fraction": float(c[2] / max(c[0], 1)),
             "check": int(ef.check())}
        return r, ef, fm, tf

    if f32_fields:
        # FP32 store, face-capped steps and the noise-floor norm
        r32, ef32, fm32, _ = fast_run(f32_fields, "fp32", True)
        out["fp32_face_noise"] = r32
        ef32.close()
        del fm32
        for f in f32_fields:
            f.close()
        torch.cuda.empty_cache()
    if fma_fields:
        # the FMA build with face-capped trial steps
        out["fma_face"], ef, fm, tf = fast_run(fma_fields, "fp64_fma", False)
        del members
        torch.cuda.empty_cache()
        # the rest of the configuration's 10 gyro-periods, as one captured
        # graph of windows of half a gyro-period with compaction between them
        wf = 0.5 * T0
        k_rest = int(math.ceil((tmax - tf) / wf - 1e-9))
        a0 = sum(int(m["cnt"][:, 1].sum()) for m in fm)
        ef.capture(k_rest, wf, stream=stream.cuda_stream)
        e0.record(stream)
        ef.replay(stream=stream.cuda_stream)
        e1.record(stream)
        stream.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3
        live, esc = ef.counts()
        c = sum(m["cnt"].sum(0).cpu().numpy() for m in fm)
        st_all = np.concatenate([m["status"].cpu().numpy() for m in fm])
        out["full_run"] = {"build": "FP64 FMA, face-capped steps", "t_gyroperiods": tmax / T0,
                           "graph_windows": k_rest, "window_gyroperiods": 0.5,
                           "seconds": sec, "accepted_steps_per_s": (int(c[1]) - a0) / sec,
                           "accepted_steps": int(c[1]), "rejected_fraction":
                           float(c[2] / max(c[0], 1)), "live": live.tolist(),
                           "escaped": esc.tolist(), "escaped_fraction": float(esc.sum()) / tot,
                           "done_fraction": float((st_all == 0).mean()),
                           "open_x_margin": ENSEMBLE_OPEN_X_MARGIN, "check": int(ef.check())}
        ef.close()
        for f in fma_fields:
            f.close()
    return out


def learned_leg(args, dev, stream):
    """The learned-controller workload (DOP853 rtol 1e-10, 256^3 with eta J):
    controllers trained on accepted-step records of the plain integrator with
    field seed 10 (the nine-input network, and the eight-input one without
    the cell-face input), then evaluated with field seed 11 on 2^20
    particles: the exact FP64 kernel with the classical controller (the
    plain kernel), with either network, and the mixed-precision kernel (FP32
    fields and gather) with the classical controller, the network, face-capped
    steps and both -- accepted steps/s, attempts, rejected fraction and
    simulated particle time per second, and the energy error of the mixed
    variants against the exact kernel after one gyro-period."""
    import torch
    from particles_gb300 import Fields, errors, fields, initial, learned, params
    cfg = WORKLOADS["dop853-256"]
    npart, window = cfg["npart"], cfg["window"]
    steps, warm = min(args.steps, 8), min(args.warmup, 3)
    tmax = cfg["periods"] * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=cfg["tol"],
                             rtol=cfg["tol"], facmin=0.333, facmax=6.0, safe=0.9, beta=0.0)
    tg = params.time_grid(cfg["periods"], tmax)
    d_time = torch.tensor(tg, device=dev)

    def setup(seed, precisions=("fp64",)):
        uu, bb, jj = fields.snapshot(cfg["n"], db_rms=cfg["db_rms"], v_rms=cfg["v_rms"],
                                     vunit=VUN, spectrum=cfg["spectrum"], nmin=1.0,
                                     nmax=cfg["nmax"], seed=seed, with_j=True, backend="torch")
        fs = {p: Fields(uu, bb, jj, precision=p, stream=stream.cuda_stream) for p in precisions}
        del uu, bb, jj
        torch.cuda.empty_cache()
        s0 = initial.isotropic_state(npart, seed, gamma_range=cfg["gamma"])
        st = torch.zeros((npart, tg.size, 8), dtype=torch.float64, device=dev)
        st[:, 0, :6] = torch.tensor(s0, device=dev)
        cnt = torch.zeros((npart, 3), dtype=torch.int64, device=dev)
        status = torch.zeros(npart, dtype=torch.int32, device=dev)
        carry = torch.zeros(int(fs["fp64"]._L.pt_carry_bytes(npart)), dtype=torch.uint8,
                            device=dev)
        return fs, st, cnt, status, carry

    # records from the classical run, field seed 10
    fs, st, cnt, status, carry = setup(10)
    f = fs["fp64"]
    rec = learned.record_buffer(torch, args.records)
    t_rec = time.perf_counter()
    w = 0
    while True:
        w += 1
        f.run_device("dop853", prm, d_time, st, cnt, status, carry, eta=cfg["eta"],
                     t_stop=w * 0.01 * T0, time_budget_s=900.0, stream=stream.cuda_stream,
                     records=rec)
        stream.synchronize()
        n_rec = int(rec[:2].cpu().numpy().view(np.uint64)[0])
        if n_rec >= args.records or w >= 40:
            break
    records = learned.records_from_buffer(rec)
    t_rec = time.perf_counter() - t_rec
    del rec, st, cnt, status, carry
    f.close()
    torch.cuda.empty_cache()
    t_tr = time.perf_counter()
    model, training = train_controller(torch, records, "dop853")
    model8, training8 = train_controller(torch, records, "dop853", face_feature=False)
    t_tr = time.perf_counter() - t_tr
    out = {"workload": "dop853-256, field seed 11 (trained on seed 10)",
           "record_seconds": t_rec, "train_seconds": t_tr, "training": training,
           "training_8_inputs": training8, "steps": steps, "warmup": warm,
           "target": "accepted log dt + at most log 2 of error headroom"}
    fs, st, cnt, status, carry = setup(11, ("fp64", "fp32"))
    snap = (st.clone(), cnt.clone(), carry.clone())
    variants = (("classical", "fp64", None, False), ("learned", "fp64", model, False),
                ("learned_8_inputs", "fp64", model8, False), ("fp32", "fp32", None, False),
                ("fp32_learned", "fp32", model, False), ("fp32_face", "fp32", None, True),
                ("fp32_learned_face", "fp32", model, True), ("fp32_noise", "fp32", None, False),
                ("fp32_learned_noise", "fp32", model, False),
                ("fp32_face_noise", "fp32", None, True),
                ("fp32_learned_face_noise", "fp32", model, True))
    for name, prec, mdl, face in variants:
        f = fs[prec]
        noise = "_noise" in name
        st.copy_(snap[0]); cnt.copy_(snap[1]); carry.copy_(snap[2])
        launch = tune(args, f, "dop853", prm, d_time, st, stream, window * T0, eta=cfg["eta"],
                      model=mdl, face_steps=face, noise_floor=noise)
        ordq = QueueOrder(torch, cnt, enabled=not args.no_order,
                          cells=(cfg["n"],) * 3 if args.order == "brick" else None, d_carry=carry)
        w = 0
        for _ in range(warm):
            w += 1
            o = ordq.before()
            f.run_device("dop853", prm, d_time, st, cnt, status, carry, eta=cfg["eta"],
                         t_stop=w * window * T0, time_budget_s=900.0,
                         stream=stream.cuda_stream, order=o, model=mdl, face_steps=face,
                         noise_floor=noise)
            ordq.after()
        stream.synchronize()
        c0 = cnt.sum(0).cpu().numpy()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            w += 1
            o = ordq.before()
            f.run_device("dop853", prm, d_time, st, cnt, status, carry, eta=cfg["eta"],
                         t_stop=w * window * T0, time_budget_s=900.0,
                         stream=stream.cuda_stream, order=o, model=mdl, face_steps=face,
                         noise_floor=noise)
            ordq.after()
        e1.record(stream)
        stream.synchronize()
        stopped = stopped_particles(f, status, f"learned leg {name}")
        d = cnt.sum(0).cpu().numpy() - c0
        sec = e0.elapsed_time(e1) * 1e-3
        out[name] = {"accepted_steps_per_s": float(d[1]) / sec,
                     "attempts_per_s": float(d[0]) / sec,
                     "rejected_fraction": float(d[2] / max(d[0], 1)),
                     "attempts": int(d[0]), "accepted": int(d[1]),
                     "particle_gyroperiods_per_s": npart * window * steps / sec,
                     "stopped_particles": stopped, "launch": launch, "precision": prec}
    # energy error of every variant against the exact kernel after one gyro-period
    na = min(16384, npart)
    res = {}
    for name, prec, mdl, face in variants:
        s1 = torch.zeros((na, tg.size, 8), dtype=torch.float64, device=dev)
        s1[:, 0] = snap[0][:na, 0]
        c1 = torch.zeros((na, 3), dtype=torch.int64, device=dev)
        q1 = torch.zeros(na, dtype=torch.int32, device=dev)
        k1 = torch.zeros(int(fs[prec]._L.pt_carry_bytes(na)), dtype=torch.uint8, device=dev)
        fs[prec].run_device("dop853", prm, d_time, s1, c1, q1, k1, eta=cfg["eta"],
                            t_stop=tg[1] * (1 + 1e-12), time_budget_s=900.0,
                            stream=stream.cuda_stream, model=mdl, face_steps=face,
                            noise_floor="_noise" in name)
        stream.synchronize()
        res[name] = s1.cpu().numpy()
    for name, *_ in variants[1:]:
        out[name]["accuracy_1_gyroperiod"] = errors.report(res["classical"], res[name],
                                                           rows=(1,))["rows"]["1"]
    model.close()
    model8.close()
    for f in fs.values():
        f.close()
    c = out["classical"]
    for name, *_ in variants[1:]:
        l = out[name]
        l["over_plain_exact"] = {"accepted": l["accepted_steps_per_s"] / c["accepted_steps_per_s"],
                                 "simulated_time": l["particle_gyroperiods_per_s"]
                                 / c["particle_gyroperiods_per_s"],
                                 "attempts": l["attempts"] / c["attempts"]}
    for name in ("learned", "learned_8_inputs"):
        sfx = "" if name == "learned" else "_8_inputs"
        for key, sub in (("accepted_steps_per_s_ratio", "accepted"),
                         ("physics_rate_ratio", "simulated_time"), ("attempts_ratio", "attempts")):
            out[key + sfx] = out[name]["over_plain_exact"][sub]
    return out


def _r(x, d=4):
    """Rounds floats to ``d`` significant digits (compact output)."""
    if isinstance(x, float):
        return float(f"{x:.{d}g}")
    if isinstance(x, dict):
        return {k: _r(v, d) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_r(v, d) for v in x]
    return x


def targets(line):
    """At most ten headline figures gathered from the legs: the plain kernel's
    roofline fractions, the mixed + learned ratios against the plain exact and
    FMA kernels as [accepted steps/s, simulated time per second], and their
    accuracy."""
    t = {}
    roof = line.get("roofline", {})
    t["exact_frac_fp64_peak"] = roof.get("frac")
    t["exact_frac_no_fma_peak"] = roof.get("frac_of_no_fma_peak")
    if "plain_fma" in line:
        t["fma_frac_fp64_peak"] = line["plain_fma"]["roofline"]["frac"]
    mx = line.get("mixed")
    if mx:
        ov, ph = mx["over_plain_exact"], mx["physics_rate_over_plain_exact"]
        fma = mx["accepted_steps_per_s"]["fp64_fma"]
        fma_ph = mx["detail"]["fp64_fma"]["particle_gyroperiods_per_s"]
        pick = {k: mx["accepted_steps_per_s"][k] for k in mx["accepted_steps_per_s"]
                if "_learned" in k}
        best = max(pick, key=pick.get)
        t["mixed_learned_rk5"] = {
            "variant": best, "x_exact": [ov[best], ph[best]],
            "x_fma": [pick[best] / fma, mx["detail"][best]["particle_gyroperiods_per_s"] / fma_ph]}
        acc = mx.get("accuracy", {}).get(best)
        if acc:
            last = max(acc["rows"], key=int)
            r1, rl = acc["rows"]["1"], acc["rows"][last]
            t["mixed_learned_rk5_err"] = {
                "t1_median": r1["energy_rel_err_median"],
                "t1_le_1e-6": r1["fraction_energy_err_le_1e-6"],
                f"t{last}_ks": rl["ks_energy"], "ks_bound": acc.get("ks_bound"),
                f"t{last}_mean": rl["mean_energy_rel_err"]}
    if "learned" in line:
        lr = line["learned"]
        t["learned_vs_classical_dop853"] = {
            "sim_time": lr["physics_rate_ratio"], "attempts": lr["attempts_ratio"],
            "sim_time_8_inputs": lr.get("physics_rate_ratio_8_inputs")}
        ml = {k: lr[k] for k in ("fp32_learned", "fp32_learned_face", "fp32_learned_noise",
                                 "fp32_learned_face_noise") if k in lr}
        if ml:
            best = max(ml, key=lambda k: ml[k]["over_plain_exact"]["simulated_time"])
            acc = ml[best].get("accuracy_1_gyroperiod", {})
            ox = ml[best]["over_plain_exact"]
            t["mixed_learned_dop853"] = {
                "variant": best, "x_exact": [ox["accepted"], ox["simulated_time"]],
                "t1_median": acc.get("energy_rel_err_median"),
                "t1_le_1e-6": acc.get("fraction_energy_err_le_1e-6")}
    return {k: v for k, v in t.items() if v is not None}


def compact_line(line, legs_path):
    """The one JSON line on stdout (under 2 KB): the contract's keys for the
    headline kernel; every leg in full goes to ``legs_path``."""
    roof = line["roofline"]
    out = {k: line[k] for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup",
                                 "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                                 "dtype", "data") if k in line}
    cfg = dict(line["config"])
    cfg["l2"] = "inputs > L2, no flush"
    out["config"] = cfg
    out["roofline"] = {"bound": roof["bound"], "achieved": roof["achieved"],
                       "peak": roof["peak"], "unit": roof["unit"], "frac": roof["frac"],
                       "traffic": roof.get("traffic"),
                       "peak_source": "FP64 FMA rate measured live",
                       "frac_of_no_fma_peak": roof.get("frac_of_no_fma_peak")}
    for k in ("e2e", "cpu_baseline", "parity", "clocks", "gpu_launches", "rejected_fraction",
              "stopped_particles"):
        if line.get(k) not in (None, {}):
            out[k] = line[k]
    if "e2e" in out:
        out["e2e"] = {k: out["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step",
                                                 "d2h_bytes_per_step")}
    if "parity" in out:
        out["parity"] = {k: out["parity"][k] for k in ("bitwise", "particles", "mismatched")}
    try:                                        # the side file, relative to the repository
        out["legs"] = str(Path(legs_path).resolve().relative_to(ROOT))
    except ValueError:
        out["legs"] = legs_path
    out = _r(out)
    out["targets"] = _r(targets(line), 3)
    return out


def main():
    global TRAIN_EPOCHS
    args = parse()
    TRAIN_EPOCHS = args.train_epochs
    rank, world, local = dist_env()
    cfg = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, cfg, rank, world)

    import torch
    from particles_gb300 import Fields, roofline
    from particles_gb300 import _native as N
    import ctypes as C

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    npart = args.particles or cfg["npart"]
    window = args.window or cfg["window"]
    big = cfg["n"] >= 512
    prm, tg, out, s0 = build_inputs(cfg, npart, rank, backend="torch" if big else "numpy")
    L = N.load()
    m = tg.size
    dev = torch.device("cuda", local)
    f = Fields(out[0], out[1], out[2] if len(out) > 2 else None, precision=args.precision)
    if big:                                   # host copies only for the CPU baseline
        out = tuple(a.cpu().numpy() for a in out) if not args.no_cpu else None
        torch.cuda.empty_cache()
    rec_bytes = {"fp32": (9 if cfg["eta"] != 0.0 else 8) * 4,
                 "bf16": (16 if cfg["eta"] != 0.0 else 8) * 2}.get(
        args.precision, (10 if cfg["eta"] != 0.0 else 6) * 8)
    stream = torch.cuda.Stream(device=dev)
    # Every torch operation of the run (allocations, queue orders, fresh
    # states) goes to the stream the kernels run on: the caching allocator
    # then reuses a freed block only for work ordered after the kernels that
    # read it (a queue-order array freed while a queued window still reads
    # it would otherwise be overwritten under that window).
    torch.cuda.set_stream(stream)
    with torch.cuda.stream(stream):
        d_time = torch.tensor(tg, device=dev)
        d_state = torch.zeros((npart, m, 8), dtype=torch.float64, device=dev)
        d_state[:, 0, :6] = torch.tensor(s0, device=dev)
        d_cnt = torch.zeros((npart, 3), dtype=torch.int64, device=dev)
        d_status = torch.zeros(npart, dtype=torch.int32, device=dev)
        d_carry = torch.zeros(int(L.pt_carry_bytes(npart)), dtype=torch.uint8, device=dev)
    stream.synchronize()

    model = None
    training = None
    ordq = QueueOrder(torch, d_cnt, enabled=not args.no_order,
                      cells=(cfg["n"],) * 3 if args.order == "brick" else None, d_carry=d_carry)

    def window_run(w, records=None):
        order = ordq.before()
        f.run_device(cfg["method"], prm, d_time, d_state, d_cnt, d_status, d_carry,
                     eta=cfg["eta"], t_stop=w * window * T0, time_budget_s=900.0,
                     stream=stream.cuda_stream, order=order, model=model, records=records,
                     face_steps=args.face, noise_floor=args.noise)
        ordq.after()

    w = 0
    if args.controller == "learned":
        from particles_gb300 import learned as LRN
        rec = LRN.record_buffer(torch, min(args.records, 4_000_000))
        w += 1
        window_run(w, records=rec)
        stream.synchronize()
        model, training = train_controller(torch, LRN.records_from_buffer(rec), cfg["method"])
        training["recorded_in"] = "the first warm-up window (classical controller)"
        del rec
    launch = tune(args, f, cfg["method"], prm, d_time, d_state, stream, window * T0,
                  eta=cfg["eta"], model=model, face_steps=args.face, noise_floor=args.noise)
    for _ in range(args.warmup - w):
        w += 1
        window_run(w)
    stream.synchronize()
    stopped_particles(f, d_status, "warm-up")
    acc0 = d_cnt.sum(0).cpu().numpy()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t_start = time.perf_counter()
        for k in range(args.steps):
            w += 1
            ev[k][0].record(stream)
            window_run(w)
            ev[k][1].record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t_start
    if world > 1:
        torch.distributed.barrier()
    stopped = stopped_particles(f, d_status, "timed run")
    # what the timed windows left behind, for the bitwise comparison with the
    # CPU oracle's sample over the same windows (rows written so far + 1)
    snap = None
    if not args.no_cpu and rank == 0 and world == 1 and args.precision == "fp64" \
            and args.controller == "classical":
        rows = min(m, int(w * window + 1e-9) + 2)
        snap = gpu_snapshot(torch, d_state, d_cnt, d_carry, npart, rows)
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(kern_ms) * 1e-3
    c_now = d_cnt.cpu().numpy()
    dcnt_tot = c_now.sum(0) - acc0
    accepted = float(dcnt_tot[1])
    elapsed = dev_s
    if world > 1:
        from particles_gb300.shard import combine
        elapsed, accepted = combine(torch, elapsed, accepted, device=dev)
    value = accepted / elapsed

    # roofline of the dominant (only) kernel: algorithmic FP64 flops / event time
    flops = roofline.run_flops(cfg["method"], np.array([dcnt_tot]), with_eta=cfg["eta"] != 0.0,
                               fresh=False)
    achieved = flops / dev_s
    pk = C.c_double()
    L.pt_probe_peak(0, 16384, C.byref(pk))
    peak = pk.value
    pk2 = C.c_double()
    L.pt_probe_peak(2, 16384, C.byref(pk2))
    peak_split = pk2.value
    bpa = DRAM_BYTES_PER_ATTEMPT.get((args.workload, args.precision))
    traffic = bpa * float(dcnt_tot[0]) / args.steps if bpa else None
    roof = {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic, "traffic_unit": "DRAM bytes per launch (one window)",
            "traffic_rule": ("DRAM bytes per attempt of a one-pass ncu capture of a 2^17-particle "
                             "window of the same kernel and workload x this run's attempts per "
                             "window (upper estimate)") if bpa else None,
            "peak_source": "FP64 FMA peak measured live on this GPU (pt_probe_peak); "
                           "the measured-peaks file lists only HBM and bf16",
            "peak_no_fma": peak_split / 1e12,
            "frac_of_no_fma_peak": achieved / peak_split,
            "no_fma_note": "the exact kernel may not contract (bit identity with the CPU "
                           "restatement): separate FP64 multiply/add chains measured live bound "
                           "what its FP64 pipe alone can do; it exceeds that bound because part "
                           "of its correctly rounded multiplies run on the integer pipes",
            "flops_per_step": flops / args.steps,
            "gather_bytes_per_step": roofline.gather_bytes(cfg["method"], np.array([dcnt_tot]),
                                                           record_bytes=rec_bytes) / args.steps}

    line = {
        "metric": ("accepted particle-steps/s (plain FP64 kernel)"
                   if args.precision == "fp64" and args.controller == "classical"
                   else f"accepted particle-steps/s ({args.precision}, {args.controller} controller"
                        f"{', face-capped steps' if args.face else ''})"),
        "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64_fma": "f64", "fp32": "f64 step machine, f32 gather/force",
                  "bf16": "f64 step machine, f32 gather/force, bf16 field store"}[args.precision],
        "data": "synthetic (seeded fields and particles)",
        "config": workload_config(cfg, npart, window, args),
        "wall_s_timed": wall, "gpu_launches": args.steps, "stopped_particles": stopped,
        "rejected_fraction": float(dcnt_tot[2] / max(dcnt_tot[0], 1)),
        "attempts_per_s": float(dcnt_tot[0]) / elapsed,
        "particle_gyroperiods_per_s": world * npart * window * args.steps / elapsed,
        "roofline": roof, "clocks": clocks.summary(), "launch": launch,
        "controller": args.controller + (", face-capped steps" if args.face else "")
                      + (", noise-floor norm" if args.noise else ""),
    }
    if training:
        line["learned_training"] = training

    # end to end through the host-buffer C ABI: pinned host copies every step
    if not args.no_e2e and rank == 0:
        h_state = torch.empty((npart, m, 8), dtype=torch.float64).pin_memory()
        h_cnt = torch.empty((npart, 3), dtype=torch.int64).pin_memory()
        h_carry = torch.empty(int(L.pt_carry_bytes(npart)), dtype=torch.uint8).pin_memory()
        h_status = torch.empty(npart, dtype=torch.int32).pin_memory()
        h_state.copy_(d_state.cpu())
        h_cnt.copy_(d_cnt.cpu())
        h_carry.copy_(d_carry.cpu())
        e2e_acc0 = float(h_cnt[:, 1].sum())
        k_e2e = max(1, min(args.steps, 4))
        from particles_gb300.integrations import _options
        from particles_gb300.params import method_id
        xfer_sum = np.zeros(2, np.int64)
        t_e = time.perf_counter()
        for _ in range(k_e2e):
            w += 1
            o = _options(args.precision, eta=cfg["eta"], t_stop=w * window * T0,
                         status=None, carry=None, time_budget_s=900.0, model=model,
                         face_steps=args.face, noise_floor=args.noise)
            o.status = C.c_void_p(h_status.data_ptr())
            o.carry = C.c_void_p(h_carry.data_ptr())
            rc = L.pt_integrate_fields(method_id(cfg["method"]), npart, m, f.handle, prm.ctypes.data_as(C.c_void_p),
                                       tg.ctypes.data_as(C.c_void_p),
                                       C.c_void_p(h_state.data_ptr()), C.c_void_p(h_cnt.data_ptr()),
                                       C.byref(o))
            if rc != N.PT_OK:
                raise RuntimeError(f"e2e step failed: {N.last_error()}")
            xfer = np.zeros(2, np.int64)
            L.pt_last_transfer_bytes(xfer.ctypes.data_as(C.c_void_p))
            xfer_sum += xfer
        el_e = time.perf_counter() - t_e
        acc_e = float(h_cnt[:, 1].sum()) - e2e_acc0
        line["e2e"] = {"value": acc_e / el_e, "unit": "particle-steps/s",
                       "h2d_bytes_per_step": int(xfer_sum[0] // k_e2e),
                       "d2h_bytes_per_step": int(xfer_sum[1] // k_e2e),
                       "steps": k_e2e, "api": "pt_integrate_fields (host pinned buffers: "
                       "state(8,m,np), counters, carry, status in and out every step)"}

    leg_s = {}
    t_leg = time.perf_counter()
    if (args.precision == "fp64" and args.controller == "classical" and rank == 0
            and "fma" in set(args.legs.split(",")) and args.workload == "dop853-256"):
        line["plain_fma"] = plain_fma_leg(args, cfg, npart, window, prm, tg, out, s0, dev, stream,
                                          peak, rec_bytes)
        line["plain_fma_face"] = plain_fma_leg(args, cfg, npart, window, prm, tg, out, s0, dev,
                                               stream, peak, rec_bytes, face=True)
        line["plain_fma_accuracy"] = headline_accuracy(cfg, prm, tg, out, s0, dev)
        leg_s["fma"] = time.perf_counter() - t_leg

    if not args.no_cpu and rank == 0 and world == 1:
        t_leg = time.perf_counter()
        line["cpu_baseline"], par = cpu_baseline(cfg, prm, tg, out, s0, window, args.warmup,
                                                 args.steps, args.cpu_seconds, gpu=snap)
        if par is not None:
            line["parity"] = par
        snap = None
        leg_s["cpu_baseline"] = time.perf_counter() - t_leg
    legs = set(args.legs.split(","))
    if not args.no_mixed and "mixed" in legs and rank == 0 and args.workload == "dop853-256":
        f.close()
        del d_state, d_cnt, d_status, d_carry
        torch.cuda.empty_cache()
        t_leg = time.perf_counter()
        line["mixed"] = mixed_leg(args, dev, stream, peak)
        leg_s["mixed"] = time.perf_counter() - t_leg
    if not args.no_learned and "learned" in legs and rank == 0 and args.workload == "dop853-256":
        torch.cuda.empty_cache()
        t_leg = time.perf_counter()
        line["learned"] = learned_leg(args, dev, stream)
        leg_s["learned"] = time.perf_counter() - t_leg
    if not args.no_ensemble and "ensemble" in legs and rank == 0 and args.workload == "dop853-256":
        torch.cuda.empty_cache()
        t_leg = time.perf_counter()
        line["ensemble"] = ensemble_leg(args, dev, stream)
        leg_s["ensemble"] = time.perf_counter() - t_leg
    line["leg_wall_seconds"] = leg_s
    if rank == 0:
        legs_out = Path(args.legs_out)
        legs_out.parent.mkdir(parents=True, exist_ok=True)
        legs_out.write_text(json.dumps(line, indent=1))
        print(json.dumps(compact_line(line, str(legs_out))), flush=True)
    if model is not None:
        model.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    f.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
