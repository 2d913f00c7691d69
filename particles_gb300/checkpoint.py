"""Checkpoint and resume of a windowed run.

Everything a run needs to continue lives in five arrays: the state
(state(8,m,np) with the output rows written so far), the counters, the
per-particle status, the controller memory (the carry of pt_carry_bytes(np)
bytes: t, dt, errold, si, f(si), next output row, flags) and the window end
reached.  `save` writes them with the run's params and output times to one
.npz file; `load` returns them ready for the next window.  A run continued
from a checkpoint, in another process or on another GPU, is bit-identical
to the uninterrupted run (the carry keeps f(si), so nothing is re-evaluated).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

FORMAT = 1


def _host(a):
    """numpy view of a numpy array or a (CUDA) torch tensor."""
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def save(path, *, state, cnt, carry, status, t_reached, params, time, method, precision="fp64",
         extra: dict | None = None):
    path = Path(path)
    meta = {"format": FORMAT, "method": str(method), "precision": str(precision)}
    np.savez(path, state=_host(state), cnt=_host(cnt), carry=_host(carry).view(np.uint8),
             status=_host(status), t_reached=np.float64(t_reached), params=_host(params),
             time=_host(time), meta=np.array(repr({**meta, **(extra or {})})))
    return path if path.suffix == ".npz" else path.with_suffix(path.suffix + ".npz")


def load(path) -> dict:
    with np.load(path, allow_pickle=False) as z:
        out = {k: z[k] for k in ("state", "cnt", "carry", "status", "params", "time")}
        out["t_reached"] = float(z["t_reached"])
        import ast
        out["meta"] = ast.literal_eval(str(z["meta"]))
    if out["meta"].get("format") != FORMAT:
        raise ValueError(f"{path}: checkpoint format {out['meta'].get('format')} != {FORMAT}")
    npart = out["state"].shape[0]
    if out["cnt"].shape != (npart, 3) or out["status"].shape != (npart,):
        raise ValueError(f"{path}: inconsistent checkpoint arrays")
    return out
