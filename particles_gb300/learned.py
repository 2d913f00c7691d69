"""The learned step-size controller: recording, training and the model handle.

Records come from the classical integrator itself (``pt_run_device`` with a
record buffer): for every accepted step, the nine controller features at its
start (the eight of the controller specification and the time to the next
cell face over the last step), its log(dt) and log(error ratio).  A model
trained with ``face_feature=False`` sees the ninth input as zero: the
8 -> 64 -> 64 -> 1 network of the first eight.  The regression target is the
accepted step enlarged by what its error ratio says it could have been, at
most by a factor of 2: log dt - clip(log err, -(order) log 2, 0) / order.
In a trilinear field the accepted error ratios are bimodal (steps inside a
cell sit near 1e-12, steps across a cell face near 1), so the error model
alone (unclipped) would propose steps that cross the next face and fail;
the accepted steps themselves are a conservative but attainable target.  Training runs on the
GPU with the library's own FP32 kernels (``pt_mlp_loss_grad``,
``pt_mlp_adam``); inference runs on the FP16 tensor cores inside the
integrator.  The embedded error estimate still accepts or rejects every
step, and a rejection falls back to the classical controller.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .integrations import _stream

FEATURES = ["log|B|", "log|E|", "log gamma", "pitch cosine", "log(|grad B|/|B|)",
            "log(Omega dt_prev)", "log(err_prev)", "log dt_prev", "log(t_face / dt_prev)"]
NIN = len(FEATURES)
REC_FLOATS = NIN + 2
assert REC_FLOATS == N.REC_FLOATS
REC_HEADER_FLOATS = 4
ORDER = {"rk5": 5, "dop853": 8, 1: 5, 2: 8}


def record_buffer(torch, capacity: int, device="cuda"):
    """Zeroed device buffer for ``capacity`` records (header included)."""
    return torch.zeros(REC_HEADER_FLOATS + capacity * REC_FLOATS, dtype=torch.float32,
                       device=device)


def records_from_buffer(buf) -> np.ndarray:
    """(n, 11) float32 records out of a device record buffer."""
    raw = buf.cpu().numpy()
    n = int(raw[:2].view(np.uint64)[0])
    cap = (raw.size - REC_HEADER_FLOATS) // REC_FLOATS
    n = min(n, cap)
    return raw[REC_HEADER_FLOATS:REC_HEADER_FLOATS + n * REC_FLOATS].reshape(n, REC_FLOATS)


def dataset(records: np.ndarray, method, face_feature: bool = True
            ) -> tuple[np.ndarray, np.ndarray]:
    """Features X (n, 9) and the target log trial step (n,) from records;
    rows with a non-finite entry are dropped.  face_feature=False zeroes the
    ninth input (the 8-input network)."""
    rec = np.asarray(records, np.float64)
    log_dt, log_err = rec[:, NIN], rec[:, NIN + 1]
    ok = np.isfinite(rec).all(axis=1)
    p = ORDER[method] + 0.0
    t = log_dt - np.clip(log_err, -p * np.log(2.0), 0.0) / p
    X = rec[ok, :NIN].astype(np.float32)
    if not face_feature:
        X[:, NIN - 1] = 0.0
    return X, t[ok].astype(np.float32)


def normalisation(X: np.ndarray, T: np.ndarray) -> np.ndarray:
    """Feature means, standard deviations, target mean and deviation (20).
    A constant input (the zeroed ninth of the 8-input network) gets its value
    as mean and deviation 1, so its standardised value is 0."""
    mu = X.mean(0)
    sd = X.std(0)
    sd[sd < 1e-6] = 1.0
    return np.concatenate([mu, sd, [T.mean(), max(T.std(), 1e-6)]]).astype(np.float32)


def init_params(seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    shapes = [(NIN, 64), (64,), (64, 64), (64,), (64,), (1,)]
    parts = []
    for sh in shapes:
        if len(sh) == 2:
            parts.append(rng.normal(0.0, 1.0 / np.sqrt(sh[0]), sh).ravel())
        else:
            parts.append(np.zeros(sh[0]))
    return np.concatenate(parts).astype(np.float32)


def train(torch, X: np.ndarray, T: np.ndarray, norm: np.ndarray, *, epochs: int = 3,
          batch: int = 8192, lr: float = 2e-3, seed: int = 0, device="cuda",
          log=None) -> tuple[np.ndarray, list]:
    """Adam on the mean-squared error of standardised targets, on the GPU.

    Returns the FP32 parameters and the per-epoch mean losses.
    """
    L = N.load()
    vp = lambda t: C.c_void_p(t.data_ptr())
    Xs = (X - norm[:NIN]) / norm[NIN:2 * NIN]
    Ts = (T - norm[2 * NIN]) / norm[2 * NIN + 1]
    dX = torch.tensor(Xs, dtype=torch.float32, device=device)
    dT = torch.tensor(Ts, dtype=torch.float32, device=device)
    p = torch.tensor(init_params(seed), device=device)
    g = torch.zeros_like(p)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    loss = torch.zeros(1, dtype=torch.float32, device=device)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    st = _stream(None, p)            # the kernels follow the torch work on the same stream
    n = dX.shape[0]
    step, hist = 0, []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).to(device)
        tot, nb = 0.0, 0
        for s in range(0, n - batch + 1, batch):
            idx = perm[s:s + batch]
            xb = dX[idx].contiguous()
            tb = dT[idx].contiguous()
            N.check(L.pt_mlp_loss_grad(vp(p), vp(xb), vp(tb), batch, vp(g), vp(loss), st),
                    "pt_mlp_loss_grad")
            step += 1
            N.check(L.pt_mlp_adam(vp(p), vp(g), vp(m), vp(v), step, lr, 0.9, 0.999, 1e-8, st),
                    "pt_mlp_adam")
            tot += float(loss.item())
            nb += 1
        hist.append(tot / max(nb, 1))
        if log:
            log(f"epoch {ep}: mse {hist[-1]:.4f}")
    return p.cpu().numpy(), hist


def predict(params: np.ndarray, norm: np.ndarray, X: np.ndarray) -> np.ndarray:
    """The network's log trial step on raw feature rows, in float64 on the host
    (for choosing the safety factor; the integrator runs the FP16 tensor-core
    version)."""
    p = np.asarray(params, np.float64)
    o = 0
    parts = []
    for shape in [(NIN, 64), (64,), (64, 64), (64,), (64,), (1,)]:
        n = int(np.prod(shape))
        parts.append(p[o:o + n].reshape(shape))
        o += n
    W1, b1, W2, b2, W3, b3 = parts
    x = (np.asarray(X, np.float64) - norm[:NIN]) / norm[NIN:2 * NIN]
    z1 = x @ W1 + b1
    h1 = z1 / (1.0 + np.exp(-z1))
    z2 = h1 @ W2 + b2
    h2 = z2 / (1.0 + np.exp(-z2))
    return (h2 @ W3 + b3[0]) * norm[2 * NIN + 1] + norm[2 * NIN]


def choose_safety(params: np.ndarray, norm: np.ndarray, X: np.ndarray, T: np.ndarray,
                  grid=None) -> tuple[float, dict]:
    """Safety factor s that maximises the expected progress per attempt on
    held-out records: a proposal exp(pred) s succeeds when it does not exceed
    the attainable step exp(T), and then advances by its length.  The
    network's prediction error makes s < 1 pay; a fixed s either wastes
    attempts (too large) or step length (too small).  Returns (s, the
    progress per attempt at s relative to proposing exp(T) itself)."""
    pred = predict(params, norm, X)
    T = np.asarray(T, np.float64)
    grid = np.linspace(-1.5, 0.3, 73) if grid is None else np.asarray(grid)
    prog = np.array([np.mean(np.exp(pred + ls) * (pred + ls <= T)) for ls in grid])
    k = int(np.argmax(prog))
    return float(np.exp(grid[k])), {"progress_per_attempt_vs_target": float(prog[k] /
                                                                           np.mean(np.exp(T))),
                                    "accepted_fraction": float(np.mean(pred + grid[k] <= T))}


class Model:
    """A trained controller uploaded for the integrator (pt_mlp handle)."""

    def __init__(self, params: np.ndarray, norm: np.ndarray, safety: float = 0.9):
        self._L = N.load()
        self._h = C.c_void_p()
        p = np.ascontiguousarray(params, np.float32)
        nm = np.ascontiguousarray(norm, np.float32)
        N.check(self._L.pt_mlp_create(p.ctypes.data_as(C.c_void_p), nm.ctypes.data_as(C.c_void_p),
                                      float(safety), C.byref(self._h)), "pt_mlp_create")
        self.params, self.norm, self.safety = p, nm, safety

    @property
    def handle(self):
        return self._h

    def infer(self, torch, X: np.ndarray) -> np.ndarray:
        """Tensor-core inference on raw feature rows (log trial dt)."""
        dX = torch.tensor(np.ascontiguousarray(X, np.float32), device="cuda")
        out = torch.empty(dX.shape[0], dtype=torch.float32, device="cuda")
        N.check(self._L.pt_mlp_infer(self._h, C.c_void_p(dX.data_ptr()), dX.shape[0],
                                     C.c_void_p(out.data_ptr()), _stream(None, dX)), "pt_mlp_infer")
        torch.cuda.synchronize()
        return out.cpu().numpy()

    def close(self):
        if self._h:
            self._L.pt_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
