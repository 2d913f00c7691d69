"""Python face of the integrator, shaped like the reference's interface.

``integrate_rk5`` / ``integrate_dp853`` take the arguments of the Fortran
subroutines (sources/integrations.F90:57 and :224) -- m, dm, params, time, uu,
bb, state, cnt -- but for all particles at once, and ``integrate`` is the
driver's dispatch on the method string (particles.F90:337-356).  Every call
goes through the C ABI of ``libparticles_gb300.so``; nothing runs on the CPU.

Layouts (numpy C order == Fortran column-major):
  uu, bb, jj : (3, dm3, dm2, dm1)      state : (np, m, 8)      cnt : (np, 3)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .params import method_id


# gather: "linear" = interpolate_lin (interpolations.F90:104-226, the reference's
# choice in accelerations.F90:82); "near" = interpolate_near (:55-83)
INTERPOLATIONS = {"linear": 0, "near": 1}


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _stream(stream, tensor=None):
    """The CUDA stream a launch goes to: `stream` when given (a handle), else
    torch's current stream on the tensor's device, so that the launch is
    ordered after the torch work that produced the tensor (and torch's
    allocator reuses its blocks only after the launch)."""
    if stream:
        return C.c_void_p(int(stream))
    if tensor is not None and getattr(tensor, "is_cuda", False):
        import torch
        h = torch.cuda.current_stream(tensor.device).cuda_stream
        return C.c_void_p(h) if h else None
    return None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _options(precision, *, eta=0.0, jj=None, open_x=False, max_steps=0, t_stop=0.0,
             status=None, carry=None, time_budget_s=0.0, model=None, records=None,
             order=None, blocks_per_sm=0, interpolation=0, face_steps=False, noise_floor=False,
             threads_per_block=0, open_x_margin=0.0):
    o = N.PtOptions()
    o.struct_size = C.sizeof(N.PtOptions)
    o.precision = N.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.open_x = int(bool(open_x))
    o.open_x_margin = float(open_x_margin)
    o.controller = ((N.PT_CTL_LEARNED if model is not None else 0)
                    | (N.PT_CTL_FACE if face_steps else 0)
                    | (N.PT_CTL_NOISE if noise_floor else 0))
    o.model = model.handle if model is not None else None
    if records is not None:                       # device tensor (float32) with header
        o.records = C.c_void_p(records.data_ptr())
        o.record_capacity = (records.numel() - N.REC_HEADER_FLOATS) // N.REC_FLOATS
    if order is not None:                         # device int32 tensor
        o.order = C.c_void_p(order.data_ptr())
    o.max_steps = int(max_steps)
    o.eta = float(eta)
    o.jj = _ptr(jj)
    o.t_stop = float(t_stop)
    o.time_budget_s = float(time_budget_s)
    o.status = _ptr(status)
    o.carry = _ptr(carry)
    o.blocks_per_sm = int(blocks_per_sm)
    o.threads_per_block = int(threads_per_block)
    o.interpolation = INTERPOLATIONS[interpolation] if isinstance(interpolation, str) else int(interpolation)
    return o


def carry_buffer(npart: int) -> np.ndarray:
    """Zero-filled (fresh) host controller memory for resumable windows."""
    return np.zeros(int(N.load().pt_carry_bytes(npart)), np.uint8)


def integrate(method, params, time, uu, bb, state, cnt=None, *, precision="fp64", eta=0.0,
              jj=None, open_x=False, open_x_margin=0.0, max_steps=0, t_stop=0.0, carry=None,
              status=None, time_budget_s=0.0, check=True, interpolation="linear",
              face_steps=False, noise_floor=False):
    """Integrate every particle of ``state`` in place on the GPU.

    Returns (state, cnt, status).  With ``check`` a negative return code
    raises ``PtError``; otherwise the code is in ``status``/``pt_last_error``.
    """
    L = N.load()
    mid = method_id(method)
    assert state.dtype == np.float64 and state.flags.c_contiguous and state.ndim == 3
    npart, m, eight = state.shape
    assert eight == 8
    if cnt is None:
        cnt = np.zeros((npart, 3), np.int64)
    if status is None:
        status = np.zeros(npart, np.int32)
    uu, bb = _f64(uu), _f64(bb)
    jj = _f64(jj) if jj is not None else None
    dm = np.array(uu.shape[:0:-1], np.int32)
    opt = _options(precision, eta=eta, jj=jj, open_x=open_x, open_x_margin=open_x_margin,
                   max_steps=max_steps, t_stop=t_stop, status=status, carry=carry,
                   time_budget_s=time_budget_s, interpolation=interpolation,
                   face_steps=face_steps, noise_floor=noise_floor)
    rc = L.pt_integrate(mid, npart, m, _ptr(dm), _ptr(_f64(params)), _ptr(_f64(time)),
                        _ptr(uu), _ptr(bb), _ptr(state), _ptr(cnt), C.byref(opt))
    if check:
        N.check(rc, "pt_integrate")
    return state, cnt, status


def integrate_rk5(m, dm, params, time, uu, bb, state, cnt, **kw):
    """Batched integrations.F90:57 (`integrate_rk5(m, dm, params, time, uu, bb, state, cnt)`)."""
    assert state.shape[1] == m and tuple(uu.shape[:0:-1]) == tuple(dm)
    return integrate("rk5", params, time, uu, bb, state, cnt, **kw)


def integrate_dp853(m, dm, params, time, uu, bb, state, cnt, **kw):
    """Batched integrations.F90:224 (`integrate_dp853(...)`)."""
    assert state.shape[1] == m and tuple(uu.shape[:0:-1]) == tuple(dm)
    return integrate("dop853", params, time, uu, bb, state, cnt, **kw)


class Fields:
    """Fields uploaded once and converted to the kernel layout on the device.

    ``uu``, ``bb`` (and ``jj``) are numpy host arrays or CUDA torch tensors in
    the reference layout.
    """

    def __init__(self, uu, bb, jj=None, precision="fp64", stream=None):
        self._L = N.load()
        self.precision = precision
        self._h = C.c_void_p()
        prec = N.PRECISIONS[precision]
        dm = np.array(tuple(uu.shape[:0:-1]), np.int32)
        self.dm = tuple(int(x) for x in dm)
        self.has_j = jj is not None
        if isinstance(uu, np.ndarray):
            uu, bb = _f64(uu), _f64(bb)
            jj = _f64(jj) if jj is not None else None
            rc = self._L.pt_fields_create(_ptr(dm), _ptr(uu), _ptr(bb), _ptr(jj), prec,
                                          C.byref(self._h))
        else:
            rc = self._L.pt_fields_create_device(
                _ptr(dm), C.c_void_p(uu.data_ptr()), C.c_void_p(bb.data_ptr()),
                C.c_void_p(jj.data_ptr()) if jj is not None else None, prec,
                _stream(stream, uu), C.byref(self._h))
        N.check(rc, "pt_fields_create")

    @property
    def handle(self):
        return self._h

    @property
    def nbytes(self) -> int:
        return int(self._L.pt_fields_bytes(self._h))

    def close(self):
        if self._h:
            self._L.pt_fields_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, method, params, time, state, cnt=None, *, eta=0.0, open_x=False,
                  open_x_margin=0.0, max_steps=0, t_stop=0.0, carry=None, status=None,
                  time_budget_s=0.0, check=True, interpolation="linear", face_steps=False,
                  noise_floor=False):
        """Host-buffer run on these fields (pt_integrate_fields)."""
        npart, m, _ = state.shape
        if cnt is None:
            cnt = np.zeros((npart, 3), np.int64)
        if status is None:
            status = np.zeros(npart, np.int32)
        opt = _options(self.precision, eta=eta, open_x=open_x, open_x_margin=open_x_margin,
                       max_steps=max_steps, t_stop=t_stop, status=status, carry=carry,
                       time_budget_s=time_budget_s, interpolation=interpolation,
                       face_steps=face_steps, noise_floor=noise_floor)
        rc = self._L.pt_integrate_fields(method_id(method), npart, m, self._h,
                                         _ptr(_f64(params)), _ptr(_f64(time)), _ptr(state),
                                         _ptr(cnt), C.byref(opt))
        if check:
            N.check(rc, "pt_integrate_fields")
        return state, cnt, status

    def run_device(self, method, params, d_time, d_state, d_cnt, d_status=None, d_carry=None,
                   *, eta=0.0, open_x=False, open_x_margin=0.0, max_steps=0, t_stop=0.0,
                   time_budget_s=0.0, stream=0, model=None, records=None, order=None,
                   blocks_per_sm=0,
                   interpolation="linear", face_steps=False, noise_floor=False,
                   threads_per_block=0):
        """Launch on device tensors (torch); returns without synchronising.

        model: a learned.Model for the learned controller; records: a device
        record buffer (learned.record_buffer); order: device int32 queue order;
        blocks_per_sm: register cap (0 = tuned or default, else 2, 3, 4 resident
        128-thread blocks); threads_per_block: 0 (tuned or 128), 64, 128 or 256;
        face_steps: trial steps end just past the next cell face (PT_CTL_FACE,
        not with precision "fp64").
        noise_floor: the error norm treats differences below the FP32
        evaluation's rounding floor as zero (PT_CTL_NOISE, "fp32" / "bf16").
        """
        npart, m, _ = d_state.shape
        opt = _options(self.precision, eta=eta, open_x=open_x, open_x_margin=open_x_margin,
                       max_steps=max_steps, t_stop=t_stop, time_budget_s=time_budget_s,
                       model=model, records=records, order=order, blocks_per_sm=blocks_per_sm,
                       threads_per_block=threads_per_block,
                       interpolation=interpolation, face_steps=face_steps,
                       noise_floor=noise_floor)
        rc = self._L.pt_run_device(
            method_id(method), npart, m, self._h, _ptr(_f64(params)),
            C.c_void_p(d_time.data_ptr()), C.c_void_p(d_state.data_ptr()),
            C.c_void_p(d_cnt.data_ptr()),
            C.c_void_p(d_status.data_ptr()) if d_status is not None else None,
            C.c_void_p(d_carry.data_ptr()) if d_carry is not None else None,
            C.byref(opt), _stream(stream, d_state))
        N.check(rc, "pt_run_device")

    def autotune(self, method, params, d_time, d_state, *, eta=0.0, open_x=False, max_steps=0,
                 t_stop=0.0, sample=0, stream=0, model=None, records=None,
                 interpolation="linear", face_steps=False, noise_floor=False):
        """Time the launch variants of the kernel run_device would use with
        these arguments (pt_autotune) and make the fastest its default.

        t_stop > 0 times a real window up to t_stop (else max_steps attempts);
        sample: particles in the trial (0 default, -1 all).
        Returns ((blocks_per_sm, threads_per_block), {(blocks_per_sm,
        threads_per_block): trial ms}) over the variants tried."""
        npart, m, _ = d_state.shape
        opt = _options(self.precision, eta=eta, open_x=open_x, max_steps=max_steps,
                       t_stop=t_stop, model=model, records=records, interpolation=interpolation,
                       face_steps=face_steps, noise_floor=noise_floor)
        chosen = (C.c_int32 * 2)()
        ms = np.zeros(9, np.float64)
        rc = self._L.pt_autotune(method_id(method), npart, m, self._h, _ptr(_f64(params)),
                                 C.c_void_p(d_time.data_ptr()), C.c_void_p(d_state.data_ptr()),
                                 C.byref(opt), int(sample), _stream(stream, d_state),
                                 chosen, _ptr(ms))
        N.check(rc, "pt_autotune")
        tried = {(2 + i // 3, (64, 128, 256)[i % 3]): float(ms[i]) for i in range(9) if ms[i] >= 0}
        return (int(chosen[0]), int(chosen[1])), tried

    def run_check(self) -> int:
        return int(self._L.pt_run_check(self._h))


class Ensemble:
    """Several runs (members) in one persistent launch per window
    (pt_ensemble_*): each member is a snapshot (a Fields handle), its
    params(1:17) and its particles on the device.  Between windows the
    finished and escaped particles leave the work lists, which are ordered
    longest first; a sequence of windows can be captured as a CUDA graph.

    members: list of dicts with keys fields, params, time, state, cnt,
    status, carry (torch CUDA tensors for the last five) and optionally
    open_x, open_x_margin, eta, max_steps.
    """

    def __init__(self, method, members, *, precision="fp64", blocks_per_sm=0,
                 time_budget_s=0.0, interpolation="linear", face_steps=False,
                 noise_floor=False):
        self._L = N.load()
        self._h = C.c_void_p()
        self.n = len(members)
        self._keep = []
        self._t0 = members[0]["state"]             # device of the launches' default stream
        arr = (N.PtMember * self.n)()
        for k, mb in enumerate(members):
            prm = _f64(mb["params"])
            self._keep.append(prm)
            st = mb["state"]
            a = arr[k]
            a.fields = mb["fields"].handle
            a.params = prm.ctypes.data_as(C.c_void_p)
            a.np, a.m = int(st.shape[0]), int(st.shape[1])
            a.open_x = int(bool(mb.get("open_x", False)))
            a.open_x_margin = float(mb.get("open_x_margin", 0.0))
            a.eta = float(mb.get("eta", 0.0))
            a.max_steps = int(mb.get("max_steps", 0))
            for key in ("time", "state", "cnt", "status", "carry"):
                setattr(a, key, C.c_void_p(mb[key].data_ptr()))
        opt = _options(precision, time_budget_s=time_budget_s, blocks_per_sm=blocks_per_sm,
                       interpolation=interpolation, face_steps=face_steps,
                       noise_floor=noise_floor)
        N.check(self._L.pt_ensemble_create(method_id(method), self.n, C.byref(arr), C.byref(opt),
                                           C.byref(self._h)), "pt_ensemble_create")

    def run(self, t_stop, stream=0):
        """One window up to t_stop (0 = to each member's tmax); no synchronisation."""
        N.check(self._L.pt_ensemble_run(self._h, float(t_stop), _stream(stream, self._t0)),
                "pt_ensemble_run")

    def capture(self, windows, dt_window, stream=0):
        N.check(self._L.pt_ensemble_capture(self._h, int(windows), float(dt_window),
                                            _stream(stream, self._t0)),
                "pt_ensemble_capture")

    def replay(self, stream=0):
        N.check(self._L.pt_ensemble_replay(self._h, _stream(stream, self._t0)),
                "pt_ensemble_replay")

    def counts(self):
        """(live, escaped) particle counts per member, after synchronising."""
        live = np.zeros(self.n, np.int64)
        esc = np.zeros(self.n, np.int64)
        N.check(self._L.pt_ensemble_counts(self._h, _ptr(live), _ptr(esc)), "pt_ensemble_counts")
        return live, esc

    def escaped(self, k):
        """Indices of member k's escaped particles, after synchronising."""
        n = C.c_int64()
        N.check(self._L.pt_ensemble_escaped(self._h, int(k), None, 0, C.byref(n)), "pt_ensemble_escaped")
        out = np.zeros(n.value, np.int32)
        N.check(self._L.pt_ensemble_escaped(self._h, int(k), _ptr(out), out.size, C.byref(n)),
                "pt_ensemble_escaped")
        return out

    def check(self) -> int:
        return int(self._L.pt_ensemble_check(self._h))

    def close(self):
        if self._h:
            self._L.pt_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OutputStream:
    """Streams finished output rows to the host while later windows run.

    After each window, call `window_done(t_stop, compute_stream)`: the rows
    whose time is <= t_stop are final for every particle still running, so
    they are copied (pt_copy_rows, one strided copy) on a side stream that
    waits for the window's kernel through an event and overlaps the next
    window.  `rows()` synchronises and returns the host array (np, m, 8)
    with every row streamed so far.
    """

    def __init__(self, torch, d_state, time):
        self._L = N.load()
        self.torch = torch
        self.d_state = d_state
        self.time = np.asarray(time, np.float64)
        npart, m, _ = d_state.shape
        self.host = torch.zeros((npart, m, 8), dtype=torch.float64).pin_memory()
        self.side = torch.cuda.Stream(device=d_state.device)
        self.done = 0
        self._bufs = []

    def window_done(self, t_stop, compute_stream=None):
        torch = self.torch
        n = int(np.searchsorted(self.time, t_stop, side="right")) if t_stop > 0 else self.time.size
        if n <= self.done:
            return 0
        ev = torch.cuda.Event()
        ev.record(compute_stream or torch.cuda.current_stream())
        self.side.wait_event(ev)
        npart, m, _ = self.d_state.shape
        buf = torch.empty((npart, n - self.done, 8), dtype=torch.float64).pin_memory()
        N.check(self._L.pt_copy_rows(C.c_void_p(self.d_state.data_ptr()), npart, m, self.done, n,
                                     C.c_void_p(buf.data_ptr()), C.c_void_p(self.side.cuda_stream)),
                "pt_copy_rows")
        self._bufs.append((self.done, n, buf))
        rows = n - self.done
        self.done = n
        return rows

    def rows(self):
        self.side.synchronize()
        for a, b, buf in self._bufs:
            self.host[:, a:b] = buf
        self._bufs = []
        return self.host.numpy()
