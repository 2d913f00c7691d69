"""CPU oracle of the particle hot path -- TEST INFRASTRUCTURE ONLY.

Python access to ``oracle/_build/liboracle.so`` (built from ``oracle.cpp`` by
``oracle/Makefile``).  The oracle restates the reference integrators
(sources/integrations.F90:57-200, :224-505, :524-589), the Lorentz force
(sources/accelerations.F90:59-96) and the trilinear gather
(sources/interpolations.F90:104-226).  Only ``tests/``, the smoke check and
the CPU-baseline leg of ``bench.py`` import this module, as the checker.

Parity status: unpinned by the reference -- it has no tests or golden
vectors and cannot be compiled here (Fortran; no Fortran compiler).  The
oracle is pinned by analytic known-answer tests (tests/test_oracle_kat.py).

Array layouts (numpy, C order, equal to the Fortran column-major arrays):
  fields uu, bb, jj : shape (3, dm3, dm2, dm1)   == uu(dm1,dm2,dm3,3)
  state             : shape (np, m, 8)           == state(8,m,np)
  cnt               : shape (np, 3)              == counter(3,np)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

ST_DONE, ST_RUNNING, ST_ESCAPED = 0, 1, 2
ST_STEP_LIMIT, ST_DT_UNDERFLOW, ST_NONFINITE = -2, -3, -4


class Carry(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("errold", C.c_double),
                ("si", C.c_double * 6), ("n", C.c_int32), ("flags", C.c_int32)]


class Ext(C.Structure):
    _fields_ = [("eta", C.c_double), ("jj", C.c_void_p), ("open_x", C.c_int32),
                ("faithful", C.c_int32), ("max_steps", C.c_int64), ("t_stop", C.c_double),
                ("carry", C.c_void_p), ("status", C.c_void_p), ("near", C.c_int32),
                ("pad", C.c_int32), ("open_x_margin", C.c_double)]


def build(force: bool = False) -> Path:
    """Build the oracle with its Makefile (g++, -ffp-contract=off, OpenMP)."""
    src = [HERE / "oracle.cpp", HERE / "oracle.h", HERE / "Makefile",
           HERE.parent / "particles_gb300" / "csrc" / "pt_detmath.h"]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in src):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        vp, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        L.or_integrate.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32]
        L.or_integrate.restype = C.c_int
        L.or_interpolate_lin.argtypes = [vp] * 8
        L.or_interpolate_near.argtypes = [vp] * 8
        L.or_acceleration.argtypes = [d, d, vp, vp, vp, vp, vp, vp, vp]
        L.or_dti_guess.argtypes = [i32, vp, vp, vp, vp, vp]
        L.or_dti_guess.restype = d
        L.or_det_pow.argtypes = [d, d]
        L.or_det_pow.restype = d
        L.or_tableau.argtypes = [i32, vp]
        L.or_tableau.restype = i32
        L.or_count_ops.argtypes = [i32, i32, i32, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def integrate(method, params, time, uu, bb, state, cnt=None, *, eta=0.0, jj=None,
              open_x=False, faithful=False, max_steps=0, t_stop=0.0, carry=None,
              status=None, nthreads=0, near=False, open_x_margin=0.0):
    """Run the oracle over all particles in place.

    ``state`` (np, m, 8) float64 is updated in place (row 0 holds the initial
    x, u).  Returns (state, cnt, status).  ``carry`` is an array of ``Carry``
    (``make_carry(np)``) for resumable windows.
    """
    method = {"rk5": 1, "dop853": 2, "dp853": 2, "rk8": 2}.get(method, method)
    assert state.dtype == np.float64 and state.flags.c_contiguous and state.ndim == 3
    npart, m, _ = state.shape
    if cnt is None:
        cnt = np.zeros((npart, 3), np.int64)
    if status is None:
        status = np.zeros(npart, np.int32)
    dm = np.array(uu.shape[:0:-1], np.int32)
    uu, bb = _f64(uu), _f64(bb)
    jj = _f64(jj) if jj is not None else None
    ext = Ext(eta, _p(jj) if jj is not None else None, int(open_x), int(faithful),
              int(max_steps), float(t_stop),
              C.cast(carry, C.c_void_p) if carry is not None else None, _p(status),
              int(bool(near)), 0, float(open_x_margin))
    rc = lib().or_integrate(int(method), npart, m, _p(dm), _p(_f64(params)), _p(_f64(time)),
                            _p(uu), _p(bb), _p(state), _p(cnt), C.byref(ext), int(nthreads))
    if rc != 0:
        raise ValueError(f"or_integrate returned {rc}")
    return state, cnt, status


def make_carry(npart):
    return (Carry * npart)()


def interpolate_lin(uu, bb, pos, xl=(0, 0, 0), xs=(1, 1, 1)):
    dm = np.array(uu.shape[:0:-1], np.int32)
    u, b = np.zeros(3), np.zeros(3)
    lib().or_interpolate_lin(_p(dm), _p(_f64(xl)), _p(_f64(xs)), _p(_f64(uu)), _p(_f64(bb)),
                             _p(_f64(pos)), _p(u), _p(b))
    return u, b


def interpolate_near(uu, bb, pos, xl=(0, 0, 0), xs=(1, 1, 1)):
    dm = np.array(uu.shape[:0:-1], np.int32)
    u, b = np.zeros(3), np.zeros(3)
    lib().or_interpolate_near(_p(dm), _p(_f64(xl)), _p(_f64(xs)), _p(_f64(uu)), _p(_f64(bb)),
                              _p(_f64(pos)), _p(u), _p(b))
    return u, b


def acceleration(qom, vun, uu, bb, vec, xl=(0, 0, 0), xs=(1, 1, 1)):
    dm = np.array(uu.shape[:0:-1], np.int32)
    acc = np.zeros(6)
    lib().or_acceleration(float(qom), float(vun), _p(dm), _p(_f64(xl)), _p(_f64(xs)),
                          _p(_f64(uu)), _p(_f64(bb)), _p(_f64(vec)), _p(acc))
    return acc


def dti_guess(iord, params, uu, bb, si):
    dm = np.array(uu.shape[:0:-1], np.int32)
    return lib().or_dti_guess(int(iord), _p(dm), _p(_f64(params)), _p(_f64(uu)), _p(_f64(bb)),
                              _p(_f64(si)))


def det_pow(x, y):
    return lib().or_det_pow(float(x), float(y))


def tableau(which):
    n = lib().or_tableau(int(which), None)
    out = np.zeros(n)
    lib().or_tableau(int(which), _p(out))
    return out


def count_ops(method, what, with_eta=False):
    """(add, mul, div, sqrt, pow) counts; see oracle.h for ``what``."""
    out = np.zeros(5, np.uint64)
    lib().or_count_ops(int(method), int(what), int(with_eta), _p(out))
    return tuple(int(v) for v in out)
