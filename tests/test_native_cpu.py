"""The C-ABI library on a machine without a GPU: it loads, exports every
symbol the public header declares, carries the same tableau as the oracle,
and rejects bad arguments before touching CUDA."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _header_functions():
    text = (ROOT / "include" / "particles_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_header_symbol(native):
    from particles_gb300 import _native as N
    declared = _header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(native, name), f"{name} missing from the library"
    assert sorted(N.EXPORTS) == declared


def test_abi_version_and_carry_size(native):
    assert native.pt_abi_version() == 1
    assert native.pt_carry_bytes(0) == 0
    assert native.pt_carry_bytes(1000) == 128 * 1000


@pytest.mark.parametrize("name,mid", [("rk5", 1), ("dop853", 2), ("dp853", 2), ("rk8", 2),
                                      ("rk5   ", 1), ("RK5", 0), ("euler", 0), ("", 0)])
def test_method_names(native, name, mid):
    assert native.pt_method_from_name(name.encode()) == mid


@pytest.mark.parametrize("which", [1, 2])
def test_tableau_bitwise_equals_oracle(native, oracle_lib, which):
    n = native.pt_tableau(which, None)
    got = np.zeros(n)
    native.pt_tableau(which, got.ctypes.data_as(C.c_void_p))
    ref = oracle_lib.tableau(which)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


def test_argument_errors_need_no_gpu(native):
    from particles_gb300 import _native as N
    dm = np.array([4, 4, 4], np.int32)
    f = np.zeros(3 * 64)
    p = np.zeros(17)
    st = np.zeros((2, 3, 8))
    cnt = np.zeros((2, 3), np.int64)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    assert native.pt_integrate(7, 2, 3, ptr(dm), ptr(p), ptr(np.zeros(3)), ptr(f), ptr(f),
                               ptr(st), ptr(cnt), None) == N.PT_ERR_ARG
    assert b"method" in native.pt_last_error()
    assert native.pt_integrate(1, -1, 3, ptr(dm), ptr(p), ptr(np.zeros(3)), ptr(f), ptr(f),
                               ptr(st), ptr(cnt), None) == N.PT_ERR_ARG
    assert native.pt_integrate(1, 0, 3, ptr(dm), ptr(p), ptr(np.zeros(3)), ptr(f), ptr(f),
                               ptr(st), ptr(cnt), None) == N.PT_OK          # empty batch
    bad = np.array([0, 4, 4], np.int32)
    h = C.c_void_p()
    assert native.pt_fields_create(ptr(bad), ptr(f), ptr(f), None, 0, C.byref(h)) == N.PT_ERR_ARG
    assert native.pt_fields_create(ptr(dm), ptr(f), ptr(f), None, 9, C.byref(h)) == N.PT_ERR_UNSUPPORTED
    assert native.pt_run_check(None) == N.PT_ERR_ARG
    assert native.pt_fields_destroy(None) == N.PT_OK


def test_options_struct_layout():
    from particles_gb300 import _native as N
    assert C.sizeof(N.PtOptions) == 128
    assert N.PtOptions.max_steps.offset == 16 and N.PtOptions.carry.offset == 64
    assert N.PtOptions.threads_per_block.offset == 112


def test_launch_variant_option_checked_on_host(native):
    """blocks_per_sm must be 0 (tuned or default) or 2..4; checked before any CUDA call."""
    from particles_gb300 import _native as N
    from particles_gb300.params import pack_params
    assert N.PtOptions.blocks_per_sm.offset == 104
    dm = np.array([8, 8, 8], np.int32)
    p = pack_params(qom=1.0, vunit=0.1, tmax=1.0)
    out = np.zeros(8)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    for v, rc in ((0, N.PT_OK), (2, N.PT_OK), (3, N.PT_OK), (4, N.PT_OK), (1, N.PT_ERR_ARG),
                  (5, N.PT_ERR_ARG), (-3, N.PT_ERR_ARG)):
        o = N.PtOptions()
        o.struct_size = C.sizeof(o)
        o.blocks_per_sm = v
        assert native.pt_debug_unpack(1, 4, 2, ptr(dm), 0, 0, ptr(p), C.byref(o), ptr(out)) == rc
    assert native.pt_autotune(1, 4, 2, None, ptr(p), None, None, None, 0, None, None, None) == N.PT_ERR_ARG
    # threads per block: 0 (tuned or 128), 64, 128, 256; read only when the
    # caller's struct_size covers the field (an older, shorter struct leaves it out)
    for t, size, rc in ((0, 0, N.PT_OK), (64, 0, N.PT_OK), (256, 120, N.PT_OK),
                        (96, 120, N.PT_ERR_ARG), (512, 0, N.PT_ERR_ARG), (96, 112, N.PT_OK)):
        o = N.PtOptions()
        o.struct_size = size
        o.threads_per_block = t
        assert native.pt_debug_unpack(1, 4, 2, ptr(dm), 0, 0, ptr(p), C.byref(o), ptr(out)) == rc


def test_ensemble_argument_errors_need_no_gpu(native):
    from particles_gb300 import _native as N
    h = C.c_void_p()
    assert native.pt_ensemble_create(1, 0, None, None, C.byref(h)) == N.PT_ERR_ARG
    arr = (N.PtMember * 9)()
    assert native.pt_ensemble_create(1, 9, C.byref(arr), None, C.byref(h)) == N.PT_ERR_ARG
    o = N.PtOptions()
    o.struct_size = C.sizeof(o)
    o.controller = 1
    assert native.pt_ensemble_create(1, 1, C.byref(arr), C.byref(o), C.byref(h)) == N.PT_ERR_UNSUPPORTED
    assert native.pt_ensemble_create(1, 1, C.byref(arr), None, C.byref(h)) == N.PT_ERR_ARG  # no fields
    assert native.pt_ensemble_run(None, 1.0, None) == N.PT_ERR_ARG
    assert native.pt_ensemble_replay(None, None) == N.PT_ERR_ARG
    assert native.pt_ensemble_destroy(None) == N.PT_OK


def test_interpolation_option_checked_on_host(native):
    from particles_gb300 import _native as N
    from particles_gb300.params import pack_params
    assert N.PtOptions.interpolation.offset == 108 and C.sizeof(N.PtOptions) == 128
    dm = np.array([8, 8, 8], np.int32)
    p = pack_params(qom=1.0, vunit=0.1, tmax=1.0)
    out = np.zeros(8)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    for v, ctl, rc in ((0, 0, N.PT_OK), (1, 0, N.PT_OK), (2, 0, N.PT_ERR_ARG),
                       (1, 1, N.PT_ERR_ARG)):       # controller 1 without a model: ARG first
        o = N.PtOptions()
        o.struct_size = C.sizeof(o)
        o.interpolation = v
        o.controller = ctl
        assert native.pt_debug_unpack(1, 4, 2, ptr(dm), 0, 0, ptr(p), C.byref(o), ptr(out)) == rc


def test_checked_variant_exports_the_same_symbols(native):
    """The bounds-checked variant is built next to the library and exports
    every symbol of the header."""
    import ctypes as C2
    from particles_gb300 import _native as N
    from particles_gb300 import build as B
    lib = C2.CDLL(str(B.build(checked=True)))
    for name in N.EXPORTS:
        assert hasattr(lib, name), name


def test_initial_state_argument_errors_need_no_gpu(native):
    import ctypes as C
    from particles_gb300 import _native as N
    p = np.zeros(8)
    p[3:6] = 1.0
    vp = C.c_void_p
    args = lambda kind, npart, m=2: (kind, npart, m, C.c_uint64(1), 0, p.ctypes.data_as(vp), None, None)
    assert native.pt_initial_state(*args(7, 10)) == N.PT_ERR_ARG        # unknown kind
    assert native.pt_initial_state(*args(N.PT_INIT_SPEED, -1)) == N.PT_ERR_ARG
    assert native.pt_initial_state(*args(N.PT_INIT_SPEED, 10, 0)) == N.PT_ERR_ARG   # m < 1
    assert native.pt_initial_state(*args(N.PT_INIT_SPEED, 0)) == N.PT_OK  # nothing to do
    assert native.pt_initial_state(*args(N.PT_INIT_SPEED, 10)) == N.PT_ERR_ARG      # NULL state
    out = np.zeros(4)
    assert native.pt_moments(0, None, 1, out.ctypes.data_as(vp), None) == N.PT_ERR_ARG


def test_face_controller_checked_on_host(native):
    """PT_CTL_FACE is a controller bit of the non-exact precisions only,
    PT_CTL_NOISE of the FP32-evaluation precisions only; other bits are
    unknown."""
    from particles_gb300 import _native as N
    from particles_gb300.params import pack_params
    dm = np.array([8, 8, 8], np.int32)
    p = pack_params(qom=1.0, vunit=0.1, tmax=1.0)
    out = np.zeros(8)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    for prec, ctl, rc in ((0, N.PT_CTL_FACE, N.PT_ERR_UNSUPPORTED), (1, N.PT_CTL_FACE, N.PT_OK),
                          (2, N.PT_CTL_FACE, N.PT_OK), (3, N.PT_CTL_FACE, N.PT_OK),
                          (2, N.PT_CTL_FACE | N.PT_CTL_LEARNED, N.PT_ERR_ARG),   # no model
                          (0, N.PT_CTL_NOISE, N.PT_ERR_UNSUPPORTED),
                          (1, N.PT_CTL_NOISE, N.PT_ERR_UNSUPPORTED),
                          (2, N.PT_CTL_NOISE, N.PT_OK), (3, N.PT_CTL_NOISE | N.PT_CTL_FACE, N.PT_OK),
                          (2, 8, N.PT_ERR_ARG), (2, -1, N.PT_ERR_ARG)):
        o = N.PtOptions()
        o.struct_size = C.sizeof(o)
        o.precision = prec
        o.controller = ctl
        assert native.pt_debug_unpack(1, 4, 2, ptr(dm), prec, 0, ptr(p), C.byref(o), ptr(out)) == rc, (prec, ctl)


def test_face_params_checked_on_host(native):
    from particles_gb300 import _native as N
    assert native.pt_debug_face_params(3, 0.1, 1e-4) == N.PT_ERR_ARG
    assert native.pt_debug_face_params(1, -0.1, 1e-4) == N.PT_ERR_ARG
    assert native.pt_debug_face_params(1, 1.0, 1e-4) == N.PT_ERR_ARG
    assert native.pt_debug_face_params(2, 0.1, 0.0) == N.PT_ERR_ARG
    assert native.pt_debug_face_params(2, 0.1, 1.0) == N.PT_ERR_ARG
    assert native.pt_debug_face_params(1, 0.1, 3e-5) == N.PT_OK        # the defaults
    assert native.pt_debug_face_params(2, 0.01, 3e-5) == N.PT_OK


def _header_arities():
    """{function: number of parameters} of the header's prototypes."""
    text = (ROOT / "include" / "particles_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(pt_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header(native):
    """Every prototype with declared ctypes argument types has as many of
    them as the header has parameters (a changed C signature must change
    the binding too)."""
    ar = _header_arities()
    assert len(ar) >= 40
    checked = 0
    for name, n in ar.items():
        fn = getattr(native, name)
        if fn.argtypes is not None:
            assert len(fn.argtypes) == n, (name, len(fn.argtypes), n)
            checked += 1
    assert checked >= 30


def test_header_is_plain_c_and_cxx(tmp_path):
    """The C ABI header compiles as C99 (the Fortran/C side) and as C++11,
    without warnings, and a C program can link against the library."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    hdr = ROOT / "include" / "particles_gb300.h"
    for lang, std in (("c", "-std=c99"), ("c++", "-std=c++11")):
        r = subprocess.run([gcc, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", lang,
                            str(hdr)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    from particles_gb300 import _native as N
    src = tmp_path / "use.c"
    src.write_text('#include "particles_gb300.h"\n#include <stdio.h>\n'
                   'int main(void) { printf("%d %d\\n", (int)pt_abi_version(), '
                   '(int)pt_method_from_name("dop853")); return 0; }\n')
    lib = N.lib_path()
    exe = tmp_path / "use"
    r = subprocess.run([gcc, "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                        "-L", str(lib.parent), "-lparticles_gb300", f"-Wl,-rpath,{lib.parent}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["1", "2"], (r.stdout, r.stderr)


def test_record_capacity_matches_the_record_width():
    """The capacity the options announce for a record buffer must be the
    number of whole records that fit after the header: the kernel trusts it
    and writes up to that many records of 11 floats."""
    import torch
    from particles_gb300 import _native as N, learned
    from particles_gb300.integrations import _options
    assert N.REC_FLOATS == learned.REC_FLOATS == learned.NIN + 2 == 11
    for cap in (1, 7, 1000):
        buf = learned.record_buffer(torch, cap, device="cpu")
        o = _options("fp64", records=buf)
        assert o.record_capacity == cap
        assert N.REC_HEADER_FLOATS + o.record_capacity * N.REC_FLOATS <= buf.numel()
