"""Build recipe of the native library ``libparticles_gb300.so`` (sm_103a only).

Plain ``nvcc`` invocations, one per translation unit, run in parallel, then
one link.  The FP64 kernel source is compiled twice: ``exact`` with
``--fmad=false`` (bit-identical to the CPU oracle) and ``fma`` with FMA
contraction; each integrator source is split by method (``PT_PART``) so the
launch variants of RK5 and DOP853 compile in parallel.  Host code is compiled with ``-ffp-contract=off`` so that host
arithmetic (parameter unpacking) rounds the same on x86-64 and aarch64.
Outputs go to ``particles_gb300/_build/`` (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libparticles_gb300.so"
# the bounds-checked variant (-DPT_CHECKED): every gather index is tested
# against the field store and counted when out of range (PT_ERR_BOUNDS)
OUT_CHECKED = OUT / "checked"
LIB_CHECKED = OUT_CHECKED / "libparticles_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-I", str(PKG.parent / "include"),
]

# (output object, source, extra flags)
UNITS = [
    ("pt_api.o", "pt_api.cu", ["--fmad=false"]),
    ("pt_fields.o", "pt_fields.cu", ["--fmad=false"]),
    ("pt_hostio.o", "pt_hostio.cu", ["--fmad=false"]),
    ("pt_ensemble.o", "pt_ensemble.cu", ["--fmad=false"]),
    ("pt_fp64_exact1.o", "pt_fp64.cu", ["--fmad=false", "-DPT_SFX=exact", "-DPT_EXACT", "-DPT_PART=1"]),
    ("pt_fp64_exact2.o", "pt_fp64.cu", ["--fmad=false", "-DPT_SFX=exact", "-DPT_EXACT", "-DPT_PART=2"]),
    ("pt_fp64_fma1.o", "pt_fp64.cu", ["--fmad=true", "-DPT_SFX=fma", "-DPT_PART=1"]),
    ("pt_fp64_fma2.o", "pt_fp64.cu", ["--fmad=true", "-DPT_SFX=fma", "-DPT_PART=2"]),
    ("pt_mixed1.o", "pt_mixed.cu", ["--fmad=true", "-DPT_PART=1"]),
    ("pt_mixed2.o", "pt_mixed.cu", ["--fmad=true", "-DPT_PART=2"]),
    ("pt_probe.o", "pt_probe.cu", ["--fmad=true"]),
    ("pt_noalloc.o", "pt_noalloc.cu", ["--fmad=false"]),
    ("pt_initial.o", "pt_initial.cu", ["--fmad=false"]),
    ("pt_mlp_train.o", "pt_mlp_train.cu", ["--fmad=true"]),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build particles_gb300")
    return exe


def _sources_newer_than(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "particles_gb300.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps if d.is_file())


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile and link the library (or its bounds-checked variant) if any
    source is newer; return its path."""
    lib, out = (LIB_CHECKED, OUT_CHECKED) if checked else (LIB, OUT)
    if not force and not _sources_newer_than(lib):
        return lib
    out.mkdir(parents=True, exist_ok=True)
    exe = nvcc()
    ptx_v = ["-Xptxas", "-v"] if verbose else []
    defs = ["-DPT_CHECKED"] if checked else []

    def compile_unit(u):
        obj, src, extra = u
        cmd = [exe, *ARCH, *COMMON, *extra, *defs, *ptx_v, "-c", str(CSRC / src), "-o",
               str(out / obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return obj, cmd, r

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS))
    log = []
    for obj, cmd, r in results:
        log.append(f"$ {' '.join(cmd)}\n{r.stdout}{r.stderr}")
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {obj}:\n{r.stdout}\n{r.stderr}")
    tmp = lib.with_suffix(".so.tmp")
    link = [exe, *ARCH, "-shared", "-o", str(tmp), *[str(out / u[0]) for u in UNITS]]
    r = subprocess.run(link, capture_output=True, text=True)
    log.append(f"$ {' '.join(link)}\n{r.stdout}{r.stderr}")
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    (out / "build.log").write_text("\n".join(log))
    return lib


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv,
              checked="--checked" in sys.argv)
    print(p)
