"""The exact build's integer-pipe product (particles_gb300/csrc/pt_smul.h)
checked on the host against the FPU's binary64 multiply: 2 x 10^6 operand
pairs in each of six classes (any bit pattern, moderate exponents, short
significands that make ties, all-ones and near-power-of-two significands,
products near overflow and near underflow).  Every product the integer path
accepts must carry the FPU's bits, and it may decline only zero, subnormal,
infinite or NaN operands and products outside the normal range."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_integer_product_matches_the_fpu(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "smul_check"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-I", str(ROOT / "particles_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "smul_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "2000000", "3"], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    lines = [l.split() for l in r.stdout.splitlines() if l.startswith("class")]
    assert len(lines) == 6
    for f in lines:
        pairs, fast = int(f[3]), int(f[5])
        assert int(f[7]) == 0 and int(f[9]) == 0
        assert fast >= pairs // 2          # the integer path covers most of every class
