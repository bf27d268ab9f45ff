"""The device code bins and interpolates wavelengths with x / 470 (the width
of the 360-830 nm range), computed with two fused multiply-adds instead of a
division.  The method (Brisebarre, Muller and Raina, IEEE Trans. Computers
53(8), 2004) is correctly rounded for a given divisor only if that divisor
passes its conditions; this test settles it for 470 by checking every float
the device code can meet there (0 and [2^-20, 2048]) against the IEEE
quotient, so the kernels' results equal those of a true division."""
import shutil
import subprocess
from pathlib import Path

import pytest


def test_fma_division_by_range_is_correctly_rounded(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = Path(__file__).with_name("division_by_range.c")
    exe = tmp_path / "division_by_range"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), str(src), "-lm"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
