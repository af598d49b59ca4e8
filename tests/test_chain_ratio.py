"""The chaining kernel's division-free diagonal-ratio test against the reference's f32
quotient (CPU, compiled with gcc)."""
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_integer_ratio_test_matches_f32_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = tmp_path / "check"
    subprocess.run([cc, "-O2", "-o", str(exe), str(ROOT / "tests" / "chain_ratio_check.c"), "-lm"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
