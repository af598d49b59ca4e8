"""The GPU striped SW's rewritten F recurrence and closed-form lazy-F pass against
the library's order of operations, on random tasks (CPU, compiled with gcc)."""
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_rewritten_f_and_lazy_f_match_the_striped_loop(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = tmp_path / "check"
    subprocess.run([cc, "-O2", "-o", str(exe), str(ROOT / "tests" / "ssw_reformulation_check.c")], check=True)
    r = subprocess.run([str(exe), "3000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
