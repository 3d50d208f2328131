"""Host checks of the FFT radix plans and the twiddle-table layout (no GPU):
tests/cpp/plan_check.cu, built with nvcc as host code, checks for every
supported length that the radices multiply to the length, that the inverse
plan is the forward one reversed, that the two leading radices sit at the ends
(the V order), that the twiddle blocks tile the table (shared by the two plans
when the V reads the same both ways), that the butterfly-to-thread map of every
pass is a bijection for every chunk width up to the bound, and that the row
pass's default chunk stays within it."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_plans_and_twiddle_layout(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "plan_check"
    subprocess.run([nvcc, "-std=c++17", f"-I{ROOT / 'cdixx_gb300' / 'csrc'}", f"-I{ROOT / 'include'}",
                    "-gencode", "arch=compute_103a,code=sm_103a", str(ROOT / "tests" / "cpp" / "plan_check.cu"),
                    "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0 and "plans ok" in r.stdout
    assert "N=2048 plan 16 8 16 twiddles 2032 (shared)" in r.stdout
