"""CPU check of the register DFTs and two-pass FFT shapes used by the fast kernels: the device
code in spfft_gb300/csrc/dft.cuh is also host-callable, so tests/dft_selftest.cu compiles it as host code and
compared with a long-double direct DFT for every supported size and both signs."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "spfft_gb300" / "csrc"


@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="nvcc not available")
def test_register_dfts_and_two_pass_shapes(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "dft_selftest"
    subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
                    "-I", str(CSRC), "-x", "cu", str(ROOT / "tests" / "dft_selftest.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
    assert int(out.stdout.split()[1]) >= 100


@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="nvcc not available")
def test_double_float_conversions(tmp_path):
    """Integer-only double <-> double-float conversions used by the FP64 kernels: exact splits,
    round trips, correctly rounded recombination, zeros, infinities and NaN."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "dd_convert_selftest"
    subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
                    "-I", str(CSRC), "-x", "cu", str(ROOT / "tests" / "dd_convert_selftest.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
