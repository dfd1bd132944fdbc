"""The device Stockham FFT (vs_fft.cuh) compiled for the host and run as a
sequential emulation of one CTA, against a long-double naive DFT (CPU only)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_fft_code_matches_naive_dft(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = os.path.join(ROOT, "tests", "native", "fft_host_emulation.cpp")
    exe = str(tmp_path / "fft_emu")
    inc = "/usr/local/cuda/include"
    r = subprocess.run([gxx, "-std=c++17", "-O2", f"-I{inc}", "-x", "c++", src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "ALL OK" in r.stdout
