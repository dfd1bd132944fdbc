"""The FP64 <-> double-float conversions of the double-float passes
(vs_df.cuh: df_from_double, df_store), compiled for the host, give the same
bits as the FP64 conversions they replace (CPU only); and the multiply-high
plane split of the strided passes (StridedArgs::plane) is an exact division
over its whole range."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_double_float_split_matches_fp64_conversions(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = os.path.join(ROOT, "tests", "native", "df_split_host.cpp")
    exe = str(tmp_path / "df_split")
    inc = "/usr/local/cuda/include"
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-I{inc}", "-x", "c++", src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "ALL OK" in r.stdout


def _plane_split(y, na):
    """StridedArgs::plane: q = umulhi(y, ceil(2^32 / na)) for na >= 2, else y."""
    mul = np.uint64(((1 << 32) + na - 1) // na) if na >= 2 else None
    y = y.astype(np.uint64)
    q = (y * mul) >> np.uint64(32) if mul is not None else y
    return q, y - q * np.uint64(na)


@pytest.mark.parametrize("na", [1, 2, 3, 7, 26, 78, 91, 105, 255, 256, 257, 1000, 4095, 4097, 32767,
                                65521, 65535, 65536])
def test_plane_split_is_exact_division(na):
    y = np.arange(65536, dtype=np.uint64)
    q, r = _plane_split(y, na)
    assert np.array_equal(q, y // np.uint64(na))
    assert np.array_equal(r, y % np.uint64(na))
