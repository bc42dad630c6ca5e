"""The integer-pipe FP64 division and square root equal the hardware
instructions bit for bit (every operand class, 2^28 pairs per seed)."""
import ctypes

import pytest

from swe_fvm_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_soft_div_sqrt_bit_exact(gpu, seed):
    L = _lib.load()
    bd, bs = ctypes.c_int64(-1), ctypes.c_int64(-1)
    assert L.swe_selftest_fp64(1 << 28, seed, ctypes.byref(bd), ctypes.byref(bs)) == 0
    assert bd.value == 0, f"{bd.value} division mismatches"
    assert bs.value == 0, f"{bs.value} square-root mismatches"
