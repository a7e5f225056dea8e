"""The stage update adds a rate of exactly +0 (components without a flux) by
an integer-pipe form of x + 0.0; the library's self-test compares it with
the FP64 add bit for bit on boundary values and 16 M pseudo-random bit
patterns."""
import ctypes as C

import pytest

from mesoflow_gb300 import abi

pytestmark = pytest.mark.gpu


def test_exact_integer_forms_match_fp64():
    lib = abi.load()
    bad = C.c_uint(12345)
    abi.check("mfg_selftest_exact_ops", lib.mfg_selftest_exact_ops(1 << 24, C.byref(bad)))
    assert bad.value == 0


def test_selftest_rejects_bad_arguments():
    lib = abi.load()
    bad = C.c_uint()
    assert lib.mfg_selftest_exact_ops(0, C.byref(bad)) == abi.ERR_ARG
    assert lib.mfg_selftest_exact_ops(16, None) == abi.ERR_ARG
