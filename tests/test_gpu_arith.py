"""The correctly rounded arithmetic of the force and solve passes on the GPU.

Those passes compute square roots, reciprocals and quotients from the
hardware approximations refined to the correctly rounded result (one range
check per pair, IEEE operations outside it). The parity claims rest on those
sequences returning the IEEE bits; fs_selftest_arithmetic compares them on
every float bit pattern (reciprocal, square root) and on 2^32 pseudo-random
operand pairs (quotients)."""
import ctypes as C

import pytest

from fluidsph import abi

pytestmark = pytest.mark.gpu


def test_fast_arithmetic_is_correctly_rounded():
    lib = abi.load()
    out = (C.c_ulonglong * 4)()
    abi.check(lib.fs_selftest_arithmetic(0, out))
    names = ["reciprocal (all 2^32 inputs)", "square root (all 2^32 inputs)",
             "quotient (2^32 random pairs)"]
    assert {n: int(v) for n, v in zip(names, out)} == {n: 0 for n in names}
    assert int(out[3]) > 2 ** 30  # the fast path was exercised


def test_selftest_rejects_bad_arguments():
    lib = abi.load()
    out = (C.c_ulonglong * 4)()
    assert lib.fs_selftest_arithmetic(-1, out) == -1  # FS_E_INVALID_ARGUMENT
    assert lib.fs_selftest_arithmetic(0, None) == -1


def test_fp32_rate_measurement(fslib):
    """The measured FP32 roofline denominator is plausible for a GB300: the
    fused rate within the nominal 152 SMs x 128 lanes x 2 FLOP x 2.07 GHz
    (80.5 TFLOP/s) and well above a third of it, and the separate
    multiply-add rate about half of the fused one (one FLOP per
    instruction)."""
    import ctypes as C
    rates = (C.c_double * 2)()
    assert fslib.fs_selftest_fp32_rate(0, rates) == 0
    fma, muladd = rates[0], rates[1]
    print(f"\nFP32 rate: fma {fma:.2f} TFLOP/s, separate mul+add {muladd:.2f} TFLOP/s")
    assert 25.0 < fma < 82.0
    assert 0.4 < muladd / fma < 0.6
