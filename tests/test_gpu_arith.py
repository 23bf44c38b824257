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
