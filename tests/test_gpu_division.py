"""The bit-exact FP64 line solvers divide by a pivot through its stored
reciprocal: one product and two fused multiply-adds that round to the IEEE
quotient (Markstein's correction).  Against the hardware division on 2^26
seeded operand pairs over the normal range (random significands, quotients
at or next to representable values, small integers, zero dividends of either
sign) not one bit pattern may differ; the parity tests of every line solver
against the oracle (which divides) check the same thing in place."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261204])
def test_division_by_stored_reciprocal_is_the_ieee_quotient(gblib, seed):
    from codesthesis_dir_gb300 import lib
    bad = C.c_longlong(-1)
    assert gblib.gb_check_division(1 << 26, seed, C.byref(bad)) == lib.GB_OK, lib.last_error()
    assert bad.value == 0
