"""The FP64 kernels' quotient by a known reciprocal (needs a GB300).

Where a divisor is a constant (6, the grid spacings) or shared by several
quotients (the sum of the WENO weights, |grad G|), the FP64 kernels form
a / b as RN(q + r y) with y = RN(1/b), q = RN(a y) and the exact remainder
r = a - b q (Markstein's theorem), which equals IEEE division bit for bit.
The self-test compares the two on 2^30 seeded pairs: the solver's divisors
and random ones, random dividends of either sign, exact multiples of the
divisor and dividends whose quotient lies next to a rounding midpoint.  It
also compares the products by 2, 4, 1/2 and 1/4 formed as exponent shifts
with the FP64 multiply on values over the whole exponent range (subnormals,
zeros, the largest finite values).
The parity tests check the kernels themselves against the oracle.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [12345, 987654321])
def test_div_and_pow2_products_equal_ieee(cuda, lsgb_mod, seed):
    bad = C.c_longlong(-1)
    rc = lsgb_mod.lib().lsgb_debug_f64_div_check(C.c_longlong(1 << 30), C.c_ulonglong(seed), C.byref(bad))
    assert rc == 0
    assert bad.value == 0
