"""The FP64 helpers the fused kernels use instead of IEEE operations, checked
on the GPU against the IEEE operations (gb300_check_fp64_helpers):

* halving and doubling on the integer pipes: identical to x*0.5 and x*2 for
  every bit pattern (zeros, subnormals, overflow, infinities, NaNs);
* the power-of-two test that selects the exact-spacing fast path, the
  product by a power of two as an exponent add, and the spacing factors
  1/p, x/(2p), 1/(p*p) of powers of two from their exponent fields: exact;
* quotients: one Newton step on the MUFU seed with one residual correction
  (d_div) and the one-step Newton reciprocal with a corrected quotient (qdiv) both
  return the IEEE quotient except in vanishingly rare near-ties, and then
  differ by one unit in the last place.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

N = 1 << 24


def test_fp64_helpers_match_ieee():
    import flow_gb300 as fg
    L = fg.lib()
    counts = (ctypes.c_longlong * 7)()
    ulp = (ctypes.c_longlong * 2)()
    seed_err = ctypes.c_double()
    assert L.gb300_check_fp64_helpers(N, 20261203, counts, ulp, ctypes.byref(seed_err)) == 0
    c = list(counts)
    print("mismatches", c, "max ulp", list(ulp), "seed rel err", seed_err.value)
    assert c[0] == 0 and c[1] == 0 and c[2] == 0 and c[5] == 0 and c[6] == 0, c
    # Near-ties: at most 1e-6 of the quotients, never more than 1 ulp away.
    assert c[3] <= N * 1e-6 and ulp[0] <= 1, (c, list(ulp))
    assert c[4] <= N * 1e-6 and ulp[1] <= 1, (c, list(ulp))
    # One Newton step and one correction need a seed better than 2^-14
    # (error to the fourth power below 2^-56); measured ~2^-20.
    assert seed_err.value < 2.0 ** -14, seed_err.value
