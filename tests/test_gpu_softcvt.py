"""The integer-pipe float <-> double conversions of the MPI program's double
chains (softcvt.cuh) give the hardware conversions' bits: the widening over
every binary32 pattern, the narrowing (round to nearest even) over 2^28
binary64 values from underflow to overflow, exact ties and binary32
images.  The batch RTM's exact mode stays bit-identical to the oracle
through them (tests/test_gpu_rtm2d.py)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [12345, 2 ** 61 + 7])
def test_integer_pipe_conversions_match_hardware(geo, seed):
    f2d, d2f = C.c_longlong(-1), C.c_longlong(-1)
    st = geo.lib().geo_selftest_conversions(1 << 28, seed, C.byref(f2d), C.byref(d2f), None)
    assert st == 0
    assert f2d.value == 0, f2d.value
    assert d2f.value == 0, d2f.value
