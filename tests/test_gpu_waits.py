"""Failure detection without a GPU fault: a pipeline wait that can never
complete gives up after its limit, the kernel reports it in an error word,
and the context keeps working."""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives(geo):
    gave_up = C.c_int(0)
    t0 = time.perf_counter()
    st = geo.lib().geo_selftest_bounded_wait(200, C.byref(gave_up), None)
    dt = time.perf_counter() - t0
    assert st == 0 and gave_up.value == 1
    assert 0.19 < dt < 5.0, dt
    # the same process keeps computing correctly afterwards
    img = np.random.default_rng(0).standard_normal((40, 30)).astype(np.float32)
    a = geo.laplace2d(img)
    b = geo.laplace2d(img)
    assert np.array_equal(a, b) and np.abs(a).max() > 0
