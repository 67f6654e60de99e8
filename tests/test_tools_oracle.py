"""The post-processing tools' CPU restatement (oracle/tools_oracle.py)
pinned against the reference's own code compiled into oracle/_ref:
smooth2float of the MPI RTM program and the direct-wave mute utility."""
import numpy as np
import pytest

from oracle import tools_oracle as T


@pytest.fixture(scope="module")
def ref(orc):
    if not orc.ref_available():
        pytest.skip("reference build not present")
    return orc


@pytest.mark.parametrize("rx,rz", [(4, 3), (10, 0), (0, 7), (1, 1)])
def test_smooth2d_pinned(ref, rx, rz):
    v = np.random.default_rng(rx * 10 + rz).standard_normal((37, 23)).astype(np.float32) * 100 + 2000
    assert np.array_equal(T.smooth2d(v, rx, rz), ref.ref_smooth2float(v, rx, rz))


def test_adcig_smooth_stack_pinned(ref):
    """The program's loop (:416-437): per CDP, smooth2float(90, 10, nz, 0)
    of the (angle, depth) panel, then the stack over angles."""
    g = np.random.default_rng(2).standard_normal((90, 6, 17)).astype(np.float32)
    sg, stk = T.adcig_smooth_stack(g, 10)
    want = np.empty_like(g)
    want_stk = np.zeros((6, 17), np.float32)
    for ix in range(6):
        panel = ref.ref_smooth2float(g[:, ix, :], 10, 0)
        want[:, ix, :] = panel
        for ia in range(90):
            want_stk[ix] = (want_stk[ix] + panel[ia]).astype(np.float32)
    assert np.array_equal(sg, want)
    assert np.array_equal(stk, want_stk)


@pytest.mark.parametrize("is_,eps,tt", [(1, 0.0, 190), (3, 0.2, 30), (7, 0.1, 0)])
def test_mute_direct_pinned(ref, is_, eps, tt):
    shot = np.random.default_rng(is_).standard_normal((53, 900)).astype(np.float32)
    kw = dict(dt=np.float32(5e-4), favg=15.0, dx=5.0, dz=5.0, fs=4, ds=9, zs=1, is_=is_, vp=2000.0, epsilon=eps, tt=tt)
    got = T.mute_direct(shot, **kw)
    assert np.count_nonzero(got == 0) > 0
    assert np.array_equal(got, ref.ref_mute_direct(shot, **kw))


def test_smooth_model3d_pinned(ref, geo):
    """The library's 3D model smoother (host code, in-place sweep) against
    the reference utility run on its own 70^3 case (20 passes from z = 20)."""
    import ctypes as C
    v = (2000 + 500 * np.random.default_rng(0).standard_normal((70, 70, 70))).astype(np.float32)
    want = ref.ref_smooth3d(v)
    got = v.copy()
    assert geo.lib().geo_smooth_model3d(70, 70, 70, 20, 20, C.c_void_p(got.ctypes.data),
                                             geo.GEO_MEM_HOST, None) == 0
    assert np.array_equal(got, want)


def test_smooth_model2d_host(geo):
    """The 2D in-place smoother (host code) against its restatement; rows
    above z0 are untouched, and a constant model stays within an ulp."""
    import ctypes as C
    v = (2500 + 300 * np.random.default_rng(1).standard_normal((30, 25))).astype(np.float32)
    got = v.copy()
    assert geo.lib().geo_smooth_model2d(30, 25, 6, 5, C.c_void_p(got.ctypes.data), geo.GEO_MEM_HOST,
                                             None) == 0
    assert np.array_equal(got, T.smooth_model2d(v, 6, 5))
    assert np.array_equal(got[:, :6], v[:, :6])
    c = np.full((12, 10), 3000.0, np.float32)
    geo.lib().geo_smooth_model2d(12, 10, 2, 3, C.c_void_p(c.ctypes.data), geo.GEO_MEM_HOST, None)
    assert np.allclose(c, 3000.0, rtol=1e-6, atol=0)
