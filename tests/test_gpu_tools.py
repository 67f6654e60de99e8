"""Post-processing tools on the GPU against their pinned CPU restatement
(bit-exact): smooth2float, the smoothed gathers and stack of the MPI RTM
program, the direct-wave mute utility."""
import ctypes as C

import numpy as np
import pytest

from oracle import tools_oracle as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,rx,rz", [((37, 23), 4, 3), ((300, 1), 5, 0), ((2, 501), 0, 9)])
def test_smooth2d(geo, shape, rx, rz):
    v = np.random.default_rng(1).standard_normal(shape).astype(np.float32) * 50 + 3000
    assert np.array_equal(geo.smooth2d(v, rx, rz), T.smooth2d(v, rx, rz))


def test_smooth_long_lines(geo):
    """Lines above 12288 samples take more than 48 KB of shared memory."""
    v = np.random.default_rng(2).standard_normal((3, 20000)).astype(np.float32)
    got = v.copy()
    geo.lib().geo_smooth_lines(C.c_void_p(got.ctypes.data), 20000, 3, 20000, 1, 6, geo.GEO_MEM_HOST, None)
    assert np.array_equal(got, T.smooth1(v, 6))


def test_adcig_smooth_stack(geo):
    g = np.random.default_rng(3).standard_normal((90, 41, 33)).astype(np.float32)
    sg, stk = geo.adcig_smooth_stack(g, 10)
    wg, wstk = T.adcig_smooth_stack(g, 10)
    assert np.array_equal(sg, wg)
    assert np.array_equal(stk, wstk)


def test_adcig_smooth_stack_device(geo):
    import torch
    g = np.random.default_rng(4).standard_normal((90, 12, 20)).astype(np.float32)
    sg, stk = geo.adcig_smooth_stack(torch.from_numpy(g).cuda(), 10)
    wg, wstk = T.adcig_smooth_stack(g, 10)
    assert sg.is_cuda and np.array_equal(sg.cpu().numpy(), wg)
    assert np.array_equal(stk.cpu().numpy(), wstk)


@pytest.mark.parametrize("is_,eps,tt", [(1, 0.0, 190), (3, 0.2, 30)])
def test_mute_direct(geo, is_, eps, tt):
    shot = np.random.default_rng(is_).standard_normal((53, 900)).astype(np.float32)
    kw = dict(dt=np.float32(5e-4), favg=15.0, dx=5.0, dz=5.0, fs=4, ds=9, zs=1, is_=is_, vp=2000.0, epsilon=eps, tt=tt)
    assert np.array_equal(geo.mute_direct(shot, **kw), T.mute_direct(shot, **kw))
