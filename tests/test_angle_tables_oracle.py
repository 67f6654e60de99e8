"""The oracle's device-table path for the GPU RTM programs' angle gathers
(orc_set_angle_cos, orc_set_angle_thresholds), CPU only: handed the host's
own weights cosf(ia*pi/180) and the bin edges of the host's acosf, it gives
the same gathers as its default path, which calls cosf and acosf itself.
So the only thing the device tables change is which function's values the
oracle uses."""
import ctypes as C

import numpy as np

from oracle import refgpu
from tests.util import layered_model, random_model_3d


def host_tables(da):
    libm = C.CDLL("libm.so.6")
    libm.cosf.restype = C.c_float
    libm.cosf.argtypes = [C.c_float]
    cos = np.array([libm.cosf(float(x)) for x in refgpu.angle_args(128)], np.float32)
    return dict(angle_cos=cos, angle_thr=refgpu.host_bin_thresholds(128, da))


def test_bin_edges_count_like_the_bin_formula():
    """Counting host edges at or above a gives the host formula's bin."""
    rng = np.random.default_rng(3)
    for da in (1, 2, 3):
        thr = refgpu.host_bin_thresholds(128, da)
        assert (np.diff(thr[thr > -2]) < 0).all()
        pts = np.concatenate([rng.uniform(-1, 1, 3000).astype(np.float32), thr[thr > -2],
                              np.nextafter(thr[thr > -2], np.float32(2)), np.float32([-1, 0, 1])])
        for a in pts:
            assert int((thr >= a).sum()) == refgpu.host_bin(float(a), da), (da, a)


def test_rtm2d_gpu_tables_path_equals_host_path(orc):
    v, e, d = layered_model(40, 30, seed=3)
    kw = dict(npml=10, nt=200, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, ns=1, fs=20, ds=0, zs=2,
              nangle=60, dangle=1)
    a = orc.rtm2d_gpu(v, e, d, **kw)
    b = orc.rtm2d_gpu(v, e, d, **host_tables(1), **kw)
    assert np.abs(a[2]).max() > 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_rtm2d_tti_tables_path_equals_host_path(orc):
    v, e, d = layered_model(40, 30, seed=4)
    th = np.full(v.shape, 20.0, np.float32)
    kw = dict(npml=10, nt=200, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, ns=1, fs=20, ds=0, zs=2,
              nangle=60, dangle=2, dcdp=2)
    a = orc.rtm2d_tti(v, e, d, th, **kw)
    b = orc.rtm2d_tti(v, e, d, th, **host_tables(2), **kw)
    assert np.abs(a[2]).max() > 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_rtm3d_tables_path_equals_host_path(orc):
    v, e, d = random_model_3d(14, 12, 14, seed=5)
    kw = dict(npd=6, nt=90, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=30.0, pfac=10.0, fsx=6, fsy=5,
              fsz=2, ns=1, sv=1, mute_tt=10)
    a = orc.rtm3d(v, e, d, adcig=(40, 3, 1), **kw)
    b = orc.rtm3d(v, e, d, adcig=(40, 3, 1), **host_tables(3), **kw)
    assert np.abs(a[3]).max() > 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
