"""The oracle's 3D TTI restatement (orc_tti3d) on the CPU: its FP32 and FP64
builds agree, and it has the azimuth symmetry of the scheme (azimuth 90 deg
on a medium symmetric under x <-> y is the transpose of azimuth 0)."""
import numpy as np

from tests.util import random_model_3d, rel_l2, smooth_angles

KW = dict(npd=8, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0)


def test_tti3d_oracle_fp32_close_to_fp64(orc):
    v, e, d = random_model_3d(16, 14, 18, seed=5)
    th, ph = smooth_angles(v.shape, seed=1)
    kw = dict(KW, nt=100, fsx=8, fsy=7, fsz=3)
    a = orc.fd3d(v, e, d, theta=th, phi=ph, **kw)
    b = orc.fd3d(v, e, d, theta=th, phi=ph, prec=64, **kw)
    assert np.abs(b).max() > 0
    assert rel_l2(a, b) < 1e-5


def test_tti3d_oracle_azimuth_symmetry(orc):
    n = 16
    v, e, d = random_model_3d(n, n, 18, seed=7)
    sym = lambda x: ((x + x.transpose(1, 0, 2)) / 2).astype(np.float32)
    v, e, d = sym(v), sym(e), sym(d)
    th = sym(smooth_angles(v.shape, seed=3)[0])
    kw = dict(KW, nt=100, fsx=8, fsy=8, fsz=3, rx0=0, drx=1, nrx=n, ry0=0, dry=1, nry=n, prec=64)
    a = orc.fd3d(v, e, d, theta=th, phi=np.zeros_like(th), **kw)
    b = orc.fd3d(v, e, d, theta=th, phi=np.full_like(th, 90.0), **kw)
    assert np.abs(a).max() > 0
    assert rel_l2(b, a.transpose(1, 0, 2)) < 1e-12
