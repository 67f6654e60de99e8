"""2D TTI oracle (CPU): float/double agreement and the 180-degree tilt
symmetry of the scheme (u,w flip sign, P and Q do not)."""
import numpy as np

from tests.util import layered_model, rel_l2

KW = dict(npd=20, nt=400, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=40, zs=10)


def _model(nx=80, nz=70, seed=3):
    v, e, d = layered_model(nx, nz, seed=seed)
    x, z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    theta = (30 + 15 * np.sin(x / 17.0) * np.cos(z / 11.0)).astype(np.float32)
    return v, e, d, theta


def test_tti_float_matches_double(orc):
    v, e, d, th = _model()
    a = orc.tti2d(v, e, d, th, **KW)
    b = orc.tti2d(v, e, d, th, prec=64, **KW)
    assert np.abs(b).max() > 0
    assert rel_l2(a, b) < 1e-4


def test_tti_half_turn_symmetry(orc):
    v, e, d, th = _model(seed=4)
    a = orc.tti2d(v, e, d, th, **KW)
    b = orc.tti2d(v, e, d, (th + 180.0).astype(np.float32), **KW)
    assert rel_l2(b, a) < 1e-4


def test_tti_zero_tilt_sv_taper_changes_only_near_field(orc):
    v, e, d, th = _model(seed=5)
    th[:] = 0.0
    a = orc.tti2d(v, e, d, th, **KW)
    b = orc.tti2d(v, e, d, th, sv=1, **KW)
    assert np.isfinite(b).all() and not np.array_equal(a, b)


RKW = dict(npml=12, nt=260, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, ns=1, fs=20, zs=2,
           mute_tt=30, nangle=65, dangle=1)


def _rtm_model(nx=41, nz=30):
    from tests.util import layered_model
    v, e, d = layered_model(nx, nz, seed=8, vlo=2000, vhi=2600)
    x, z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    th = (20 + 15 * np.sin(x / 7.0) * np.cos(z / 5.0)).astype(np.float32)
    return v, e, d, th


def test_tti_rtm_cdp_decimation(orc):
    """Gathers at dcdp = 2 are the dcdp = 1 gathers of CDPs 0, 2, 4, ...
    (nx = 41: the last CDP is dropped, as nx/dcdp drops it)."""
    v, e, d, th = _rtm_model()
    m1, i1, a1, s1 = orc.rtm2d_tti(v, e, d, th, dcdp=1, **RKW)
    m2, i2, a2, s2 = orc.rtm2d_tti(v, e, d, th, dcdp=2, **RKW)
    assert np.abs(a1).max() > 0
    assert np.array_equal(m1, m2) and np.array_equal(i1, i2) and np.array_equal(s1, s2)
    assert a2.shape == (20, 65, 30)
    assert np.array_equal(a2, a1[0:40:2])


def test_tti_rtm_half_turn(orc):
    """theta + 180 degrees negates cos and sin of the tilt: particle
    velocities change sign, P and Q do not, and neither do the Poynting
    vectors' angles -- with the same observed shots, image and gathers agree
    to rounding.  (The program's mute velocity takes cos(theta) with its
    sign, so the modelled, muted records themselves differ.)"""
    v, e, d, th = _rtm_model()
    m1, _, a1, s1 = orc.rtm2d_tti(v, e, d, th, **RKW)
    m1, _, a1, _ = orc.rtm2d_tti(v, e, d, th, obs=s1, **RKW)
    m2, _, a2, _ = orc.rtm2d_tti(v, e, d, th + 180, obs=s1, **RKW)
    assert np.abs(m1).max() > 0
    assert rel_l2(m2, m1) < 1e-4
    assert rel_l2(a2, a1) < 1e-2
