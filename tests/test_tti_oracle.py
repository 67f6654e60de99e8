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
