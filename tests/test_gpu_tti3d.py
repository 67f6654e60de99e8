"""3D TTI (tilt + azimuth) on the GPU against the oracle's CPU restatement
(orc_tti3d): records, final fields and RTM images are bit-identical to its
FP32 build; the distance to its FP64 build is stated per test.  No
reference program has a 3D TTI scheme ("parity unpinned" against the
reference); the physics checks are the azimuth symmetry below."""
import numpy as np
import pytest

from tests.util import random_model_3d, rel_l2, smooth_angles

pytestmark = pytest.mark.gpu

KW = dict(npd=8, nt=140, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0)


def test_tti3d_bit_exact_vs_oracle(geo, orc):
    v, e, d = random_model_3d(22, 19, 26, seed=5)
    th, ph = smooth_angles(v.shape, seed=1)
    kw = dict(KW, fsx=11, fsy=9, fsz=3)
    ref = orc.fd3d(v, e, d, theta=th, phi=ph, **kw)
    out = geo.fd3d_shot(v, e, d, theta=th, phi=ph, mode="fast", **kw)
    assert np.abs(ref).max() > 0 and np.isfinite(out).all()
    assert np.array_equal(out, ref), rel_l2(out, ref)
    # against FP64 (measured 4.4e-7 on this case)
    ref64 = orc.fd3d(v, e, d, theta=th, phi=ph, prec=64, **kw)
    assert rel_l2(out, ref64) < 2e-5


def test_tti3d_fields_receiver_grid_and_source_on_device(geo, orc):
    import torch
    v, e, d = random_model_3d(20, 24, 18, seed=6)
    th, ph = smooth_angles(v.shape, seed=2)
    kw = dict(KW, fsx=9, fsy=11, fsz=4, rec_iz=8 + 3, rx0=1, drx=2, nrx=9, ry0=2, dry=3, nry=7)
    ref, rp, rq = orc.fd3d(v, e, d, theta=th, phi=ph, final=True, **kw)
    plan = geo.FD3DPlan(nx=20, ny=24, nz=18, mode="fast", **kw)
    plan.set_model(v, e, d)
    plan.set_tilt(torch.from_numpy(th).cuda(), torch.from_numpy(ph).cuda())  # device angles
    out = plan.run_shot(0)
    P, Q = plan.fields()
    plan.close()
    assert np.array_equal(out, ref)
    assert np.array_equal(P, rp)
    assert np.array_equal(Q, rq)


def test_tti3d_azimuth_symmetry(geo):
    """On a medium symmetric under x <-> y, azimuth 90 deg gives the x <-> y
    transpose of azimuth 0 (the rotated frame's x' and y' swap with the grid
    axes; cos 90 deg in FP32 is 4e-8, not 0)."""
    n = 20
    v, e, d = random_model_3d(n, n, 22, seed=7)
    sym = lambda a: ((a + a.transpose(1, 0, 2)) / 2).astype(np.float32)
    v, e, d = sym(v), sym(e), sym(d)
    th, _ = smooth_angles(v.shape, seed=3)
    th = sym(th)
    kw = dict(KW, fsx=10, fsy=10, fsz=3, rx0=0, drx=1, nrx=n, ry0=0, dry=1, nry=n, mode="fast")
    a = geo.fd3d_shot(v, e, d, theta=th, phi=np.zeros_like(th), **kw)
    b = geo.fd3d_shot(v, e, d, theta=th, phi=np.full_like(th, 90.0), **kw)
    assert np.abs(a).max() > 0
    assert rel_l2(b, a.transpose(1, 0, 2)) < 1e-5


def test_tti3d_needs_fast_form_and_angles(geo):
    v, e, d = random_model_3d(12, 10, 14, seed=9)
    th, ph = smooth_angles(v.shape)
    plan = geo.FD3DPlan(nx=12, ny=10, nz=14, npd=8, nt=10, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0, fsx=6,
                        fsy=5, fsz=2, mode="exact")
    plan.set_model(v, e, d)
    with pytest.raises(geo.GeoError):
        plan.set_tilt(th, ph)
    plan.close()
    bad = th.copy()
    bad[1, 2, 3] = np.nan
    with pytest.raises(geo.GeoError):
        geo.fd3d_shot(v, e, d, theta=bad, phi=ph, npd=8, nt=10, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0,
                      fsx=6, fsy=5, fsz=2, mode="fast")


@pytest.mark.parametrize("method", ["boundary", "snapshot", "checkpoint"])
def test_tti3d_rtm_bit_exact(geo, orc, method):
    v, e, d = random_model_3d(18, 16, 20, seed=12, vlo=2000, vhi=2600)
    th, ph = smooth_angles(v.shape, seed=4)
    kw = dict(npd=8, nt=160, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, fsx=9, fsy=8,
              fsz=1, mute_tt=5)
    snap = 0 if method == "boundary" else 4   # checkpoint recompute images as the snapshot method
    mig_ref, ill_ref, _ = orc.rtm3d(v, e, d, theta=th, phi=ph, snap_every=snap, **kw)
    mig, ill = geo.rtm3d(v, e, d, theta=th, phi=ph, mode="fast", method=method, snap_every=4, ckpt_every=12,
                         laplace=False, illum=True, **kw)
    assert np.abs(mig_ref).max() > 0
    assert np.array_equal(ill, ill_ref)
    assert np.array_equal(mig, mig_ref), rel_l2(mig, mig_ref)
    mig64, _, _ = orc.rtm3d(v, e, d, theta=th, phi=ph, snap_every=snap, prec=64, **kw)
    assert rel_l2(mig, mig64) < 1e-4   # measured 2.6e-6 - 3.4e-6
