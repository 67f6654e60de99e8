"""3D boundary-saving RTM on the GPU against the oracle (bit-exact)."""
import numpy as np
import pytest

from oracle.refgpu import cuda_angle_tables
from tests.util import random_model_3d, rel_l2

pytestmark = pytest.mark.gpu

KW = dict(npd=8, nt=150, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0,
          fsx=6, fsy=8, fsz=2, dsx=7, ns=2, mute_tt=20)


@pytest.mark.parametrize("mode,sv", [(0, 0), (1, 0), (1, 1)])
def test_rtm3d_bit_exact(geo, orc, mode, sv):
    v, e, d = random_model_3d(20, 17, 23, seed=11)
    mig_o, ill_o, _ = orc.rtm3d(v, e, d, mode=mode, sv=sv, **KW)
    lap_o = orc.laplace3d_adj(mig_o)
    mig, lap, ill = geo.rtm3d(v, e, d, mode=mode, sv=sv, laplace=True, illum=True, **KW)
    assert np.abs(mig_o).max() > 0 and np.abs(ill_o).max() > 0
    assert np.array_equal(ill, ill_o), rel_l2(ill, ill_o)
    assert np.array_equal(mig, mig_o), rel_l2(mig, mig_o)
    assert np.array_equal(lap, lap_o), rel_l2(lap, lap_o)


@pytest.mark.parametrize("mode,sv,ck", [(0, 0, 12), (1, 1, 20), (1, 0, 0)])
def test_rtm3d_checkpoint_equals_snapshot(geo, orc, mode, sv, ck):
    """Checkpoint recompute (full state every ck steps, ck not dividing nt;
    0 = automatic) images exactly what the stored-snapshot method does, and
    both equal the oracle's snapshot RTM."""
    v, e, d = random_model_3d(20, 17, 23, seed=15)
    mig_o, ill_o, _ = orc.rtm3d(v, e, d, mode=mode, sv=sv, snap_every=4, **KW)
    rk = dict(KW, mode=mode, sv=sv, snap_every=4, laplace=False, illum=True)
    mig_s, ill_s = geo.rtm3d(v, e, d, method="snapshot", **rk)
    mig_c, ill_c = geo.rtm3d(v, e, d, method="checkpoint", ckpt_every=ck, **rk)
    assert np.abs(mig_o).max() > 0
    assert np.array_equal(mig_s, mig_o)
    assert np.array_equal(ill_s, ill_o)
    assert np.array_equal(mig_c, mig_s)
    assert np.array_equal(ill_c, ill_s)
    with pytest.raises(geo.GeoError):
        geo.rtm3d(v, e, d, method="checkpoint", ckpt_every=6, **rk)   # not a multiple of snap_every


def test_rtm3d_device_buffers(geo, orc):
    import torch
    v, e, d = random_model_3d(18, 16, 20, seed=12)
    kw = dict(KW, ns=1)
    mig_o, _, _ = orc.rtm3d(v, e, d, mode=1, **kw)
    tv, te, td = (torch.from_numpy(a).cuda() for a in (v, e, d))
    mig = geo.rtm3d(tv, te, td, mode="fast", laplace=False, **kw)
    assert mig.is_cuda
    assert np.array_equal(mig.cpu().numpy(), mig_o)


def test_rtm3d_fast_close_to_exact(geo):
    v, e, d = random_model_3d(20, 18, 22, seed=13)
    a = geo.rtm3d(v, e, d, mode="exact", laplace=False, **KW)
    b = geo.rtm3d(v, e, d, mode="fast", laplace=False, **KW)
    assert rel_l2(b, a) < 1e-4


@pytest.mark.parametrize("mode,adcig", [(0, (65, 1, 1)), (1, (65, 1, 1)), (1, (40, 2, 2)), (0, (7, 3, 3))])
def test_rtm3d_adcig_bit_exact(geo, orc, mode, adcig):
    """Poynting angle gathers (Poynting_Adcigs + adcigs_illum) bit-exact,
    together with the image and the illumination of the same run."""
    v, e, d = random_model_3d(20, 17, 23, seed=14)
    mig_o, ill_o, _, ag_o = orc.rtm3d(v, e, d, mode=mode, adcig=adcig, **cuda_angle_tables(adcig[1]), **KW)
    mig, ill, ag = geo.rtm3d(v, e, d, mode=mode, laplace=False, illum=True, adcig=adcig, **KW)
    na, _, dcdp = adcig
    assert ag.shape == (17 // dcdp, 20 // dcdp, na, 23)
    filled = np.count_nonzero(np.abs(ag_o).sum(axis=(0, 1, 3)))
    assert filled >= min(na, 5), filled          # several angle bins receive energy
    assert np.array_equal(ill, ill_o)
    assert np.array_equal(mig, mig_o)
    assert np.array_equal(ag, ag_o), rel_l2(ag, ag_o)


def test_rtm3d_adcig_needs_boundary_method(geo):
    from geophysics_gb300 import GeoError
    v, e, d = random_model_3d(16, 16, 16, seed=15)
    with pytest.raises(GeoError):
        geo.rtm3d(v, e, d, method="snapshot", snap_every=2, adcig=(65, 1, 1), **dict(KW, ns=1, nt=40))


@pytest.mark.parametrize("method", ["boundary", "snapshot", "checkpoint"])
def test_rtm3d_receiver_grid(geo, orc, method):
    """A decimated surface grid (every 2nd node from x 1, y 0) records and
    takes the record back instead of every node; image and illumination
    equal the oracle's run with the same grid, on VTI and (checkpoint) TTI."""
    from tests.util import smooth_angles
    v, e, d = random_model_3d(20, 17, 23, seed=13)
    grid = (1, 2, 9, 0, 2, 9)
    kw = dict(KW, receivers=grid)
    snap = 0 if method == "boundary" else 4
    mig_o, ill_o, rec_o = orc.rtm3d(v, e, d, mode=1, snap_every=snap, **kw)
    mig, ill = geo.rtm3d(v, e, d, mode="fast", method=method, snap_every=4, laplace=False, illum=True, **kw)
    assert rec_o.shape == (9, 9, KW["nt"]) and np.abs(mig_o).max() > 0
    assert np.array_equal(ill, ill_o), rel_l2(ill, ill_o)
    assert np.array_equal(mig, mig_o), rel_l2(mig, mig_o)
    full = geo.rtm3d(v, e, d, mode="fast", method=method, snap_every=4, laplace=False, **KW)
    assert not np.array_equal(full, mig)
    if method == "checkpoint":
        th, ph = smooth_angles(v.shape, seed=3)
        mig_o, _, _ = orc.rtm3d(v, e, d, snap_every=4, theta=th, phi=ph, **kw)
        mig = geo.rtm3d(v, e, d, mode="fast", method=method, snap_every=4, laplace=False, theta=th, phi=ph, **kw)
        assert np.array_equal(mig, mig_o), rel_l2(mig, mig_o)
