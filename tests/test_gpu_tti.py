"""2D TTI on the GPU against the oracle (bit-exact)."""
import numpy as np
import pytest

from tests.util import layered_model, rel_l2

pytestmark = pytest.mark.gpu

KW = dict(npd=20, nt=300, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=40, zs=10)


def _model(nx=90, nz=67, seed=3):
    v, e, d = layered_model(nx, nz, seed=seed)
    x, z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    theta = (25 + 20 * np.sin(x / 13.0) * np.cos(z / 9.0)).astype(np.float32)
    return v, e, d, theta


@pytest.mark.parametrize("sv", [0, 1])
def test_tti2d_bit_exact(geo, orc, sv):
    v, e, d, th = _model()
    ref, rs = orc.tti2d(v, e, d, th, sv=sv, snap_every=100, **KW)
    out, snaps = geo.tti2d_shot(v, e, d, th, sv=sv, snap_every=100, **KW)
    assert np.abs(ref).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)
    assert snaps.shape == rs.shape == (2, 130, 107)
    assert np.array_equal(snaps, rs)


def test_tti2d_device_buffers_and_second_shot(geo, orc):
    import torch
    v, e, d, th = _model(seed=4)
    kw = dict(KW, ds=7.0, is_=2, rec_iz=22)
    ref = orc.tti2d(v, e, d, th, **kw)
    t = [torch.from_numpy(a).cuda() for a in (v, e, d, th)]
    out = geo.tti2d_shot(*t, **kw)
    assert out.is_cuda
    assert np.array_equal(out.cpu().numpy(), ref)


def test_tti2d_rejects_bad_input(geo):
    v, e, d, th = _model()
    th[3, 4] = np.nan
    with pytest.raises(geo.GeoError):
        geo.tti2d_shot(v, e, d, th, **KW)
