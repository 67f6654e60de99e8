"""3D forward modelling on the GPU against the oracle."""
import numpy as np
import pytest

from tests.util import random_model_3d, rel_l2

pytestmark = pytest.mark.gpu

KW = dict(npd=8, nt=140, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0,
          fsx=11, fsy=9, fsz=3)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("sv", [0, 1])
def test_fd3d_bit_exact(geo, orc, mode, sv):
    v, e, d = random_model_3d(22, 19, 26, seed=5)
    ref = orc.fd3d(v, e, d, mode=mode, sv=sv, **KW)
    out = geo.fd3d_shot(v, e, d, mode=mode, sv=sv, **KW)
    assert np.abs(ref).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)


def test_fd3d_fields_and_receiver_grid(geo, orc):
    v, e, d = random_model_3d(20, 24, 18, seed=6)
    kw = dict(KW, rec_iz=8 + 3, rx0=1, drx=2, nrx=9, ry0=2, dry=3, nry=7)
    ref, rp, rq = orc.fd3d(v, e, d, mode=1, final=True, **kw)
    plan = geo.FD3DPlan(nx=20, ny=24, nz=18, mode="fast", **kw)
    plan.set_model(v, e, d)
    out = plan.run_shot(0)
    P, Q = plan.fields()
    plan.close()
    assert np.array_equal(out, ref)
    assert np.array_equal(P, rp)
    assert np.array_equal(Q, rq)


def test_fd3d_fast_close_to_exact(geo):
    v, e, d = random_model_3d(24, 24, 24, seed=8)
    a = geo.fd3d_shot(v, e, d, mode="exact", **KW)
    b = geo.fd3d_shot(v, e, d, mode="fast", **KW)
    assert rel_l2(b, a) < 1e-5


def test_fd3d_dropin(geo, orc, tmp_path):
    v, e, d = random_model_3d(16, 14, 15, seed=3)
    # the reference file layout is iz + nz*(ix + nx*iy)
    for name, a in (("v", v), ("e", e), ("d", d)):
        a.tofile(tmp_path / (name + ".bin"))
    geo.GPU_vti3dfd(16, 14, 15, 10, 10, 10, 8, 0, str(tmp_path / "v.bin"), str(tmp_path / "e.bin"),
                    str(tmp_path / "d.bin"), 25, 1, 8, 0, 7, 0, 2, 0, str(tmp_path / "shot.bin"),
                    str(tmp_path / "snap.bin"), 120, 1000)
    shot = np.fromfile(tmp_path / "shot.bin", np.float32).reshape(14, 16, 120)
    ref = orc.fd3d(v, e, d, mode=0, npd=8, nt=120, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0,
                   pfac=10.0, fsx=8, fsy=7, fsz=2).copy()
    import ctypes as C
    orc.lib().orc_mute3d(16, 14, 120, np.float32(1e-3), 25.0, 10.0, 10.0, 10.0, 8, 7, 0, 0, 2, 0,
                         np.float32(v[0, 0, 0]), np.float32(e[0, 0, 0]), 100, ref.ctypes.data_as(C.POINTER(C.c_float)))
    assert np.array_equal(shot, ref)


@pytest.mark.parametrize("chunks", ["1", "3"])
@pytest.mark.parametrize("shape", [(21, 19, 27), (34, 17, 45)])
def test_fd3d_chunks_and_ragged_extents(geo, orc, monkeypatch, chunks, shape):
    """y split into chunks (warm-up planes recomputed per chunk) and z
    extents whose padded length is not a multiple of 4 (padded z stride)."""
    monkeypatch.setenv("GEO_FD3D_CHUNKS", chunks)
    ny, nx, nz = shape
    v, e, d = random_model_3d(nx, ny, nz, seed=11)
    kw = dict(KW, npd=7, fsx=nx // 2, fsy=ny // 2, fsz=4)
    for mode in (0, 1):
        ref = orc.fd3d(v, e, d, mode=mode, **kw)
        out = geo.fd3d_shot(v, e, d, mode=mode, **kw)
        assert np.array_equal(out, ref), (mode, rel_l2(out, ref))


def test_fd3d_model_checked_on_device(geo):
    """The model is checked and padded on the GPU; a bad value is reported
    with the first offending index, as the host check reports it."""
    from tests.util import random_model_3d
    v, e, d = random_model_3d(12, 10, 14, seed=9)
    kw = dict(npd=8, nt=10, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0, fsx=6, fsy=5, fsz=2)
    for arr, idx, val, what in ((0, 57, np.nan, "velocity[57]"), (0, 3, -1.0, "velocity[3]"),
                                (2, 90, -0.7, "1+2*delta[90]"), (1, 11, np.inf, "eps/del[11]")):
        m = [v.copy(), e.copy(), d.copy()]
        m[arr].reshape(-1)[idx] = val
        m[arr].reshape(-1)[idx + 200] = val           # a later bad point is not the one reported
        with pytest.raises(geo.GeoError) as ei:
            geo.fd3d_shot(*m, **kw)
        assert ei.value.status == 4 and what in str(ei.value), str(ei.value)
