"""2D forward modelling on the GPU against the oracle (bit-exact: the
kernels keep the reference's operation order with contraction off)."""
import numpy as np
import pytest

from tests.util import layered_model, rel_l2

pytestmark = pytest.mark.gpu

KW = dict(npd=20, nt=300, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=30.0, zs=5.0)


@pytest.mark.parametrize("variant,sv", [("cpu", 0), ("cpu", 1), ("gpu", 0), ("gpu", 1), ("mpi", 1)])
def test_fd2d_bit_exact(geo, orc, variant, sv):
    v, e, d = layered_model(61, 51, seed=1)
    var = {"cpu": orc.V_CPU, "gpu": orc.V_GPU, "mpi": orc.V_MPI}[variant]
    ref = orc.fd2d(v, e, d, variant=var, sv=sv, **KW)
    out = geo.fd2d_shot(v, e, d, variant=variant, sv=sv, **KW)
    assert np.abs(ref).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)


def test_fd2d_snapshots_and_receiver_row(geo, orc):
    v, e, d = layered_model(48, 40, seed=2)
    kw = dict(KW, fs=20.0, zs=3.0, nt=160)
    ref, rs = orc.fd2d(v, e, d, rec_iz=20 + 4, snap_every=40, **kw)
    out, os_ = geo.fd2d_shot(v, e, d, rec_iz=20 + 4, snap_every=40, **kw)
    assert np.array_equal(out, ref)
    assert np.array_equal(os_, rs)


def test_fd2d_device_buffers(geo, orc):
    import torch
    v, e, d = layered_model(61, 51, seed=1)
    ref = orc.fd2d(v, e, d, **KW)
    tv, te, td = (torch.from_numpy(a).cuda() for a in (v, e, d))
    out = geo.fd2d_shot(tv, te, td, **KW)
    assert out.is_cuda
    assert np.array_equal(out.cpu().numpy(), ref)


def test_fd2d_ragged_sizes(geo, orc):
    # extents that are not multiples of the 32x8 tile
    v, e, d = layered_model(37, 29, seed=9)
    kw = dict(KW, npd=7, fs=18.0, zs=4.0, nt=90)
    for variant, var in (("cpu", orc.V_CPU), ("gpu", orc.V_GPU)):
        assert np.array_equal(geo.fd2d_shot(v, e, d, variant=variant, **kw), orc.fd2d(v, e, d, variant=var, **kw))


@pytest.mark.parametrize("variant", ["cpu", "gpu"])
def test_fd2d_source_at_tile_seams(geo, orc, variant):
    """The CPU and GPU forms keep each block's tile of the fields in shared
    memory and exchange halos; sources on and next to the seams between
    tiles (x every 8 or more cells, z every 32 or more) reach every copy of
    the source cell the step reads."""
    v, e, d = layered_model(70, 60, seed=5)
    var = {"cpu": orc.V_CPU, "gpu": orc.V_GPU}[variant]
    for fs, zs in ((13.0, 13.0), (14.0, 14.0), (21.0, 12.0), (29.0, 45.0), (30.0, 44.0)):
        kw = dict(KW, fs=fs, zs=zs, nt=120)
        ref = orc.fd2d(v, e, d, variant=var, **kw)
        out = geo.fd2d_shot(v, e, d, variant=variant, **kw)
        assert np.array_equal(out, ref), (fs, zs, rel_l2(out, ref))


@pytest.mark.parametrize("tile", ["32x8", "64x12", "128x24", "256x8"])
def test_fd2d_tile_shapes(geo, orc, monkeypatch, tile):
    """Tile shapes other than the automatic one (GEO_FD2D_TILE): many small
    tiles (up to 4 per SM), wide and narrow ones, ragged edges, 400 steps of
    halo exchange and grid barriers, both forms bit-exact."""
    monkeypatch.setenv("GEO_FD2D_TILE", tile)
    v, e, d = layered_model(157, 131, seed=12)
    kw = dict(KW, fs=77.0, zs=9.0, nt=400)
    for variant, var in (("cpu", orc.V_CPU), ("gpu", orc.V_GPU)):
        ref = orc.fd2d(v, e, d, variant=var, **kw)
        out = geo.fd2d_shot(v, e, d, variant=variant, **kw)
        assert np.abs(ref).max() > 0
        assert np.array_equal(out, ref), (tile, variant, rel_l2(out, ref))


def test_fd2d_gpu_form_snapshots_while_source_on(geo, orc):
    """Snapshots every 3 steps end a launch every 3 steps while the GPU
    form's point source is still on: each launch reloads the tiles and adds
    the source to the reloaded cell."""
    v, e, d = layered_model(70, 60, seed=8)
    kw = dict(KW, fs=29.0, zs=13.0, nt=61)
    ref, rs = orc.fd2d(v, e, d, variant=orc.V_GPU, snap_every=3, **kw)
    out, os_ = geo.fd2d_shot(v, e, d, variant="gpu", snap_every=3, **kw)
    assert np.array_equal(out, ref), rel_l2(out, ref)
    assert np.array_equal(os_, rs)


def test_fd2d_grid_beyond_resident_tiles(geo, orc):
    """A grid too large for every tile to stay in shared memory at once
    takes the launch that reads the fields through L2: same results."""
    v, e, d = layered_model(1250, 820, seed=6)
    kw = dict(KW, fs=600.0, zs=5.0, nt=30)
    for variant, var in (("cpu", orc.V_CPU), ("gpu", orc.V_GPU)):
        assert np.array_equal(geo.fd2d_shot(v, e, d, variant=variant, **kw), orc.fd2d(v, e, d, variant=var, **kw))


def test_dropin_files_match_oracle(geo, orc, tmp_path):
    v, e, d = layered_model(50, 45, seed=4)
    for name, arr in (("v", v), ("e", e), ("d", d)):
        arr.tofile(tmp_path / (name + ".bin"))
    args = dict(nx=50, nz=45, dx=10, dz=10, npd=20, SV=0, FNv=str(tmp_path / "v.bin"), FNe=str(tmp_path / "e.bin"),
                FNd=str(tmp_path / "d.bin"), favg=20, ns=2, fs=20, ds=5, zs=5, nt=160, dt=1000)
    geo.CPU_vti2dfd(FNshot=str(tmp_path / "shot.bin"), FNsnap=str(tmp_path / "snap.bin"), **args)
    shots = np.fromfile(tmp_path / "shot.bin", np.float32).reshape(2, 50, 160)
    snaps = np.fromfile(tmp_path / "snap.bin", np.float32).reshape(-1, 90, 85)
    for is_ in (1, 2):
        ref = orc.fd2d(v, e, d, npd=20, nt=160, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0,
                       fs=20.0, ds=5.0, zs=5.0, is_=is_)
        assert np.array_equal(shots[is_ - 1], ref)
    _, rs = orc.fd2d(v, e, d, npd=20, nt=160, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=20.0,
                     zs=5.0, snap_every=50)
    assert np.array_equal(snaps, rs)
    # GPU-form drop-in: point source + direct-wave mute (tt=100)
    geo.GPU_vti2dfd(FNshot=str(tmp_path / "gshot.bin"), FNsnap=str(tmp_path / "gsnap.bin"), **args)
    g = np.fromfile(tmp_path / "gshot.bin", np.float32).reshape(2, 50, 160)
    ref = orc.fd2d(v, e, d, npd=20, nt=160, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0,
                   fs=20.0, zs=5.0, variant=orc.V_GPU)
    ref = ref.copy()
    vp1 = v[0, 0] * np.sqrt(np.float32(1) + np.float32(2) * e[0, 0])
    orc.lib().orc_mute2d(0, 50, 160, np.float32(1e-3), 20.0, 10.0, 10.0, 20, 5, 5, 1, np.float32(vp1), 100,
                         ref.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_float)))
    assert np.array_equal(g[0], ref)


def test_fd2d_bad_arguments(geo):
    v, e, d = layered_model(30, 30, seed=1)
    with pytest.raises(geo.GeoError):
        geo.fd2d_shot(v, e, d, **dict(KW, npd=3))
    bad = v.copy()
    bad[3, 3] = np.nan
    with pytest.raises(geo.GeoError) as ei:
        geo.fd2d_shot(bad, e, d, **KW)
    assert ei.value.status == 4
