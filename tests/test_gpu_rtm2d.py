"""Batched 2D RTM (MPI-program semantics) against the oracle: per-shot
images, the shot-ordered stack and the Laplacian are bit-exact."""
import numpy as np
import pytest

from oracle.refgpu import cuda_angle_tables
from tests.util import layered_model

pytestmark = pytest.mark.gpu


def model(nx=101, nz=50):
    rng = np.random.default_rng(3)
    v, e, d = layered_model(nx, nz, seed=3, vlo=2000, vhi=2600)
    v += rng.uniform(0, 40, v.shape).astype(np.float32)
    return v, e, d


@pytest.mark.parametrize("tile_x", [0, 4, 8])
def test_rtm2d_batch_bit_exact(geo, orc, tile_x):
    v, e, d = model()
    xs, ws = [35, 55, 48], [41, 53, 31]
    kw = dict(npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0)
    acc = np.zeros(v.shape, np.float32)
    refs = []
    for k, (x, w) in enumerate(zip(xs, ws)):
        mo, off, _ = orc.rtm2d_mpi_shot(v, e, d, fs_sxd=x, ds_sxd=0, zs_sxd=1, is_=k + 1, nxs=w, **kw)
        refs.append(mo)
        orc.stack2d(acc, mo, off)
    lap = orc.laplace2d_adj(acc)
    img, per = geo.rtm2d_batch(v, e, d, zs=1, shot_x=xs, shot_nxs=ws, per_shot=True, tile_x=tile_x, **kw)
    for a, b in zip(per, refs):
        assert np.array_equal(a, b)
    assert np.array_equal(img, lap)
    raw = geo.rtm2d_batch(v, e, d, zs=1, shot_x=xs, shot_nxs=ws, laplace=False, **kw)
    assert np.array_equal(raw, acc)


def test_rtm2d_batch_fast_mode_within_rounding(geo, orc):
    """The fast mode forms the program's double-precision chains in FP32.
    Both modes are FP32 roundings of one computation whose image is a small
    residual of large correlations: the exact mode itself is 1.3e-3 to
    5.3e-3 (rel-L2) from the oracle's FP64 build here.  Bound: the fast
    image is no further from FP64 than 1.5x the exact one, and within 1e-2
    of it."""
    from tests.util import rel_l2
    v, e, d = model()
    xs, ws = [35, 55, 48], [41, 53, 31]
    kw = dict(npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0)
    run = dict(kw, zs=1, shot_x=xs, shot_nxs=ws, per_shot=True)
    img, per = geo.rtm2d_batch(v, e, d, **run)
    fimg, fper = geo.rtm2d_batch(v, e, d, mode="fast", **run)
    assert np.isfinite(fimg).all() and np.abs(img).max() > 0
    for k, (x, w) in enumerate(zip(xs, ws)):
        ref = orc.rtm2d_mpi_shot(v, e, d, fs_sxd=x, ds_sxd=0, zs_sxd=1, is_=k + 1, nxs=w, prec=64, **kw)[0]
        e_exact, e_fast = rel_l2(per[k], ref), rel_l2(fper[k], ref)
        assert e_fast <= 1.5 * e_exact, (k, e_fast, e_exact)
        assert rel_l2(fper[k], per[k]) < 1e-2, k
    assert rel_l2(fimg, img) < 1e-2
    with pytest.raises(geo.GeoError):
        geo.rtm2d_batch(v, e, d, mode=7, **run)


def test_rtm2d_golden(geo):
    import os
    r = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_rtm2d_mpi.npz"))
    xs = [int(r["fs"]) + (int(s) - 1) * int(r["ds"]) for s in r["shots"]]
    img = geo.rtm2d_batch(r["v"], r["e"], r["d"], npd=int(r["npd"]), nt=int(r["nt"]), dx=10.0, dz=10.0, dt_ms=1.0,
                          favg=20.0, pfac=1000.0, zs=1, shot_x=xs, shot_nxs=list(r["widths"]))
    assert np.abs(img - r["image"]).max() <= 1e-5 * np.abs(r["image"]).max()


def test_rtm2d_window_outside_model(geo):
    v, e, d = model()
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm2d_batch(v, e, d, npd=15, nt=50, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0, zs=1,
                        shot_x=[10], shot_nxs=[41])
    assert ei.value.status == 6


def test_laplace_gpu_vs_oracle(geo, orc):
    img = np.random.default_rng(1).standard_normal((83, 47)).astype(np.float32)
    assert np.array_equal(geo.laplace2d(img), orc.laplace2d_adj(img))
    vol = np.random.default_rng(2).standard_normal((9, 13, 11)).astype(np.float32)
    assert np.array_equal(geo.laplace3d(vol), orc.laplace3d_adj(vol))


def test_rtm2d_adcig_bit_exact(geo, orc):
    """Poynting angle gathers (the MPI program's flag_adcig = 1): the
    batched run's stacked gathers equal the oracle's, angle plane by angle
    plane, and the image is unchanged by asking for them."""
    v, e, d = model()
    xs, ws = [35, 55, 48], [41, 53, 31]
    kw = dict(npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0)
    acc = np.zeros(v.shape, np.float32)
    ago = np.zeros((90,) + v.shape, np.float32)
    for k, (x, w) in enumerate(zip(xs, ws)):
        mo, off, _, ag = orc.rtm2d_mpi_shot(v, e, d, fs_sxd=x, ds_sxd=0, zs_sxd=1, is_=k + 1, nxs=w, adcig=True, **kw)
        orc.stack2d(acc, mo, off)
        for ia in range(90):
            orc.stack2d(ago[ia], ag[ia], off)
    img, gathers = geo.rtm2d_batch(v, e, d, zs=1, shot_x=xs, shot_nxs=ws, laplace=False, adcig=True, **kw)
    assert np.array_equal(img, acc)
    assert gathers.shape == (90,) + v.shape
    assert (np.abs(ago).reshape(90, -1).max(axis=1) > 0).sum() > 10
    assert np.array_equal(gathers, ago)


GKW = dict(npml=20, nt=700, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, ns=2, fs=30, ds=35, zs=2,
           mute_tt=20, nangle=70, dangle=1)


def test_rtm2d_gpu_program_bit_exact(geo, orc):
    """The 2D GPU RTM program (ring saving, forward-stepped reconstruction,
    Poynting gathers): image, illumination, gathers, angle stack and
    records equal the oracle's."""
    v, e, d = model(nx=96, nz=60)
    mig, ill, ag, shots = orc.rtm2d_gpu(v, e, d, **cuda_angle_tables(GKW["dangle"]), **GKW)
    out = geo.rtm2d_gpu(v, e, d, **GKW)
    assert np.abs(ill).max() > 0 and np.abs(ag).max() > 0
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["illum"], ill)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag)
    stk = np.zeros(v.shape, np.float32)
    for ia in range(GKW["nangle"]):
        stk = (stk + ag[:, ia, :]).astype(np.float32)
    assert np.array_equal(out["stk_lap"], orc.laplace2d_adj(stk))


def test_rtm2d_gpu_program_observed_shots(geo, orc):
    v, e, d = model(nx=96, nz=60)
    kw = dict(GKW, ns=1, nt=520)          # nt < 512 rounding: the mute's surplus threads span traces
    obs = np.random.default_rng(5).standard_normal((1, 96, 520)).astype(np.float32) * 1e-3
    mig, ill, ag, _ = orc.rtm2d_gpu(v, e, d, obs=obs, **cuda_angle_tables(kw["dangle"]), **kw)
    out = geo.rtm2d_gpu(v, e, d, obs=obs, **kw)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag)


def test_rtm2d_gpu_program_thin_sponge_large_grid(geo, orc):
    """npml = 5 puts the ring's bottom row and right column outside the
    updated band (they carry saved and restored values only), and a grid of
    more points than one wave of resident threads makes each thread of the
    persistent passes stride over several points."""
    v, e, d = model(nx=700, nz=400)
    kw = dict(GKW, npml=5, ns=1, nt=150, fs=350)
    mig, ill, ag, shots = orc.rtm2d_gpu(v, e, d, **cuda_angle_tables(kw["dangle"]), **kw)
    out = geo.rtm2d_gpu(v, e, d, **kw)
    assert np.abs(ill).max() > 0
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["illum"], ill)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag)


@pytest.mark.parametrize("every", ["0", "7"])
def test_rtm2d_gpu_program_independent_of_launch_segments(geo, orc, monkeypatch, every):
    monkeypatch.setenv("GEO_WATCH_EVERY", every)
    v, e, d = model(nx=80, nz=50)
    kw = dict(GKW, ns=1, nt=130)
    mig, ill, ag, shots = orc.rtm2d_gpu(v, e, d, **cuda_angle_tables(kw["dangle"]), **kw)
    out = geo.rtm2d_gpu(v, e, d, **kw)
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["illum"], ill)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag)


def test_rtm2d_gpu_program_stability_check(geo):
    v, e, d = model(nx=96, nz=60)
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm2d_gpu(v, e, d, **dict(GKW, dt=np.float32(5e-3)))
    assert ei.value.status == 5
