"""Par-file runs (geo_fd2d, geo_fd3d, geo_rtm2d) against the same runs made
through the library's descriptor entry points: files and device buffers
bit-identical."""
import numpy as np
import pytest

from tests.util import layered_model, random_model_3d

pytestmark = pytest.mark.gpu


def _write(tmp, name, a):
    path = tmp / name
    np.ascontiguousarray(a, np.float32).tofile(path)
    return str(path)


def _par(tmp, name, **kv):
    path = tmp / name
    path.write_text("".join("%12s= %s\n" % (k, v) for k, v in kv.items()))
    return str(path)


def test_fd2d_par(geo, tmp_path):
    import torch
    v, e, d = layered_model(61, 51, seed=2)
    kw = dict(nx=61, nz=51, dx=10, dz=10, npd=20, nt=300, dt=1000, favg=20, ns=2, fs=20, ds=15, zs=3, SV=1,
              FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e), FNd=_write(tmp_path, "d", d),
              FNshot=str(tmp_path / "shot"), FNsnap=str(tmp_path / "snap"))
    out = geo.fd2d_par(_par(tmp_path, "fd.par", **kw), device=0, out_shape=(2, 61, 300))
    shots = np.fromfile(tmp_path / "shot", np.float32).reshape(2, 61, 300)
    snaps = np.fromfile(tmp_path / "snap", np.float32).reshape(6, 101, 91)
    for is_ in (1, 2):
        ref = geo.fd2d_shot(v, e, d, npd=20, nt=300, dx=10.0, dz=10.0, dt=1e-3, favg=20.0, fs=20, ds=15, zs=3,
                            is_=is_, variant="gpu", sv=1, mute_tt=100, snap_every=50 if is_ == 1 else 0)
        rec = ref[0] if is_ == 1 else ref
        assert np.abs(rec).max() > 0
        assert np.array_equal(shots[is_ - 1], rec)
        assert np.array_equal(out[is_ - 1].cpu().numpy(), rec)
        if is_ == 1:
            assert np.array_equal(snaps, ref[1])


def test_fd3d_par(geo, tmp_path):
    v, e, d = random_model_3d(20, 18, 22, seed=5)
    kw = dict(nx=20, ny=18, nz=22, dx=10, dy=10, dz=10, npml=10, nt=200, dt=1000, favg=25, ns=2, fsx=6, fsy=8,
              fsz=2, dsx=5, SV=1, mute_tt=5, FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e),
              FNd=_write(tmp_path, "d", d), FNshot=str(tmp_path / "shot"))
    out = geo.fd3d_par(_par(tmp_path, "fd3.par", **kw), out_shape=(2, 18, 20, 200))
    shots = np.fromfile(tmp_path / "shot", np.float32).reshape(2, 18, 20, 200)
    plan = geo.FD3DPlan(nx=20, ny=18, nz=22, npd=10, nt=200, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0, fsx=6,
                        fsy=8, fsz=2, dsx=5, sv=1, mode="exact", mute_tt=5)
    try:
        plan.set_model(v, e, d)
        for is_ in (0, 1):
            rec = plan.run_shot(is_)
            assert np.abs(rec).max() > 0
            assert np.array_equal(shots[is_], rec)
            assert np.array_equal(out[is_].cpu().numpy(), rec)
    finally:
        plan.close()


def test_fd3d_par_tti(geo, tmp_path):
    """The par run on a 3D TTI medium (FNtheta, FNphi) equals the plan with
    set_tilt."""
    from tests.util import smooth_angles
    v, e, d = random_model_3d(20, 18, 22, seed=6)
    th, ph = smooth_angles(v.shape, seed=5)
    kw = dict(nx=20, ny=18, nz=22, dx=10, dy=10, dz=10, npml=10, nt=160, dt=1000, favg=25, ns=1, fsx=6, fsy=8,
              fsz=2, mode="fast", mute_tt=5, FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e),
              FNd=_write(tmp_path, "d", d), FNtheta=_write(tmp_path, "th", th), FNphi=_write(tmp_path, "ph", ph),
              FNshot=str(tmp_path / "shot"))
    geo.fd3d_par(_par(tmp_path, "fd3t.par", **kw))
    shot = np.fromfile(tmp_path / "shot", np.float32).reshape(18, 20, 160)
    plan = geo.FD3DPlan(nx=20, ny=18, nz=22, npd=10, nt=160, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0, fsx=6,
                        fsy=8, fsz=2, mode="fast", mute_tt=5)
    try:
        plan.set_model(v, e, d)
        plan.set_tilt(th, ph)
        rec = plan.run_shot(0)
        assert np.abs(rec).max() > 0
        assert np.array_equal(shot, rec)
    finally:
        plan.close()
    bad = dict(kw, FNphi="")
    del bad["FNphi"]
    with pytest.raises(geo.GeoError):
        geo.fd3d_par(_par(tmp_path, "fd3bad.par", **bad))


@pytest.mark.parametrize("seismic", [1, 2])
def test_rtm2d_par(geo, tmp_path, seismic):
    rng = np.random.default_rng(3)
    v, e, d = layered_model(101, 50, seed=3, vlo=2000, vhi=2600)
    v = v + rng.uniform(0, 40, v.shape).astype(np.float32)
    names = {}
    for k, a in (("FN1", v), ("FN2", e), ("FN3", d)):
        if seismic == 2:
            names[k] = str(tmp_path / (k + ".su"))
            geo.su_write(names[k], a, dt_us=1000, big_endian=True)
        else:
            names[k] = _write(tmp_path, k, a)
    outs = {k: str(tmp_path / k) for k in ("FN6", "FN7", "FN8", "FN9", "FN10")}
    kw = dict(nx=101, nz=50, dx=10, dz=10, npd=15, nt=650, dt=1, favg=20, pfac=1000, ns_sxd=3, fs_sxd=35, ds_sxd=10,
              zs_sxd=1, nxs=41, seismic=seismic, **names, **outs)
    img_dev = geo.rtm2d_par(_par(tmp_path, "rtm.par", **kw), out_shape=(101, 50))
    img, per, gathers = geo.rtm2d_batch(v, e, d, npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0,
                                        zs=1, shot_x=[35, 45, 55], shot_nxs=[41] * 3, laplace=False, per_shot=True,
                                        adcig=True)
    sg, stk = geo.adcig_smooth_stack(gathers, 10)
    f = lambda k: np.fromfile(outs[k], np.float32)
    assert np.abs(img).max() > 0
    assert np.array_equal(f("FN6").reshape(101, 50), img)
    assert np.array_equal(img_dev.cpu().numpy(), img)
    assert np.array_equal(f("FN7"), np.concatenate([p.ravel() for p in per]))
    assert np.array_equal(f("FN8").reshape(101, 90, 50), gathers.transpose(1, 0, 2))
    assert np.array_equal(f("FN9").reshape(101, 90, 50), sg.transpose(1, 0, 2))
    assert np.array_equal(f("FN10").reshape(101, 50), stk)


def test_par_device_out_of_range(geo, tmp_path):
    v, e, d = layered_model(31, 31, seed=2)
    kw = dict(nx=31, nz=31, dx=10, dz=10, npd=20, nt=50, dt=1000, favg=20, ns=1, fs=15, ds=0, zs=3,
              FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e), FNd=_write(tmp_path, "d", d),
              FNshot=str(tmp_path / "shot"))
    with pytest.raises(geo.GeoError):
        geo.fd2d_par(_par(tmp_path, "fd.par", **kw), device=4096)


def _resume_case(geo, tmp_path, run, nrec, ns, shot_file, done_file):
    """Run to completion, then make the state of a run stopped after shot 0:
    the manifest lists shot 0 only, the later records are overwritten with
    junk, and shot 0's record is overwritten with a marker.  A rerun must
    leave the marker (shot 0 is not recomputed) and restore the rest bit for
    bit."""
    run()
    full = np.fromfile(shot_file, np.float32).copy()
    lines = open(done_file).read().splitlines()
    assert lines[0].startswith("geo_fd") and lines[1:] == ["shot %d" % k for k in range(ns)]
    # a second run with everything done recomputes nothing
    run()
    assert np.array_equal(np.fromfile(shot_file, np.float32), full)
    # stopped after the first shot
    open(done_file, "w").write("\n".join(lines[:2]) + "\n")
    junk = full.copy()
    junk[:nrec] = 7.0
    junk[nrec:] = np.nan
    junk.tofile(shot_file)
    run()
    got = np.fromfile(shot_file, np.float32)
    assert np.all(got[:nrec] == 7.0)
    assert np.array_equal(got[nrec:], full[nrec:])
    assert open(done_file).read().splitlines()[1:] == ["shot %d" % k for k in range(ns)]
    return full


def test_fd2d_par_resume(geo, tmp_path):
    v, e, d = layered_model(61, 51, seed=2)
    kw = dict(nx=61, nz=51, dx=10, dz=10, npd=20, nt=200, dt=1000, favg=20, ns=3, fs=20, ds=10, zs=3,
              FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e), FNd=_write(tmp_path, "d", d),
              FNshot=str(tmp_path / "shot"), resume=1)
    par = _par(tmp_path, "fd.par", **kw)
    full = _resume_case(geo, tmp_path, lambda: geo.fd2d_par(par), 61 * 200, 3, tmp_path / "shot",
                        tmp_path / "shot.done")
    # the same as a run without resume
    kw.pop("resume")
    kw["FNshot"] = str(tmp_path / "plain")
    geo.fd2d_par(_par(tmp_path, "plain.par", **kw))
    assert np.array_equal(np.fromfile(tmp_path / "plain", np.float32), full)
    # a manifest from another run is refused
    kw.update(FNshot=str(tmp_path / "shot"), resume=1, nt=150)
    with pytest.raises(geo.GeoError) as ei:
        geo.fd2d_par(_par(tmp_path, "other.par", **kw))
    assert ei.value.status == 1 and "another run" in str(ei.value)


def test_fd3d_par_resume(geo, tmp_path):
    v, e, d = random_model_3d(20, 18, 22, seed=5)
    kw = dict(nx=20, ny=18, nz=22, dx=10, dy=10, dz=10, npml=10, nt=120, dt=1000, favg=25, ns=3, fsx=6, fsy=8,
              fsz=2, dsx=4, mute_tt=5, FNv=_write(tmp_path, "v", v), FNe=_write(tmp_path, "e", e),
              FNd=_write(tmp_path, "d", d), FNshot=str(tmp_path / "shot"), FNdone=str(tmp_path / "m.txt"),
              resume=1)
    par = _par(tmp_path, "fd3.par", **kw)
    nrec = 18 * 20 * 120
    full = _resume_case(geo, tmp_path, lambda: geo.fd3d_par(par), nrec, 3, tmp_path / "shot", tmp_path / "m.txt")
    # with a device buffer the completed shots come back from the file
    out = geo.fd3d_par(par, out_shape=(3, 18, 20, 120)).cpu().numpy().reshape(-1)
    assert np.array_equal(out, np.fromfile(tmp_path / "shot", np.float32))
    assert np.array_equal(out[nrec:], full[nrec:])
