"""The library's drop-ins GPU_vti3dfd and GPU_vti2dfd, its 2D TTI shot and
its three GPU-program RTMs against the reference's own GPU programs
(2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu, GPU_vti2dfd_kernels.cu,
2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu,
2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu,
2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu,
3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu), whose device
code was compiled unmodified and run on a GPU: the golden outputs of
tests/golden/make_golden_refgpu.py, and, where the cubins are present
(oracle/_ref), the 400^3 headline shot run through the reference program
itself.

Tolerances: the exact 3D form and the 2D GPU-program form are bit-identical
to the program built with contraction to FMA off.  The fast 3D form (FMAs at
fixed places, unsplit interior) is held to the distance between the
reference program's own two builds (default FMA contraction against none),
with a margin of 1.5x: that distance is what rounding alone does to this
computation."""
import os

import numpy as np
import pytest

from tests.test_oracle_pin_gpuprog import M, _load
from tests.util import rel_l2

pytestmark = pytest.mark.gpu


def _files(tmp_path, tag, v, e, d):
    names = []
    for name, a in (("v", v), ("e", e), ("d", d)):
        p = tmp_path / ("%s_%s.bin" % (name, tag))
        a.tofile(p)
        names.append(str(p))
    return names


def _run3d(geo, tmp_path, g, case, mode, monkeypatch):
    v, e, d = g["v"], g["e"], g["d"]
    ny, nx, nz = v.shape
    kw = M.CASES3[case]
    monkeypatch.setenv("GEO_FD3D_MODE", mode)
    fv, fe, fd = _files(tmp_path, case, v, e, d)
    shot, snap = str(tmp_path / ("shot3_%s_%s.bin" % (case, mode))), str(tmp_path / ("snap3_%s_%s.bin" % (case, mode)))
    geo.GPU_vti3dfd(nx, ny, nz, kw["dx"], kw["dy"], kw["dz"], kw["npml"], kw["sv"], fv, fe, fd, kw["favg"], kw["ns"],
                    kw["fsx"], kw["dsx"], kw["fsy"], kw["dsy"], kw["fsz"], kw["dsz"], shot, snap, kw["nt"], kw["dt_us"])
    out = np.fromfile(shot, np.float32).reshape(kw["ns"], ny, nx, kw["nt"])
    sn = np.fromfile(snap, np.float32) if os.path.getsize(snap) else None
    return out, sn


@pytest.mark.parametrize("case", sorted(M.CASES3))
def test_GPU_vti3dfd_exact_form_bit_exact_vs_reference_program(geo, tmp_path, monkeypatch, case):
    g = _load("golden_fd3d_gpu.npz")
    out, sn = _run3d(geo, tmp_path, g, case, "exact", monkeypatch)
    ref = g["shot_%s_nofma" % case]
    assert np.abs(out).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)
    if "snap_%s_nofma" % case in g:
        rs = g["snap_%s_nofma" % case].reshape(-1)
        assert sn is not None and np.array_equal(sn[:rs.size], rs)


@pytest.mark.parametrize("case", sorted(M.CASES3))
def test_GPU_vti3dfd_fast_form_within_the_reference_builds_distance(geo, tmp_path, monkeypatch, case):
    g = _load("golden_fd3d_gpu.npz")
    out, _ = _run3d(geo, tmp_path, g, case, "fast", monkeypatch)
    fma, nofma = g["shot_%s_fma" % case], g["shot_%s_nofma" % case]
    own = rel_l2(fma, nofma)
    assert rel_l2(out, nofma) <= 1.5 * own, (rel_l2(out, nofma), own)
    assert rel_l2(out, fma) <= 1.5 * own, (rel_l2(out, fma), own)


@pytest.mark.parametrize("case", sorted(M.CASES2))
def test_GPU_vti2dfd_bit_exact_vs_reference_program(geo, tmp_path, case):
    g = _load("golden_fd2d_gpu.npz")
    v, e, d = g["v"], g["e"], g["d"]
    nx, nz = v.shape
    kw = M.CASES2[case]
    fv, fe, fd = _files(tmp_path, "2d" + case, v, e, d)
    shot, snap = str(tmp_path / "shot2.bin"), str(tmp_path / "snap2.bin")
    geo.GPU_vti2dfd(nx, nz, kw["dx"], kw["dz"], kw["npd"], kw["sv"], fv, fe, fd, kw["favg"], kw["ns"], kw["fs"], kw["ds"],
                    kw["zs"], shot, snap, kw["nt"], kw["dt_us"])
    out = np.fromfile(shot, np.float32).reshape(kw["ns"], nx, kw["nt"])
    ref = g["shot_%s_nofma" % case]
    assert np.abs(out).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)
    if "snap_%s_nofma" % case in g:
        rs = g["snap_%s_nofma" % case].reshape(-1)
        assert np.array_equal(np.fromfile(snap, np.float32)[:rs.size], rs)


@pytest.mark.parametrize("case", sorted(M.CASEST))
def test_tti2d_shot_bit_exact_vs_reference_program(geo, case):
    """geo_tti2d_shot against the 2D TTI forward program
    (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:312-470)."""
    g = _load("golden_tti2d_gpu.npz")
    v, e, d, th = g["v"], g["e"], g["d"], g["theta"]
    kw = M.CASEST[case]
    snap_every = 100 if "snap_%s_nofma" % case in g else 0
    for is_ in range(1, kw["ns"] + 1):
        out = geo.tti2d_shot(v, e, d, th, npd=kw["npml"], nt=kw["nt"], dx=kw["dx"], dz=kw["dz"], dt=kw["dt"],
                             favg=kw["favg"], pfac=kw["pfac"], fs=float(kw["fs"]), ds=float(kw["ds"]),
                             zs=float(kw["zs"]), is_=is_, sv=kw["sv"], snap_every=snap_every)
        shot, snaps = out if snap_every else (out, None)
        ref = g["shot_%s_nofma" % case][is_ - 1]
        assert np.abs(shot).max() > 0
        assert np.array_equal(shot, ref), rel_l2(shot, ref)
        if snaps is not None and is_ == 1:
            assert np.array_equal(snaps, g["snap_%s_nofma" % case])


def _rtm_case(name):
    """The RTM fixture's case `name` as (library kwargs, golden tag)."""
    kw = dict(M.RTM_VTI)
    kw["dt"] = np.float32(kw["dt"])
    if name == "vti_b":
        kw.update(ns=1, fs=31)
    return kw, name + "_nofma"


@pytest.mark.parametrize("name", ["vti_a", "vti_b"])
def test_rtm2d_gpu_program_bit_exact_vs_reference_program(geo, orc, name):
    """geo_rtm2d_gpu against the 2D GPU RTM program's RTM()
    (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:1184-1566): muted records, image,
    illumination and Poynting gathers (both divided by the illumination),
    with modelled (a) and observed (b, readShot) records.  The program
    filters its image on the host with its own Laplacian; the library's is
    compared through the oracle's, which is pinned to laplace.c."""
    g = _load("golden_rtm2d_gpu.npz")
    kw, t = _rtm_case(name)
    obs = g["obs"] if name == "vti_b" else None
    out = geo.rtm2d_gpu(g["v"], g["e"], g["d"], mute_tt=20, obs=obs, **kw)
    assert np.abs(g["ag_" + t]).max() > 0
    assert np.array_equal(out["shots"], g["shots_" + t])
    assert np.array_equal(out["illum"], g["ill_" + t])
    assert np.array_equal(out["adcigs"], g["ag_" + t]), rel_l2(out["adcigs"], g["ag_" + t])
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(g["mig_" + t]))


@pytest.mark.parametrize("name,dcdp", [("tti_a", 1), ("tti_b", 3)])
def test_rtm2d_tti_program_bit_exact_vs_reference_program(geo, orc, name, dcdp):
    """geo_rtm2d_tti against the 2D TTI GPU RTM program
    (Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:500-800), gathers at every
    CDP and at every third (64 traces: not a multiple of 3)."""
    g = _load("golden_rtm2d_gpu.npz")
    kw = dict(M.RTM_TTI)
    kw["dt"] = np.float32(kw["dt"])
    t = name + "_nofma"
    out = geo.rtm2d_tti(g["tv"], g["te"], g["td"], g["theta"], dcdp=dcdp, mute_tt=30, **kw)
    assert np.abs(g["ag_" + t]).max() > 0
    assert np.array_equal(out["shots"], g["shots_tti_a_nofma"])
    assert np.array_equal(out["illum"], g["ill_" + t])
    assert np.array_equal(out["adcigs"], g["ag_" + t]), rel_l2(out["adcigs"], g["ag_" + t])
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(g["mig_" + t]))


def rtm3d_kwargs(kw):
    """The library's / oracle's arguments for a 3D RTM program case: the
    program runs the SV taper on every propagation and mutes with tt = 70."""
    return dict(npd=kw["npml"], nt=kw["nt"], dx=kw["dx"], dy=kw["dy"], dz=kw["dz"], dt=np.float32(kw["dt"]),
                favg=kw["favg"], pfac=kw["pfac"], fsx=kw["fsx"], fsy=kw["fsy"], fsz=kw["zs"], dsx=kw["dsx"],
                dsy=kw["dsy"], ns=kw["ns"], sv=1, mute_tt=70)


@pytest.mark.parametrize("case", sorted(M.CASES_RTM3))
def test_rtm3d_program_bit_exact_vs_reference_program(geo, case):
    """geo_rtm3d (boundary method, exact form) against the 3D GPU RTM
    program (Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:686-981): image and
    gathers divided by the illumination, and the illumination; the fast
    form within the distance between the program's two builds (x1.5)."""
    g = _load("golden_rtm3d_gpu.npz")
    kw = M.CASES_RTM3[case]
    k = rtm3d_kwargs(kw)
    ad = (kw["na"], kw["da"], kw["dcdp"])
    t = case + "_nofma"
    mig, ill, ag = geo.rtm3d(g["v"], g["e"], g["d"], mode="exact", laplace=False, illum=True, adcig=ad, **k)
    assert np.abs(g["ag_" + t]).max() > 0
    assert np.array_equal(mig, g["mig_" + t]), rel_l2(mig, g["mig_" + t])
    assert np.array_equal(ill, g["ill_" + t])
    assert np.array_equal(ag, g["ag_" + t]), rel_l2(ag, g["ag_" + t])
    if "mig_%s_fma" % case in g:
        own = rel_l2(g["mig_%s_fma" % case], g["mig_" + t])
        fast = geo.rtm3d(g["v"], g["e"], g["d"], mode="fast", laplace=False, **k)
        assert rel_l2(fast, g["mig_" + t]) <= 1.5 * own and rel_l2(fast, g["mig_%s_fma" % case]) <= 1.5 * own


@pytest.mark.parametrize("da", [1, 2, 3])
def test_poynting_bin_edges_reproduce_device_bins(da):
    """The GPU RTM programs' angle bin (int)((float)(0.5*acosf(a)*180/pi)/da)
    with the device's acosf is, for every float a in [-1, 1] (2.1e9 values,
    on the GPU), the number of the device's bin edges at or above a -- the
    form the CPU oracle is given and the library's gathers use.  The host's
    acosf puts a few cosines next to an edge in the neighbouring bin
    (printed)."""
    from oracle import refgpu
    thr = refgpu.cuda_angle_thresholds(da, 128)
    assert (np.diff(thr[thr > -2]) < 0).all()
    assert refgpu.bin_check(128, da, thr) == 0
    host = refgpu.host_bin_thresholds(128, da)
    print("POYNTING_BINS da=%d: edges differing host/device %d, floats binned differently by the host's acosf %d"
          % (da, int((host != thr).sum()), refgpu.bin_check(128, da)))


def test_headline_shot_against_reference_program(geo):
    """The 400^3 + 40 headline shot (2500 steps, dt 0.8 ms, 15 Hz, the
    bench's random-field model), every surface node recorded and muted as
    GPU_vti3dfd records it: the exact form is bit-identical to the reference
    program built without contraction; the fast form is held to the
    distance between the reference program's two builds."""
    from oracle import refgpu
    if not refgpu.available("vti3d"):
        pytest.skip("reference program cubins not built (oracle/_ref)")
    import bench
    v, e, d = (a.cpu().numpy() for a in bench.make_model(device="cpu"))
    n, npd, nt = bench.NX, bench.NPD, bench.NT
    rkw = dict(dx=10, dy=10, dz=10, npml=npd, sv=0, favg=15, ns=1, fsx=n // 2, dsx=0, fsy=n // 2, dsy=0, fsz=1,
               dsz=0, nt=nt, dt_us=800)
    ref_nofma, _, ms_nofma = refgpu.vti3d(v, e, d, fma=False, **rkw)
    ref_fma, _, ms_fma = refgpu.vti3d(v, e, d, fma=True, **rkw)
    out = {}
    for mode in ("exact", "fast"):
        plan = geo.FD3DPlan(nx=n, ny=n, nz=n, npd=npd, nt=nt, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(0.0008),
                            favg=15.0, pfac=10.0, fsx=n // 2, fsy=n // 2, fsz=1, mode=mode, mute_tt=100)
        plan.set_model(v, e, d)
        out[mode] = plan.run_shot(0)
        plan.close()
    own = rel_l2(ref_fma[0], ref_nofma[0])
    res = {"exact_vs_nofma": rel_l2(out["exact"], ref_nofma[0]), "exact_vs_fma": rel_l2(out["exact"], ref_fma[0]),
           "fast_vs_nofma": rel_l2(out["fast"], ref_nofma[0]), "fast_vs_fma": rel_l2(out["fast"], ref_fma[0]),
           "fast_vs_exact": rel_l2(out["fast"], out["exact"]), "fma_vs_nofma": own,
           "ref_ms_per_step_fma": ms_fma, "ref_ms_per_step_nofma": ms_nofma}
    print("HEADLINE_VS_REFERENCE", res)
    assert np.abs(out["exact"]).max() > 0
    assert np.array_equal(out["exact"], ref_nofma[0])
    assert res["fast_vs_nofma"] <= 1.5 * own and res["fast_vs_fma"] <= 1.5 * own
