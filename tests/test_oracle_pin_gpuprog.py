"""The oracle's GPU-program restatements against the reference's own GPU
programs: golden outputs made by running GPU_vti3dfd and GPU_vti2dfd
(2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu:371,
GPU_vti2dfd_kernels.cu:301), the 2D TTI forward program
(2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:312) and the three
GPU RTM programs (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:1184,
2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:500,
3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:686), their
device code compiled unmodified, on a GPU
(tests/golden/make_golden_refgpu.py).  CPU only.  Where the programs call
cosf on the device (the TTI tilt, the angle-gather weights) and acosf (the
angle-gather bins), the fixtures carry the device's values and bin edges,
and the oracle is given them.

The programs were built twice: with contraction to FMA off ("nofma"), which
the oracle reproduces bit for bit, and with the compiler's defaults ("fma",
how the reference's Makefile builds them), from which any reordering of the
same arithmetic -- the reference's own no-FMA build included -- sits at a
rounding distance."""
import ctypes as C
import hashlib
import os
import sys

import numpy as np
import pytest

from tests.util import rel_l2

GOLD = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLD)
import make_golden_refgpu as M  # noqa: E402


def _load(name):
    path = os.path.join(GOLD, name)
    sums = dict(l.split()[::-1] for l in open(os.path.join(GOLD, "SHA256SUMS")) if l.strip())
    assert hashlib.sha256(open(path, "rb").read()).hexdigest() == sums[name], "fixture %s changed" % name
    return np.load(path)


def oracle_fd3d_dropin(orc, v, e, d, kw, is_):
    """The oracle's exact 3D form with GPU_vti3dfd's receivers (every
    surface node at iz = npml) and its direct-wave mute (tt = 100)."""
    ny, nx, nz = v.shape
    dt = np.float32(kw["dt_us"] * 1.0 / 1000000)
    r = orc.fd3d(v, e, d, mode=0, sv=kw["sv"], npd=kw["npml"], nt=kw["nt"], dx=float(kw["dx"]), dy=float(kw["dy"]),
                 dz=float(kw["dz"]), dt=dt, favg=float(kw["favg"]), pfac=10.0, fsx=kw["fsx"], fsy=kw["fsy"],
                 fsz=kw["fsz"], dsx=kw["dsx"], dsy=kw["dsy"], dsz=kw["dsz"], is_=is_).copy()
    orc.lib().orc_mute3d(nx, ny, kw["nt"], dt, float(kw["favg"]), float(kw["dx"]), float(kw["dy"]), float(kw["dz"]),
                         kw["fsx"], kw["fsy"], kw["dsx"], kw["dsy"], kw["fsz"], is_, np.float32(v[0, 0, 0]),
                         np.float32(e[0, 0, 0]), 100, r.ctypes.data_as(C.POINTER(C.c_float)))
    return r


def oracle_fd2d_dropin(orc, v, e, d, kw, is_, snap_every=0):
    """The oracle's GPU-program 2D form with GPU_vti2dfd's mute (tt = 100)."""
    nx, nz = v.shape
    dt = np.float32(kw["dt_us"] * 1.0 / 1000000)
    out = orc.fd2d(v, e, d, npd=kw["npd"], nt=kw["nt"], dx=float(kw["dx"]), dz=float(kw["dz"]), dt=dt,
                   favg=float(kw["favg"]), pfac=10.0, fs=float(kw["fs"]), ds=float(kw["ds"]), zs=float(kw["zs"]),
                   is_=is_, sv=kw["sv"], variant=orc.V_GPU, snap_every=snap_every)
    r, snaps = (out if snap_every else (out, None))
    r = r.copy()
    vp1 = v[0, 0] * np.sqrt(np.float32(1) + np.float32(2) * e[0, 0])
    orc.lib().orc_mute2d(0, nx, kw["nt"], dt, float(kw["favg"]), float(kw["dx"]), float(kw["dz"]), kw["fs"], kw["ds"],
                         kw["zs"], is_, np.float32(vp1), 100, r.ctypes.data_as(C.POINTER(C.c_float)))
    return r, snaps


@pytest.mark.parametrize("case", sorted(M.CASES3))
def test_fd3d_oracle_bit_exact_vs_GPU_vti3dfd(orc, case):
    g = _load("golden_fd3d_gpu.npz")
    v, e, d = g["v"], g["e"], g["d"]
    kw = M.CASES3[case]
    ref = g["shot_%s_nofma" % case]
    for is_ in range(kw["ns"]):
        mine = oracle_fd3d_dropin(orc, v, e, d, kw, is_)
        assert np.abs(mine).max() > 0
        assert np.array_equal(mine, ref[is_]), (is_, rel_l2(mine, ref[is_]))
        # the default (FMA) build of the same program: rounding distance
        assert rel_l2(mine, g["shot_%s_fma" % case][is_]) < 1e-4


@pytest.mark.parametrize("case", sorted(M.CASES2))
def test_fd2d_gpu_variant_oracle_bit_exact_vs_GPU_vti2dfd(orc, case):
    g = _load("golden_fd2d_gpu.npz")
    v, e, d = g["v"], g["e"], g["d"]
    kw = M.CASES2[case]
    ref = g["shot_%s_nofma" % case]
    for is_ in range(1, kw["ns"] + 1):
        mine, snaps = oracle_fd2d_dropin(orc, v, e, d, kw, is_, snap_every=50 if "snap_%s_nofma" % case in g else 0)
        assert np.abs(mine).max() > 0
        assert np.array_equal(mine, ref[is_ - 1]), (is_, rel_l2(mine, ref[is_ - 1]))
        assert rel_l2(mine, g["shot_%s_fma" % case][is_ - 1]) < 1e-4
        if snaps is not None and is_ == 1:
            assert np.array_equal(snaps, g["snap_%s_nofma" % case])


@pytest.mark.parametrize("case", sorted(M.CASEST))
def test_tti2d_oracle_bit_exact_vs_reference_program(orc, case):
    g = _load("golden_tti2d_gpu.npz")
    v, e, d, th = g["v"], g["e"], g["d"], g["theta"]
    kw = M.CASEST[case]
    ref = g["shot_%s_nofma" % case]
    snap_every = 100 if "snap_%s_nofma" % case in g else 0
    for is_ in range(1, kw["ns"] + 1):
        out = orc.tti2d(v, e, d, th, npd=kw["npml"], nt=kw["nt"], dx=kw["dx"], dz=kw["dz"], dt=np.float32(kw["dt"]),
                        favg=kw["favg"], pfac=kw["pfac"], fs=float(kw["fs"]), ds=float(kw["ds"]), zs=float(kw["zs"]),
                        is_=is_, sv=kw["sv"], snap_every=snap_every, trig=(g["cos_dev"], g["sin_dev"]))
        mine, snaps = out if snap_every else (out, None)
        assert np.abs(mine).max() > 0
        assert np.array_equal(mine, ref[is_ - 1]), (is_, rel_l2(mine, ref[is_ - 1]))
        assert rel_l2(mine, g["shot_%s_fma" % case][is_ - 1]) < 1e-4
        if snaps is not None and is_ == 1:
            assert np.array_equal(snaps, g["snap_%s_nofma" % case])


def test_reference_builds_differ_by_rounding_only():
    """The reference program's two builds agree to FP32 rounding, and no
    closer: the target 'within 1e-5 of the reference' is met by the
    reference's own no-FMA build only up to this distance."""
    for name, cases in (("golden_fd3d_gpu.npz", M.CASES3), ("golden_fd2d_gpu.npz", M.CASES2),
                        ("golden_tti2d_gpu.npz", M.CASEST)):
        g = _load(name)
        for c in cases:
            a, b = g["shot_%s_fma" % c], g["shot_%s_nofma" % c]
            assert not np.array_equal(a, b)
            assert rel_l2(a, b) < 1e-4


def _rtm2d_kw(name):
    kw = dict(M.RTM_VTI)
    kw["dt"] = np.float32(kw["dt"])
    if name == "vti_b":
        kw.update(ns=1, fs=31)
    return kw


@pytest.mark.parametrize("name", ["vti_a", "vti_b"])
def test_rtm2d_gpu_oracle_bit_exact_vs_reference_program(orc, name):
    """orc_rtm2d_gpu against the 2D GPU RTM program's RTM() (ring saving,
    forward-stepped reconstruction, illumination, Poynting gathers; b reads
    observed records): image and gathers divided by the illumination, the
    illumination and the muted records, bit for bit."""
    g = _load("golden_rtm2d_gpu.npz")
    t = name + "_nofma"
    obs = g["obs"] if name == "vti_b" else None
    mig, ill, ag, shots = orc.rtm2d_gpu(g["v"], g["e"], g["d"], mute_tt=20, obs=obs,
                                        angle_cos=g["angle_cos_dev"], angle_thr=g["angle_thr_dev"],
                                        **_rtm2d_kw(name))
    assert np.abs(ag).max() > 0 and (np.abs(ag).max(axis=(0, 2)) > 0).all()
    assert np.array_equal(shots, g["shots_" + t])
    assert np.array_equal(ill, g["ill_" + t])
    assert np.array_equal(mig, g["mig_" + t])
    assert np.array_equal(ag, g["ag_" + t]), rel_l2(ag, g["ag_" + t])
    if "mig_%s_fma" % name in g:
        assert rel_l2(mig, g["mig_%s_fma" % name]) < 1e-4


@pytest.mark.parametrize("name,dcdp", [("tti_a", 1), ("tti_b", 3)])
def test_rtm2d_tti_oracle_bit_exact_vs_reference_program(orc, name, dcdp):
    """orc_rtm2d_tti against the 2D TTI GPU RTM program, gathers at every CDP
    and every third (64 traces: not a multiple of 3)."""
    g = _load("golden_rtm2d_gpu.npz")
    kw = dict(M.RTM_TTI)
    kw["dt"] = np.float32(kw["dt"])
    t = name + "_nofma"
    mig, ill, ag, shots = orc.rtm2d_tti(g["tv"], g["te"], g["td"], g["theta"], dcdp=dcdp, mute_tt=30,
                                        trig=(g["tcos_dev"], g["tsin_dev"]), angle_cos=g["angle_cos_dev"],
                                        angle_thr=g["angle_thr_dev"], **kw)
    assert np.abs(ag).max() > 0
    assert np.array_equal(shots, g["shots_tti_a_nofma"])
    assert np.array_equal(ill, g["ill_" + t])
    assert np.array_equal(mig, g["mig_" + t])
    assert np.array_equal(ag, g["ag_" + t]), rel_l2(ag, g["ag_" + t])
    if "mig_%s_fma" % name in g:
        assert rel_l2(mig, g["mig_%s_fma" % name]) < 1e-4


@pytest.mark.parametrize("case", sorted(M.CASES_RTM3))
def test_rtm3d_oracle_bit_exact_vs_reference_program(orc, case):
    """orc_rtm3d_shot (boundary-saving RTM, exact form, SV taper on every
    propagation as the program runs it) against the 3D GPU RTM program:
    image and gathers divided by the illumination, the illumination and the
    last shot's muted record, bit for bit."""
    g = _load("golden_rtm3d_gpu.npz")
    kw = M.CASES_RTM3[case]
    k = dict(npd=kw["npml"], nt=kw["nt"], dx=kw["dx"], dy=kw["dy"], dz=kw["dz"], dt=np.float32(kw["dt"]),
             favg=kw["favg"], pfac=kw["pfac"], fsx=kw["fsx"], fsy=kw["fsy"], fsz=kw["zs"], dsx=kw["dsx"],
             dsy=kw["dsy"], ns=kw["ns"], sv=1, mute_tt=70)
    t = case + "_nofma"
    mig, ill, rec, ag = orc.rtm3d(g["v"], g["e"], g["d"], mode=0, adcig=(kw["na"], kw["da"], kw["dcdp"]),
                                  angle_cos=g["angle_cos_dev"], angle_thr=g["angle_thr_dev"], **k)
    assert np.abs(ag).max() > 0
    assert np.array_equal(rec, g["shots_a_nofma"][kw["ns"] - 1])
    assert np.array_equal(ill, g["ill_" + t])
    assert np.array_equal(mig, g["mig_" + t])
    assert np.array_equal(ag, g["ag_" + t]), rel_l2(ag, g["ag_" + t])
    if "mig_%s_fma" % case in g:
        assert rel_l2(mig, g["mig_%s_fma" % case]) < 1e-4
