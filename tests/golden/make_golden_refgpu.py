"""Generate the golden fixtures of the reference's own GPU programs by
running them on a GPU: their device code compiled unmodified into cubins
(oracle/Makefile, from the reference tree) and driven by
oracle/ref_harness/refgpu.c through the CUDA driver API.

  python tests/golden/make_golden_refgpu.py [OUTDIR] [fd|rtm]   (needs a GPU)

(fd: the three forward programs' fixtures, rtm: the two RTM programs'; both
by default.)

Each case is run twice: with the compiler's default build of the program
(contraction to FMA on, as the reference's own Makefile builds it) and with
contraction off.

golden_fd3d_gpu.npz  GPU_vti3dfd (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu:371)
                     on a 20x16x24 smooth random VTI model, npml 8:
                     case a: SV off, 2 shots (source moving by dsx=2, dsy=1),
                             200 steps
                     case b: SV taper on, 1 shot, 310 steps with the P
                             snapshot window at it = 300
golden_fd2d_gpu.npz  GPU_vti2dfd (GPU_vti2dfd_kernels.cu:301) on a 61x51
                     layered VTI model, npd 20:
                     case a: SV off, 2 shots (ds = 5), 300 steps, with the
                             padded P snapshots of shot 1 every 50 steps
                     case b: SV taper on, 1 shot, 300 steps
golden_tti2d_gpu.npz the 2D TTI forward program
                     (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu,
                     main :312) on a 61x51 layered VTI model with a smooth
                     tilt field (5-40 degrees), npml 20:
                     case a: SV off (as its main), 2 shots (ds = 5), 300
                             steps, with the padded P snapshots of shot 1
                             every 100 steps
                     case b: SV taper on, 1 shot, 300 steps
                     plus cos_dev, sin_dev: the device's cosf/sinf of the
                     tilt in radians (what the program's kernels evaluate),
                     which the CPU oracle is given
golden_rtm2d_gpu.npz the two 2D GPU RTM programs, whole runs (forward with
                     the ring saved, mute, backward reconstruction, image,
                     illumination, Poynting gathers, both divided by the
                     illumination; the programs' host Laplacian is not part
                     of it):
                     vti_a: Toa_gpu2DvtiFdRtmAdcigsLaplace.cu RTM() on a
                            64x48 layered VTI model, npml 20, 2 shots
                            (fs 20, ds 25), 400 steps, 30 angles
                     vti_b: the same program reading observed records
                            (readShot), 1 shot
                     tti_a, tti_b: Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu
                            on a 64x48 layered model with a smooth tilt field,
                            2 shots, 400 steps, gathers at every CDP (a) and
                            every third (b: 64 is not a multiple of 3)
                     plus tcos_dev, tsin_dev: the device's cosf/sinf of the
                     tilt, angle_cos_dev: the device's gather weights
                     cosf(ia*pi/180), and angle_thr_dev: the device's
                     angle-bin edges for da = 1 (128 each), for the CPU
                     oracle
golden_rtm3d_gpu.npz the 3D GPU RTM program
                     (Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu main) on a
                     20x16x20 smooth random VTI model, npml 8, SV taper on (as
                     the program runs it), 260 steps:
                     a: 2 shots (dsx 7, dsy 2), gathers at every CDP, 20 angles
                     b: 1 shot, gathers at every second CDP
                     plus angle_cos_dev, angle_thr_dev as above
Of the default builds the RTM fixtures keep the image and the illumination
only (the distance of the two builds).
The VTI programs' records are muted (tt = 100) as the programs write them;
the TTI program's mute call is commented out in its main.  The RTM
programs mute with tt = 20 (VTI) and 30 (TTI).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import refgpu  # noqa: E402
from tests.util import layered_model, random_model_3d  # noqa: E402

CASES3 = {
    "a": dict(dx=10, dy=10, dz=10, npml=8, sv=0, favg=25, ns=2, fsx=10, dsx=2, fsy=8, dsy=1, fsz=3, dsz=0,
              nt=200, dt_us=1000),
    "b": dict(dx=10, dy=10, dz=10, npml=8, sv=1, favg=25, ns=1, fsx=9, dsx=0, fsy=7, dsy=0, fsz=4, dsz=0,
              nt=310, dt_us=1000),
}
CASES2 = {
    "a": dict(dx=10, dz=10, npd=20, sv=0, favg=20, ns=2, fs=30, ds=5, zs=5, nt=300, dt_us=1000),
    "b": dict(dx=10, dz=10, npd=20, sv=1, favg=20, ns=1, fs=28, ds=0, zs=6, nt=300, dt_us=1000),
}


CASEST = {
    "a": dict(dx=10.0, dz=10.0, npml=20, sv=0, favg=20.0, pfac=10.0, ns=2, fs=30, ds=5, zs=5, nt=300, dt=1e-3),
    "b": dict(dx=10.0, dz=10.0, npml=20, sv=1, favg=20.0, pfac=10.0, ns=1, fs=27, ds=0, zs=6, nt=300, dt=1e-3),
}


RTM_VTI = dict(npml=20, nt=400, dx=10.0, dz=10.0, dt=1e-3, favg=20.0, pfac=10.0, ns=2, fs=20, ds=25, zs=2,
               nangle=30, dangle=1)
RTM_TTI = dict(RTM_VTI)


def model_rtm():
    return layered_model(64, 48, seed=11)


def model_rtm_tti():
    v, e, d = layered_model(64, 48, seed=13)
    x, z = np.meshgrid(np.arange(64), np.arange(48), indexing="ij")
    th = (20.0 + 15.0 * np.sin(x / 11.0) * np.cos(z / 9.0)).astype(np.float32)
    return v, e, d, th


def rtm_obs(nx, nt, seed=17):
    """Observed records for the readShot case: a seeded smooth random field."""
    rng = np.random.default_rng(seed)
    r = rng.standard_normal((1, nx, nt)).astype(np.float64)
    for _ in range(6):
        r = (np.roll(r, 1, 2) + 2 * r + np.roll(r, -1, 2)) / 4
    return (0.05 * r).astype(np.float32)


RTM_3D = dict(npml=8, nt=260, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, favg=25.0, pfac=10.0, ns=2, fsx=6, dsx=7, fsy=5,
              dsy=2, zs=2, na=20, da=1, dcdp=1)
CASES_RTM3 = {"a": dict(RTM_3D), "b": dict(RTM_3D, ns=1, dcdp=2)}


def model_rtm3d():
    return random_model_3d(20, 16, 20, seed=23)          # (ny, nx, nz) = (16, 20, 20)


def model_tti():
    v, e, d = layered_model(61, 51, seed=9)
    x, z = np.meshgrid(np.arange(61), np.arange(51), indexing="ij")
    th = (22.5 + 17.5 * np.sin(x / 9.0) * np.cos(z / 13.0)).astype(np.float32)
    return v, e, d, th


def model3():
    return random_model_3d(20, 16, 24, seed=21)          # (ny, nx, nz) = (16, 20, 24)


def model2():
    return layered_model(61, 51, seed=7)


def write_sums(folder):
    with open(os.path.join(folder, "SHA256SUMS"), "w") as f:
        for name in sorted(os.listdir(folder)):
            if name.endswith(".npz"):
                h = hashlib.sha256(open(os.path.join(folder, name), "rb").read()).hexdigest()
                f.write("%s  %s\n" % (h, name))


def main_rtm(out):
    v, e, d = model_rtm()
    # the device's gather weights and bin edges (da = 1), for the CPU oracle
    acos_dev, athr_dev = refgpu.cuda_angle_cos(128), refgpu.cuda_angle_thresholds(1, 128)
    res = dict(v=v, e=e, d=d, angle_cos_dev=acos_dev, angle_thr_dev=athr_dev)
    obs = rtm_obs(v.shape[0], RTM_VTI["nt"])
    res["obs"] = obs
    cases = {"vti_a": dict(RTM_VTI), "vti_b": dict(RTM_VTI, ns=1, fs=31, obs=obs)}
    for name, kw in cases.items():
        for fma in ((True, False) if name == "vti_a" else (False,)):
            mig, ill, ag, shots, ms = refgpu.rtm2d(v, e, d, fma=fma, **kw)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res.update({"mig_" + tag: mig, "ill_" + tag: ill})
            if not fma:
                res.update({"ag_" + tag: ag, "shots_" + tag: shots})
            print("RTM %s: max|mig| %.4g, max|ag| %.4g, %.3f ms/step" % (tag, np.abs(mig).max(), np.abs(ag).max(),
                                                                        ms))
    v, e, d, th = model_rtm_tti()
    ct, st = refgpu.cuda_trig(th)
    res.update(tv=v, te=e, td=d, theta=th, tcos_dev=ct, tsin_dev=st)
    for name, dcdp in (("tti_a", 1), ("tti_b", 3)):
        for fma in ((True, False) if name == "tti_a" else (False,)):
            mig, ill, ag, shots, ms = refgpu.rtm2d_tti(v, e, d, th, dcdp=dcdp, fma=fma, **RTM_TTI)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res.update({"mig_" + tag: mig, "ill_" + tag: ill})
            if not fma:
                res["ag_" + tag] = ag
            if tag == "tti_a_nofma":      # the records do not depend on dcdp
                res["shots_" + tag] = shots
            print("RTM %s: max|mig| %.4g, max|ag| %.4g, %.3f ms/step" % (tag, np.abs(mig).max(), np.abs(ag).max(),
                                                                        ms))
    np.savez_compressed(os.path.join(out, "golden_rtm2d_gpu.npz"), **res)
    v, e, d = model_rtm3d()
    res = dict(v=v, e=e, d=d, angle_cos_dev=acos_dev, angle_thr_dev=athr_dev)
    for name, kw in CASES_RTM3.items():
        for fma in ((True, False) if name == "a" else (False,)):
            mig, ill, ag, shots, ms = refgpu.rtm3d(v, e, d, fma=fma, **kw)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res.update({"mig_" + tag: mig, "ill_" + tag: ill})
            if not fma:
                res["ag_" + tag] = ag
            if tag == "a_nofma":          # b's one shot is a's first
                res["shots_" + tag] = shots
            print("RTM3D %s: max|mig| %.4g, max|ag| %.4g, %.3f ms/step" % (tag, np.abs(mig).max(),
                                                                          np.abs(ag).max(), ms))
    np.savez_compressed(os.path.join(out, "golden_rtm3d_gpu.npz"), **res)


def main(out, which=("fd", "rtm")):
    os.makedirs(out, exist_ok=True)
    if "rtm" in which:
        main_rtm(out)
    if "fd" in which:
        main_fd(out)
    write_sums(out)


def main_fd(out):
    v, e, d = model3()
    res = dict(v=v, e=e, d=d)
    for name, kw in CASES3.items():
        for fma in (True, False):
            shot, snap, ms = refgpu.vti3d(v, e, d, fma=fma, snaps=(kw["nt"] > 300), **kw)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res["shot_" + tag] = shot
            if snap is not None:
                res["snap_" + tag] = snap
            print("3D case %s: max|shot| %.4g, %.3f ms/step" % (tag, np.abs(shot).max(), ms))
    np.savez_compressed(os.path.join(out, "golden_fd3d_gpu.npz"), **res)
    v, e, d = model2()
    res = dict(v=v, e=e, d=d)
    for name, kw in CASES2.items():
        for fma in (True, False):
            shot, snap, ms = refgpu.vti2d(v, e, d, fma=fma, snaps=(name == "a"), **kw)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res["shot_" + tag] = shot
            if snap is not None:
                res["snap_" + tag] = snap
            print("2D case %s: max|shot| %.4g, %.3f ms/step" % (tag, np.abs(shot).max(), ms))
    np.savez_compressed(os.path.join(out, "golden_fd2d_gpu.npz"), **res)
    v, e, d, th = model_tti()
    ct, st = refgpu.cuda_trig(th)     # the device's cos/sin of the tilt, for the CPU oracle
    res = dict(v=v, e=e, d=d, theta=th, cos_dev=ct, sin_dev=st)
    for name, kw in CASEST.items():
        for fma in (True, False):
            shot, snap, ms = refgpu.tti2d(v, e, d, th, fma=fma, snaps=(name == "a"), **kw)
            tag = "%s_%s" % (name, "fma" if fma else "nofma")
            res["shot_" + tag] = shot
            if snap is not None:
                res["snap_" + tag] = snap
            print("TTI case %s: max|shot| %.4g, %.3f ms/step" % (tag, np.abs(shot).max(), ms))
    np.savez_compressed(os.path.join(out, "golden_tti2d_gpu.npz"), **res)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE, tuple(sys.argv[2:]) or ("fd", "rtm"))
