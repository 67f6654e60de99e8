"""Generate the golden fixtures of the reference's own GPU programs by
running them on a GPU: their device code compiled unmodified into cubins
(oracle/Makefile, from the reference tree) and driven by
oracle/ref_harness/refgpu.c through the CUDA driver API.

  python tests/golden/make_golden_refgpu.py [OUTDIR]      (needs a GPU)

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
The VTI programs' records are muted (tt = 100) as the programs write them;
the TTI program's mute call is commented out in its main.
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


def main(out):
    os.makedirs(out, exist_ok=True)
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
    write_sums(out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
