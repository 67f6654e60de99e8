"""ctypes binding of oracle/librefgpu.so: the reference's own GPU programs
GPU_vti3dfd and GPU_vti2dfd (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu,
GPU_vti2dfd_kernels.cu) and the 2D TTI forward program
(2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu), their device code
compiled unmodified into cubins
under oracle/_ref/ by oracle/Makefile and driven by
oracle/ref_harness/refgpu.c, which repeats each program's host side with
arrays instead of files.

Test infrastructure only: the golden-fixture script and the parity tests
use it as the checker; the library never loads it.  Needs a GPU and the
cubins (built where the reference tree is, carried as files).
"""
import ctypes as C
import os

import numpy as np

from . import orc

HERE = os.path.dirname(os.path.abspath(__file__))
REFDIR = os.path.join(HERE, "_ref")

_lib = None


def cubin(name, fma=True):
    """Path of the reference program's cubin: name "vti3d", "vti2d" or "tti2d";
    fma=True is the compiler's default build, False contraction off."""
    base = {"vti3d": "gpu_vti3dfd", "vti2d": "gpu_vti2dfd", "tti2d": "gpu_tti2dfd"}[name]
    return os.path.join(REFDIR, base + ("" if fma else "_nofma") + ".cubin")


def available(name="vti3d"):
    return os.path.exists(cubin(name, True)) and os.path.exists(cubin(name, False))


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "librefgpu.so")
        if not os.path.exists(path):
            orc.build(with_ref=False)
        L = C.CDLL(path)
        fp = C.POINTER(C.c_float)
        L.refgpu_vti3d.argtypes = [C.c_char_p] + [C.c_int] * 8 + [fp] * 3 + [C.c_int] * 10 + [fp] * 3
        L.refgpu_vti3d.restype = C.c_int
        L.refgpu_vti2d.argtypes = [C.c_char_p] + [C.c_int] * 6 + [fp] * 3 + [C.c_int] * 7 + [fp] * 3
        L.refgpu_vti2d.restype = C.c_int
        L.refgpu_tti2d.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int] + \
            [fp] * 4 + [C.c_float, C.c_float] + [C.c_int] * 5 + [C.c_float] + [fp] * 3
        L.refgpu_tti2d.restype = C.c_int
        L.refgpu_cuda_trig.argtypes = [C.c_char_p, fp, fp, fp, C.c_long]
        L.refgpu_cuda_trig.restype = C.c_int
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def vti3d(v, e, d, *, dx, dy, dz, npml, sv, favg, ns, fsx, dsx, fsy, dsy, fsz, dsz, nt, dt_us, fma=True,
          snaps=False):
    """GPU_vti3dfd on models shaped (ny, nx, nz) (the model files' order).
    Returns (shots (ns, ny, nx, nt), snapshots or None, ms per step)."""
    v, e, d = (np.ascontiguousarray(a, np.float32) for a in (v, e, d))
    ny, nx, nz = v.shape
    if ny > nx:
        raise ValueError("GPU_vti3dfd needs ny <= nx (its y sponge arrays have nnx elements)")
    shot = np.zeros((ns, ny, nx, nt), np.float32)
    snap = np.zeros(((nt - 1) // 300, ny, nx, nz), np.float32) if snaps else None
    ms = C.c_float()
    rc = lib().refgpu_vti3d(cubin("vti3d", fma).encode(), nx, ny, nz, dx, dy, dz, npml, sv, _fp(v), _fp(e), _fp(d),
                            favg, ns, fsx, dsx, fsy, dsy, fsz, dsz, nt, dt_us, _fp(shot), _fp(snap), C.byref(ms))
    if rc:
        raise RuntimeError("reference GPU_vti3dfd run failed")
    return shot, snap, ms.value


def vti2d(v, e, d, *, dx, dz, npd, sv, favg, ns, fs, ds, zs, nt, dt_us, fma=True, snaps=False):
    """GPU_vti2dfd on models shaped (nx, nz).  Returns (shots (ns, nx, nt),
    padded P snapshots of shot 1 every 50 steps or None, ms per step)."""
    v, e, d = (np.ascontiguousarray(a, np.float32) for a in (v, e, d))
    nx, nz = v.shape
    shot = np.zeros((ns, nx, nt), np.float32)
    snap = np.zeros(((nt - 1) // 50 + 1, nx + 2 * npd, nz + 2 * npd), np.float32) if snaps else None
    ms = C.c_float()
    rc = lib().refgpu_vti2d(cubin("vti2d", fma).encode(), nx, nz, dx, dz, npd, sv, _fp(v), _fp(e), _fp(d), favg, ns,
                            fs, ds, zs, nt, dt_us, _fp(shot), _fp(snap), C.byref(ms))
    if rc:
        raise RuntimeError("reference GPU_vti2dfd run failed")
    return shot, snap, ms.value


def tti2d(v, e, d, theta, *, dx, dz, npml, sv, favg, pfac, ns, fs, ds, zs, nt, dt, fma=True, snaps=False):
    """The 2D TTI forward program on models shaped (nx, nz), theta in
    degrees.  Returns (shots (ns, nx, nt), padded P snapshots of shot 1 at
    it = 100, 200, ... or None, ms per step)."""
    v, e, d, theta = (np.ascontiguousarray(a, np.float32) for a in (v, e, d, theta))
    nx, nz = v.shape
    shot = np.zeros((ns, nx, nt), np.float32)
    snap = np.zeros(((nt - 1) // 100, nx + 2 * npml, nz + 2 * npml), np.float32) if snaps else None
    ms = C.c_float()
    rc = lib().refgpu_tti2d(cubin("tti2d", fma).encode(), nx, nz, dx, dz, npml, sv, _fp(v), _fp(e), _fp(d),
                            _fp(theta), favg, pfac, ns, fs, ds, zs, nt, dt, _fp(shot), _fp(snap), C.byref(ms))
    if rc:
        raise RuntimeError("reference 2D TTI program run failed")
    return shot, snap, ms.value


def tilt_radians(theta_deg):
    """The 2D TTI programs' tilt in radians: theta *= pi/180 of a float with
    pi = 3.141592653 (read_file, Toa_gpu_2dtti_fd_1orderfunction.cu:235)."""
    return (np.asarray(theta_deg, np.float32).astype(np.float64) * (3.141592653 / 180.0)).astype(np.float32)


def cuda_trig(theta_deg):
    """(cos, sin) of the tilt as the GPU TTI programs form them: the device's
    cosf/sinf of the radians above (oracle/ref_harness/trig.cu).  Needs a GPU."""
    th = np.ascontiguousarray(tilt_radians(theta_deg))
    c, s = np.empty_like(th), np.empty_like(th)
    path = os.path.join(HERE, "trig.cubin")
    if not os.path.exists(path):
        orc.build(with_ref=False)
    if lib().refgpu_cuda_trig(path.encode(), _fp(th), _fp(c), _fp(s), th.size):
        raise RuntimeError("device trig failed")
    return c, s
