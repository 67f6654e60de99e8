"""ctypes binding of oracle/librefgpu.so: the reference's own GPU programs
GPU_vti3dfd and GPU_vti2dfd (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu,
GPU_vti2dfd_kernels.cu), their device code compiled unmodified into cubins
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
    """Path of the reference program's cubin: name "vti3d" or "vti2d";
    fma=True is the compiler's default build, False contraction off."""
    base = {"vti3d": "gpu_vti3dfd", "vti2d": "gpu_vti2dfd"}[name]
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
