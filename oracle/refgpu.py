"""ctypes binding of oracle/librefgpu.so: the reference's own GPU programs
GPU_vti3dfd and GPU_vti2dfd (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu,
GPU_vti2dfd_kernels.cu), the 2D TTI forward program
(2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu) and the three GPU
RTM programs (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu,
2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu,
3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu), their device
code compiled unmodified into cubins
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
    """Path of the reference program's cubin: name "vti3d", "vti2d", "tti2d",
    "rtm2d", "rtm2d_tti" or "rtm3d"; fma=True is the compiler's default
    build, False contraction off."""
    base = {"vti3d": "gpu_vti3dfd", "vti2d": "gpu_vti2dfd", "tti2d": "gpu_tti2dfd", "rtm2d": "gpu_rtm2d_vti",
            "rtm2d_tti": "gpu_rtm2d_tti", "rtm3d": "gpu_rtm3d"}[name]
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
        rtm = [C.c_char_p] + [C.c_int] * 4 + [C.c_float] * 5 + [C.c_int] * 4
        L.refgpu_rtm2d.argtypes = rtm + [C.c_int] * 3 + [fp] * 9
        L.refgpu_rtm2d.restype = C.c_int
        L.refgpu_rtm2d_tti.argtypes = rtm + [C.c_int] * 4 + [fp] * 9
        L.refgpu_rtm2d_tti.restype = C.c_int
        L.refgpu_rtm3d.argtypes = [C.c_char_p] + [C.c_int] * 5 + [C.c_float] * 6 + [C.c_int] * 9 + [fp] * 8
        L.refgpu_rtm3d.restype = C.c_int
        L.refgpu_bin_check.argtypes = [C.c_char_p, fp, C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]
        L.refgpu_bin_check.restype = C.c_int
        L.refgpu_bin_thresholds.argtypes = [C.c_char_p, fp, C.c_int, C.c_int]
        L.refgpu_bin_thresholds.restype = C.c_int
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


def rtm2d(v, e, d, *, npml, nt, dx, dz, dt, favg, pfac, wtype=1, ns, fs, ds, zs, nangle, dangle, obs=None,
          fma=True):
    """The 2D GPU RTM program's RTM() on models shaped (nx, nz).  Returns
    (image / illumination before the program's Laplacian, illumination,
    angle gathers / illumination (nx, nangle, nz), muted modelled records
    (ns, nx, nt), ms per step).  Its mute uses tt = 20."""
    v, e, d = (np.ascontiguousarray(a, np.float32) for a in (v, e, d))
    nx, nz = v.shape
    mig, ill = np.zeros((nx, nz), np.float32), np.zeros((nx, nz), np.float32)
    ag = np.zeros((nx, nangle, nz), np.float32)
    shots = np.zeros((ns, nx, nt), np.float32)
    ob = np.ascontiguousarray(obs, np.float32) if obs is not None else None
    ms = C.c_float()
    rc = lib().refgpu_rtm2d(cubin("rtm2d", fma).encode(), nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype, ns, fs,
                            ds, zs, nangle, dangle, _fp(v), _fp(e), _fp(d), _fp(ob), _fp(mig), _fp(ill), _fp(ag),
                            _fp(shots), C.byref(ms))
    if rc:
        raise RuntimeError("reference 2D GPU RTM program run failed")
    return mig, ill, ag, shots, ms.value


def rtm2d_tti(v, e, d, theta, *, npml, nt, dx, dz, dt, favg, pfac, wtype=1, ns, fs, ds, zs, nangle, dangle, dcdp,
              fma=True):
    """The 2D TTI GPU RTM program on models shaped (nx, nz), theta in
    degrees.  Returns (image / illumination before the Laplacian,
    illumination, gathers / illumination (nx//dcdp, nangle, nz), muted
    records (ns, nx, nt), ms per step).  Its mute uses tt = 30."""
    v, e, d, theta = (np.ascontiguousarray(a, np.float32) for a in (v, e, d, theta))
    nx, nz = v.shape
    mig, ill = np.zeros((nx, nz), np.float32), np.zeros((nx, nz), np.float32)
    ag = np.zeros((nx // dcdp, nangle, nz), np.float32)
    shots = np.zeros((ns, nx, nt), np.float32)
    ms = C.c_float()
    rc = lib().refgpu_rtm2d_tti(cubin("rtm2d_tti", fma).encode(), nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype,
                                ns, fs, ds, zs, nangle, dangle, dcdp, _fp(v), _fp(e), _fp(d), _fp(theta), _fp(mig),
                                _fp(ill), _fp(ag), _fp(shots), C.byref(ms))
    if rc:
        raise RuntimeError("reference 2D TTI GPU RTM program run failed")
    return mig, ill, ag, shots, ms.value


def rtm3d(v, e, d, *, npml, nt, dx, dy, dz, dt, favg, pfac, ns, fsx, dsx, fsy, dsy, zs, na, da, dcdp, fma=True):
    """The 3D GPU RTM program on models shaped (ny, nx, nz) (ny <= nx, as the
    program needs).  Returns (image / illumination, illumination, angle
    gathers / illumination (ny//dcdp, nx//dcdp, na, nz), muted records
    (ns, ny, nx, nt), ms per step).  Its mute uses tt = 70."""
    v, e, d = (np.ascontiguousarray(a, np.float32) for a in (v, e, d))
    ny, nx, nz = v.shape
    if ny > nx:
        raise ValueError("the 3D RTM program needs ny <= nx (its y sponge arrays have nnx elements)")
    mig, ill = np.zeros((ny, nx, nz), np.float32), np.zeros((ny, nx, nz), np.float32)
    ag = np.zeros((ny // dcdp, nx // dcdp, na, nz), np.float32)
    shots = np.zeros((ns, ny, nx, nt), np.float32)
    ms = C.c_float()
    rc = lib().refgpu_rtm3d(cubin("rtm3d", fma).encode(), nx, ny, nz, npml, nt, dx, dy, dz, dt, favg, pfac, ns, fsx,
                            dsx, fsy, dsy, zs, na, da, dcdp, _fp(v), _fp(e), _fp(d), _fp(mig), _fp(ill), _fp(ag),
                            _fp(shots), C.byref(ms))
    if rc:
        raise RuntimeError("reference 3D GPU RTM program run failed")
    return mig, ill, ag, shots, ms.value


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


PI_GPU = 3.141592653          # the GPU programs' pi


def angle_args(n=128):
    """The arguments of the GPU RTM programs' gather weight cosf(ia*pi/180):
    the double ia*pi/180 rounded to float, ia < n."""
    return np.array([ia * PI_GPU / 180.0 for ia in range(n)], np.float64).astype(np.float32)


def cuda_angle_cos(n=128):
    """The device's cosf(ia*pi/180), ia < n: the angle-gather weights the GPU
    RTM programs' Poynting_Adcigs kernels use (oracle/ref_harness/trig.cu).
    Needs a GPU."""
    th = np.ascontiguousarray(angle_args(n))
    c, s = np.empty_like(th), np.empty_like(th)
    path = os.path.join(HERE, "trig.cubin")
    if not os.path.exists(path):
        orc.build(with_ref=False)
    if lib().refgpu_cuda_trig(path.encode(), _fp(th), _fp(c), _fp(s), th.size):
        raise RuntimeError("device trig failed")
    return c


def _host_acosf():
    libm = C.CDLL("libm.so.6")
    libm.acosf.restype = C.c_float
    libm.acosf.argtypes = [C.c_float]
    return libm.acosf


def host_bin(a, da, acosf=None):
    """The programs' Poynting bin (int)((float)(0.5*acosf(a)*180/pi)/(da*1.0))
    with the host's acosf (the one the CPU oracle calls)."""
    acosf = acosf or _host_acosf()
    deg = np.float32(0.5 * acosf(float(a)) * 180.0 / PI_GPU)
    return int(float(deg) / (da * 1.0))


def host_bin_thresholds(na, da):
    """thr[k] = largest float a in [-1, 1] whose host-acosf bin is >= k+1,
    -2 where none is, k < na (a binary search over the ordered floats)."""
    acosf = _host_acosf()

    def key(f):
        b = int(np.float32(f).view(np.uint32))
        return (~b & 0xffffffff) if b & 0x80000000 else (b | 0x80000000)

    def flt(k):
        b = (k & 0x7fffffff) if k & 0x80000000 else (~k & 0xffffffff)
        return float(np.uint32(b).view(np.float32))

    thr = np.full(na, -2.0, np.float32)
    for k in range(1, na + 1):
        if host_bin(-1.0, da, acosf) < k:
            continue
        lo, hi = key(-1.0), key(1.0)
        while lo < hi:
            m = lo + (hi - lo + 1) // 2
            if host_bin(flt(m), da, acosf) >= k:
                lo = m
            else:
                hi = m - 1
        thr[k - 1] = flt(lo)
    return thr


def cuda_angle_thresholds(da, na=128):
    """thr[k] = largest float a in [-1, 1] whose Poynting bin by the
    device's acosf is >= k+1, -2 where none is, k < na: the bins the GPU RTM
    programs' kernels form, as thresholds the CPU oracle can count
    (oracle/ref_harness/trig.cu).  Needs a GPU."""
    thr = np.zeros(na, np.float32)
    path = os.path.join(HERE, "trig.cubin")
    if not os.path.exists(path):
        orc.build(with_ref=False)
    if lib().refgpu_bin_thresholds(path.encode(), _fp(thr), na, da):
        raise RuntimeError("device bin thresholds failed")
    return thr


def cuda_angle_tables(da):
    """The device's angle-gather weights and bin edges for angle step da, as
    the oracle's angle_cos / angle_thr arguments.  Needs a GPU."""
    return dict(angle_cos=cuda_angle_cos(128), angle_thr=cuda_angle_thresholds(da, 128))


def bin_check(na, da, thr=None):
    """Number of floats a in [-1, 1] whose Poynting bin by the device's
    acosf (capped at na) differs from the count of thresholds thr[0..na) at
    or above a; thr defaults to the host-acosf thresholds.  Needs a GPU."""
    thr = np.ascontiguousarray(host_bin_thresholds(na, da) if thr is None else np.asarray(thr, np.float32)[:na])
    bad = C.c_ulonglong(0)
    path = os.path.join(HERE, "trig.cubin")
    if not os.path.exists(path):
        orc.build(with_ref=False)
    if lib().refgpu_bin_check(path.encode(), _fp(thr), na, da, C.byref(bad)):
        raise RuntimeError("device bin check failed")
    return bad.value
