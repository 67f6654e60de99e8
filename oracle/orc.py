"""ctypes bindings of the CPU oracle (liborc32/liborc64) and of the
reference's own CPU code built into oracle/_ref.

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the library.
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

V_CPU, V_GPU, V_MPI, V_GPURTM = 0, 1, 2, 3

_f = np.float32
_P = np.ctypeslib.ndpointer


def build(with_ref=None):
    """Compile the oracle (and the reference pin when its tree exists)."""
    target = [] if with_ref is None else (["all"] if with_ref else ["oracle"])
    subprocess.run(["make", "-s", "-C", HERE] + target, check=True)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


class FD2DDesc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "nz", "npd", "nt", "variant", "sv", "wtype")] + \
               [(n, C.c_float) for n in ("dx", "dz", "dt", "favg", "pfac", "fs", "ds", "zs")] + \
               [("is_", C.c_int), ("rec_iz", C.c_int), ("rec_scale", C.c_float)]


class FD3DDesc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "nz", "npd", "nt", "sv", "wtype", "mode")] + \
               [(n, C.c_float) for n in ("dx", "dy", "dz", "dt", "favg", "pfac")] + \
               [(n, C.c_int) for n in ("fsx", "fsy", "fsz", "dsx", "dsy", "dsz", "is_",
                                       "rec_iz", "rx0", "drx", "nrx", "ry0", "dry", "nry")]


_libs = {}


def lib(prec=32):
    key = "orc%d" % prec
    if key not in _libs:
        path = os.path.join(HERE, "liborc%d.so" % prec)
        if not os.path.exists(path):
            build(with_ref=False)
        L = C.CDLL(path)
        L.orc_fd2d.argtypes = [C.POINTER(FD2DDesc)] + [C.POINTER(C.c_float)] * 5 + [C.c_int]
        L.orc_tti2d.argtypes = [C.POINTER(FD2DDesc)] + [C.POINTER(C.c_float)] * 6 + [C.c_int]
        L.orc_set_tilt_trig.argtypes = [C.POINTER(C.c_float)] * 2
        L.orc_set_angle_cos.argtypes = [C.POINTER(C.c_float)]
        L.orc_set_angle_thresholds.argtypes = [C.POINTER(C.c_float)]
        L.orc_fd3d.argtypes = [C.POINTER(FD3DDesc)] + [C.POINTER(C.c_float)] * 6
        L.orc_tti3d.argtypes = [C.POINTER(FD3DDesc)] + [C.POINTER(C.c_float)] * 8
        L.orc_rtm3d_tti_shot.argtypes = [C.POINTER(FD3DDesc), C.c_int] + [C.POINTER(C.c_float)] * 8
        L.orc_rtm3d_tti_snap_shot.argtypes = [C.POINTER(FD3DDesc), C.c_int, C.c_int] + [C.POINTER(C.c_float)] * 7
        L.orc_rtm2d_mpi_shot.argtypes = [C.c_int] * 4 + [C.c_float] * 5 + [C.c_int] * 5 + \
            [C.POINTER(C.c_float)] * 4 + [C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_laplace2d_adj.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_laplace3d_adj.argtypes = [C.c_int] * 3 + [C.POINTER(C.c_float)] * 2
        L.orc_stack2d.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_mute2d.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_float] * 4 + [C.c_int] * 4 + \
            [C.c_float, C.c_int, C.POINTER(C.c_float)]
        L.orc_mute3d.argtypes = [C.c_int] * 3 + [C.c_float] * 5 + [C.c_int] * 6 + [C.c_float] * 2 + \
            [C.c_int, C.POINTER(C.c_float)]
        L.orc_rtm3d_shot.argtypes = [C.POINTER(FD3DDesc), C.c_int] + [C.POINTER(C.c_float)] * 6 + \
            [C.c_int] * 3 + [C.POINTER(C.c_float)]
        L.orc_adcig3d_illum.argtypes = [C.c_int] * 5 + [C.POINTER(C.c_float)] * 2
        L.orc_rtm3d_snap_shot.argtypes = [C.POINTER(FD3DDesc), C.c_int, C.c_int] + [C.POINTER(C.c_float)] * 5
        L.orc_rtm2d_gpu.argtypes = [C.c_int] * 4 + [C.c_float] * 5 + [C.c_int] * 8 + [C.POINTER(C.c_float)] * 8
        L.orc_rtm2d_tti.argtypes = [C.c_int] * 4 + [C.c_float] * 5 + [C.c_int] * 9 + [C.POINTER(C.c_float)] * 9
        L.orc_image_illum.argtypes = [C.c_long, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        _libs[key] = L
    return _libs[key]


def c32(a):
    return np.ascontiguousarray(a, dtype=_f)


def fd2d(v, e, d, *, npd, nt, dx, dz, dt, favg, pfac, fs, zs, ds=0.0, is_=1, variant=V_CPU,
         sv=0, wtype=1, rec_iz=None, rec_scale=None, snap_every=0, prec=32):
    """2D forward modelling of one shot; returns shot (nx, nt) [and snaps]."""
    v, e, d = c32(v), c32(e), c32(d)
    nx, nz = v.shape
    desc = FD2DDesc(nx=nx, nz=nz, npd=npd, nt=nt, variant=variant, sv=sv, wtype=wtype,
                    dx=dx, dz=dz, dt=dt, favg=favg, pfac=pfac, fs=fs, ds=ds, zs=zs, is_=is_,
                    rec_iz=npd if rec_iz is None else rec_iz,
                    rec_scale=(2.0 if variant == V_CPU else 1.0) if rec_scale is None else rec_scale)
    shot = np.zeros((nx, nt), _f)
    snaps = None
    if snap_every:
        nn = (nx + 2 * npd) * (nz + 2 * npd)
        snaps = np.zeros(((nt - 1) // snap_every + 1, nx + 2 * npd, nz + 2 * npd), _f)
    lib(prec).orc_fd2d(C.byref(desc), _fp(v), _fp(e), _fp(d), _fp(shot), _fp(snaps), snap_every)
    return (shot, snaps) if snap_every else shot


class _TiltTrig:
    """Hand the device's cos/sin of the tilt (nx*nz each) to the oracle for
    one call (orc_set_tilt_trig); None keeps the host's cosf/sinf."""

    def __init__(self, prec, trig):
        self.L = lib(prec)
        self.trig = None if trig is None else (c32(trig[0]), c32(trig[1]))

    def __enter__(self):
        if self.trig is not None:
            self.L.orc_set_tilt_trig(_fp(self.trig[0]), _fp(self.trig[1]))
        return self

    def __exit__(self, *a):
        self.L.orc_set_tilt_trig(None, None)


class _AngleTables:
    """Hand the device's angle-gather weights cosf(ia*pi/180) and bin edges
    (128 entries each; refgpu.cuda_angle_cos, refgpu.cuda_angle_thresholds)
    to the oracle for one call (orc_set_angle_cos, orc_set_angle_thresholds);
    None keeps the host's cosf / acosf."""

    def __init__(self, prec, cos, thr):
        self.L = lib(prec)
        self.cos = None if cos is None else c32(cos)
        self.thr = None if thr is None else c32(thr)
        for t in (self.cos, self.thr):
            if t is not None and t.size < 128:
                raise ValueError("angle tables need 128 entries")

    def __enter__(self):
        if self.cos is not None:
            self.L.orc_set_angle_cos(_fp(self.cos))
        if self.thr is not None:
            self.L.orc_set_angle_thresholds(_fp(self.thr))
        return self

    def __exit__(self, *a):
        self.L.orc_set_angle_cos(None)
        self.L.orc_set_angle_thresholds(None)


def tti2d(v, e, d, theta, *, npd, nt, dx, dz, dt, favg, pfac, fs, zs, ds=0.0, is_=1, sv=0, wtype=1, rec_iz=None,
          snap_every=0, prec=32, trig=None):
    """2D TTI forward modelling (GPU TTI program semantics); theta in degrees.
    trig: (cos, sin) of the tilt as the GPU forms them (refgpu.cuda_trig);
    without it the host's cosf/sinf."""
    v, e, d, theta = c32(v), c32(e), c32(d), c32(theta)
    nx, nz = v.shape
    desc = FD2DDesc(nx=nx, nz=nz, npd=npd, nt=nt, variant=V_GPU, sv=sv, wtype=wtype, dx=dx, dz=dz, dt=dt, favg=favg,
                    pfac=pfac, fs=fs, ds=ds, zs=zs, is_=is_, rec_iz=npd if rec_iz is None else rec_iz, rec_scale=1.0)
    shot = np.zeros((nx, nt), _f)
    snaps = np.zeros(((nt - 1) // snap_every, nx + 2 * npd, nz + 2 * npd), _f) if snap_every else None
    with _TiltTrig(prec, trig):
        lib(prec).orc_tti2d(C.byref(desc), _fp(v), _fp(e), _fp(d), _fp(theta), _fp(shot), _fp(snaps), snap_every)
    return (shot, snaps) if snap_every else shot


def fd3d(v, e, d, *, npd, nt, dx, dy, dz, dt, favg, pfac, fsx, fsy, fsz, dsx=0, dsy=0, dsz=0,
         is_=0, sv=0, wtype=1, mode=0, rec_iz=None, rx0=0, drx=1, nrx=None, ry0=0, dry=1, nry=None,
         final=False, prec=32, theta=None, phi=None):
    """3D forward modelling (GUI GPU semantics); v,e,d shaped (ny, nx, nz).
    With theta and phi (tilt and azimuth in degrees, same shape) the 3D TTI
    step of orc_tti3d instead (premultiplied model, mode ignored)."""
    v, e, d = c32(v), c32(e), c32(d)
    ny, nx, nz = v.shape
    nrx = nx if nrx is None else nrx
    nry = ny if nry is None else nry
    desc = FD3DDesc(nx=nx, ny=ny, nz=nz, npd=npd, nt=nt, sv=sv, wtype=wtype, mode=mode,
                    dx=dx, dy=dy, dz=dz, dt=dt, favg=favg, pfac=pfac, fsx=fsx, fsy=fsy, fsz=fsz,
                    dsx=dsx, dsy=dsy, dsz=dsz, is_=is_, rec_iz=npd if rec_iz is None else rec_iz,
                    rx0=rx0, drx=drx, nrx=nrx, ry0=ry0, dry=dry, nry=nry)
    shot = np.zeros((nry, nrx, nt), _f)
    fp = fq = None
    if final:
        shape = (ny + 2 * npd, nx + 2 * npd, nz + 2 * npd)
        fp, fq = np.zeros(shape, _f), np.zeros(shape, _f)
    if theta is not None:
        th, ph = c32(theta), c32(phi)
        lib(prec).orc_tti3d(C.byref(desc), _fp(v), _fp(e), _fp(d), _fp(th), _fp(ph), _fp(shot), _fp(fp), _fp(fq))
    else:
        lib(prec).orc_fd3d(C.byref(desc), _fp(v), _fp(e), _fp(d), _fp(shot), _fp(fp), _fp(fq))
    return (shot, fp, fq) if final else shot


def rtm3d(v, e, d, *, npd, nt, dx, dy, dz, dt, favg, pfac, fsx, fsy, fsz, dsx=0, dsy=0, dsz=0,
          ns=1, sv=0, wtype=1, mode=0, mute_tt=70, snap_every=0, prec=32, adcig=None, theta=None, phi=None,
          receivers=None, angle_cos=None, angle_thr=None):
    """3D boundary-saving RTM over shots 0..ns-1 (3D GPU RTM program
    semantics; with snap_every > 0 the stored-snapshot method instead);
    v,e,d shaped (ny, nx, nz).  Returns (mig divided by the illumination,
    illum, last shot's muted record (ny, nx, nt); zeros for snap_every > 0)
    [+ the Poynting angle gathers (ny/dcdp, nx/dcdp, na, nz) divided by the
    illumination, when adcig = (na, da, dcdp)].  theta/phi (degrees): the
    3D TTI medium (no angle gathers).  angle_cos, angle_thr: the device's
    gather weights cosf(ia*pi/180) and angle-bin edges for da
    (refgpu.cuda_angle_cos, cuda_angle_thresholds); without them the host's
    cosf and acosf."""
    v, e, d = c32(v), c32(e), c32(d)
    tti = theta is not None
    if tti:
        if adcig is not None:
            raise ValueError("no angle gathers on the TTI medium")
        th, ph = c32(theta), c32(phi)
    ny, nx, nz = v.shape
    mig = np.zeros((ny, nx, nz), _f)
    ill = np.zeros((ny, nx, nz), _f)
    rec = np.zeros((int(receivers[5]), int(receivers[2]), nt) if receivers is not None else (ny, nx, nt), _f)
    na = da = dcdp = 0
    ag = None
    if adcig is not None:
        if snap_every:
            raise ValueError("angle gathers need the boundary method")
        na, da, dcdp = adcig
        ag = np.zeros((ny // dcdp, nx // dcdp, na, nz), _f)
    rx0, drx, nrx, ry0, dry, nry = receivers if receivers is not None else (0, 1, nx, 0, 1, ny)
    for is_ in range(ns):
        desc = FD3DDesc(nx=nx, ny=ny, nz=nz, npd=npd, nt=nt, sv=sv, wtype=wtype, mode=mode,
                        dx=dx, dy=dy, dz=dz, dt=dt, favg=favg, pfac=pfac, fsx=fsx, fsy=fsy, fsz=fsz,
                        dsx=dsx, dsy=dsy, dsz=dsz, is_=is_, rec_iz=npd,
                        rx0=rx0, drx=drx, nrx=nrx, ry0=ry0, dry=dry, nry=nry)
        if tti and snap_every:
            lib(prec).orc_rtm3d_tti_snap_shot(C.byref(desc), mute_tt, snap_every, _fp(v), _fp(e), _fp(d), _fp(th),
                                              _fp(ph), _fp(mig), _fp(ill))
        elif tti:
            lib(prec).orc_rtm3d_tti_shot(C.byref(desc), mute_tt, _fp(v), _fp(e), _fp(d), _fp(th), _fp(ph),
                                         _fp(mig), _fp(ill), _fp(rec))
        elif snap_every:
            lib(prec).orc_rtm3d_snap_shot(C.byref(desc), mute_tt, snap_every, _fp(v), _fp(e), _fp(d), _fp(mig),
                                          _fp(ill))
        else:
            with _AngleTables(prec, angle_cos, angle_thr):
                lib(prec).orc_rtm3d_shot(C.byref(desc), mute_tt, _fp(v), _fp(e), _fp(d), _fp(mig), _fp(ill),
                                         _fp(rec), na, da, dcdp, _fp(ag))
    lib(prec).orc_image_illum(mig.size, _fp(mig), _fp(ill))
    if ag is None:
        return mig, ill, rec
    lib(prec).orc_adcig3d_illum(nx, ny, nz, na, dcdp, _fp(ag), _fp(ill))
    return mig, ill, rec, ag


def rtm2d_mpi_shot(v, e, d, *, npd, nt, dx, dz, dt_ms, favg, pfac, fs_sxd, ds_sxd, zs_sxd, is_, nxs,
                   prec=32, adcig=False):
    """One MPI-semantics RTM shot; returns (mig_is (nxs,nz), offset, p_cal_x
    (nxs,nt)) [+ the shot's angle gathers adcig_is (90,nxs,nz)]."""
    v, e, d = c32(v), c32(e), c32(d)
    nx, nz = v.shape
    mig = np.zeros((nxs, nz), _f)
    pcal = np.zeros((nxs, nt), _f)
    ag = np.zeros((90, nxs, nz), _f) if adcig else None
    off = C.c_int(0)
    lib(prec).orc_rtm2d_mpi_shot(nx, nz, npd, nt, dx, dz, dt_ms, favg, pfac, fs_sxd, ds_sxd, zs_sxd,
                                 is_, nxs, _fp(v), _fp(e), _fp(d), _fp(mig), C.byref(off), _fp(pcal), _fp(ag))
    return (mig, off.value, pcal, ag) if adcig else (mig, off.value, pcal)


def rtm2d_gpu(v, e, d, *, npml, nt, dx, dz, dt, favg, pfac, wtype=1, ns=1, fs=1, ds=0, zs=1, mute_tt=20,
              nangle=70, dangle=1, obs=None, prec=32, angle_cos=None, angle_thr=None):
    """The 2D GPU RTM program; returns (mig/ill (nx,nz), ill, adcigs (nx,nangle,nz),
    muted modelled shots (ns,nx,nt)).  angle_cos, angle_thr: as for rtm3d."""
    v, e, d = c32(v), c32(e), c32(d)
    nx, nz = v.shape
    mig = np.zeros((nx, nz), _f)
    ill = np.zeros((nx, nz), _f)
    ag = np.zeros((nx, nangle, nz), _f)
    shots = np.zeros((ns, nx, nt), _f)
    ob = c32(obs) if obs is not None else None
    with _AngleTables(prec, angle_cos, angle_thr):
        lib(prec).orc_rtm2d_gpu(nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype, ns, fs, ds, zs, mute_tt, nangle,
                                dangle, _fp(v), _fp(e), _fp(d), _fp(ob), _fp(mig), _fp(ill), _fp(ag), _fp(shots))
    return mig, ill, ag, shots


def rtm2d_tti(v, e, d, theta, *, npml, nt, dx, dz, dt, favg, pfac, wtype=1, ns=1, fs=1, ds=0, zs=1, mute_tt=30,
              nangle=65, dangle=1, dcdp=1, obs=None, prec=32, trig=None, angle_cos=None,
              angle_thr=None):
    """The 2D TTI GPU RTM program; theta in degrees.  Returns (mig/ill (nx,nz),
    ill, adcigs (nx//dcdp,nangle,nz), muted modelled shots (ns,nx,nt)).
    trig: as for tti2d; angle_cos, angle_thr: as for rtm3d."""
    v, e, d, theta = c32(v), c32(e), c32(d), c32(theta)
    nx, nz = v.shape
    mig = np.zeros((nx, nz), _f)
    ill = np.zeros((nx, nz), _f)
    ag = np.zeros((nx // dcdp, nangle, nz), _f)
    shots = np.zeros((ns, nx, nt), _f)
    ob = c32(obs) if obs is not None else None
    with _TiltTrig(prec, trig), _AngleTables(prec, angle_cos, angle_thr):
        lib(prec).orc_rtm2d_tti(nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype, ns, fs, ds, zs, mute_tt, nangle,
                                dangle, dcdp, _fp(v), _fp(e), _fp(d), _fp(theta), _fp(ob), _fp(mig), _fp(ill),
                                _fp(ag), _fp(shots))
    return mig, ill, ag, shots


def stack2d(full, mig_is, offset):
    lib().orc_stack2d(full.shape[1], mig_is.shape[0], offset, _fp(c32(mig_is)), _fp(full))


def laplace2d_adj(img):
    img = c32(img)
    out = np.zeros_like(img)
    nx, nz = img.shape
    lib().orc_laplace2d_adj(nz, nx, _fp(img), _fp(out))
    return out


def laplace3d_adj(img):
    img = c32(img)
    out = np.zeros_like(img)
    ny, nx, nz = img.shape
    lib().orc_laplace3d_adj(nz, nx, ny, _fp(img), _fp(out))
    return out


# ------------------------------------------------------------- the reference
REF = os.path.join(HERE, "_ref")


def ref_available():
    return os.path.exists(os.path.join(REF, "librefcpu2d.so"))


def ref_cpu_vti2dfd(v, e, d, *, npd, nt, dx, dz, dt_us, favg, fs, zs, ns=1, ds=0, sv=0):
    """Run the reference's CPU_vti2dfd (unmodified) through its file interface.

    Returns (shots (ns, nx, nt), snaps (k, nnx, nnz)) -- snapshots are the
    padded P of shot 1 every 50 steps, as the reference writes them."""
    L = C.CDLL(os.path.join(REF, "librefcpu2d.so"))
    L.CPU_vti2dfd.restype = None
    v, e, d = c32(v), c32(e), c32(d)
    nx, nz = v.shape
    with tempfile.TemporaryDirectory() as td:
        names = {}
        for k, a in (("v", v), ("e", e), ("d", d)):
            names[k] = os.path.join(td, k + ".bin").encode()
            a.tofile(names[k].decode())
        fshot = os.path.join(td, "shot.bin").encode()
        fsnap = os.path.join(td, "snap.bin").encode()
        L.CPU_vti2dfd(C.c_int(nx), C.c_int(nz), C.c_int(int(dx)), C.c_int(int(dz)), C.c_int(npd), C.c_int(sv),
                      names["v"], names["e"], names["d"], C.c_int(int(favg)), C.c_int(ns), C.c_int(fs),
                      C.c_int(ds), C.c_int(zs), fshot, fsnap, C.c_int(nt), C.c_int(int(dt_us)), C.c_int(1))
        shots = np.fromfile(fshot.decode(), _f).reshape(ns, nx, nt)
        snaps = np.fromfile(fsnap.decode(), _f).reshape(-1, nx + 2 * npd, nz + 2 * npd)
    return shots, snaps


def ref_rtm_mpi_shot(v, e, d, acc, *, npd, nt, dx, dz, dt_ms, favg, pfac, fs_sxd, ds_sxd, zs_sxd, is_, nxs,
                     adcig_acc=None):
    """The reference MPI RTM for one shot; stacks into `acc` (nx,nz) in place
    (and its angle gathers into `adcig_acc` (90,nx,nz) when given)."""
    L = C.CDLL(os.path.join(REF, "librefrtm.so"))
    L.ref_rtm_mpi_shot.argtypes = [C.c_int] * 4 + [C.c_float] * 5 + [C.c_int] * 5 + [C.POINTER(C.c_float)] * 7
    v, e, d = c32(v), c32(e), c32(d)
    nx, nz = v.shape
    mig = np.zeros((nxs, nz), _f)
    pcal = np.zeros((nxs, nt), _f)
    rc = L.ref_rtm_mpi_shot(nx, nz, npd, nt, dx, dz, dt_ms, favg, pfac, fs_sxd, ds_sxd, zs_sxd, is_, nxs,
                            _fp(v), _fp(e), _fp(d), _fp(acc), _fp(mig), _fp(pcal), _fp(adcig_acc))
    if rc:
        raise ValueError("aperture window leaves the model")
    return mig, pcal


def ref_laplace2d_adj(img):
    """laplac2_lop(adj=1) from the reference utility; `out` is pre-zeroed
    here because the utility accumulates into it without clearing."""
    L = C.CDLL(os.path.join(REF, "libreflap.so"))
    L.laplac2_lop.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    img = c32(img)
    out = np.zeros_like(img)
    nx, nz = img.shape
    L.laplac2_lop(1, nz, nx, _fp(img), _fp(out))
    return out


def _rows(a):
    """float** of the rows of a C-contiguous 2D float32 array."""
    return (C.POINTER(C.c_float) * a.shape[0])(*[a[i].ctypes.data_as(C.POINTER(C.c_float)) for i in range(a.shape[0])])


def ref_smooth2float(v, rx, rz):
    """The MPI RTM program's smooth2float on a copy of v (nx, nz)."""
    L = C.CDLL(os.path.join(REF, "librefrtm.so"))
    L.smooth2float.restype = None
    L.smooth2float.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    a = np.array(v, dtype=_f, copy=True, order="C")
    rows = _rows(a)
    L.smooth2float(a.shape[0], rx, a.shape[1], rz, rows)
    return a


def ref_mute_direct(shot, *, dt, favg, dx, dz, fs, ds, zs, is_, vp, epsilon=0.0, tt=190):
    """The direct-wave mute utility's mute_directwave on a copy of shot (nx, nt)."""
    L = C.CDLL(os.path.join(REF, "librefmute.so"))
    L.mute_directwave.restype = None
    L.mute_directwave.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float] + [C.c_int] * 4 + \
        [C.c_float, C.c_float, C.POINTER(C.c_float), C.c_int]
    a = np.array(shot, dtype=_f, copy=True, order="C")
    L.mute_directwave(a.shape[0], a.shape[1], dt, favg, dx, dz, fs, ds, zs, is_, vp, epsilon, _fp(a), tt)
    return a


_SMOOTH3D_RUN = r"""
import ctypes as C, sys
L = C.CDLL(sys.argv[1])
L.ref_smooth3d_main()
C.CDLL(None).fflush(None)   # the program leaves its output stream open
"""


def ref_smooth3d(v):
    """The reference 3D model smoother (utils-3D-smooth-f95/Toa_smooth3D.c) run
    through its file interface on v shaped (70, 70, 70) as (y, x, z): 20
    passes from z = 20.  Runs in a child process (the program works in its
    current directory and leaves its output file open)."""
    import subprocess
    import sys
    v = c32(v)
    assert v.shape == (70, 70, 70)
    with tempfile.TemporaryDirectory() as td:
        v.tofile(os.path.join(td, "vel707070.dat"))
        subprocess.run([sys.executable, "-c", _SMOOTH3D_RUN, os.path.join(REF, "librefsmooth3d.so")], cwd=td,
                       check=True, capture_output=True)
        return np.fromfile(os.path.join(td, "vel707070initial.dat"), _f).reshape(70, 70, 70)
