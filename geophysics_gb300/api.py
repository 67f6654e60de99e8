"""Array-level and file-level entry points over libgeofd.

Inputs may be numpy arrays (host memory) or torch CUDA tensors (device
memory, run on torch's current stream); outputs come back as the same kind.
Array layouts are the reference's: 2D models (nx, nz), 3D models (ny, nx, nz),
shot records (ntraces, nt).
"""
import ctypes as C

import numpy as np

from ._lib import (FD2DDesc, FD3DDesc, GEO_MEM_DEVICE, GEO_MEM_HOST, GEO_MODE_EXACT, GEO_MODE_FAST,
                   GEO_RTM_BOUNDARY, GEO_RTM_CHECKPOINT, GEO_RTM_LEARNED, GEO_RTM_SNAPSHOT, GEO_VARIANT_CPU, GEO_VARIANT_GPU,
                   GEO_VARIANT_MPI, RTM2DDesc, RTM2DGpuDesc, RTM3DDesc, check, lib)

_VARIANTS = {"cpu": GEO_VARIANT_CPU, "gpu": GEO_VARIANT_GPU, "mpi": GEO_VARIANT_MPI}
_MODES = {"exact": GEO_MODE_EXACT, "fast": GEO_MODE_FAST}


def _torch():
    try:
        import torch
        return torch
    except ImportError:  # pragma: no cover - torch is part of the image
        return None


def _is_dev(a):
    t = _torch()
    return t is not None and isinstance(a, t.Tensor) and a.is_cuda


class _Bufs:
    """Pointer marshalling for one call: all arrays host or all device."""

    def __init__(self, *arrays):
        devs = {_is_dev(a) for a in arrays if a is not None}
        if len(devs) > 1:
            raise ValueError("mix of host and device arrays")
        self.dev = devs.pop() if devs else False
        self.keep = []

    @property
    def mem(self):
        return GEO_MEM_DEVICE if self.dev else GEO_MEM_HOST

    def stream(self):
        if not self.dev:
            return None
        return C.c_void_p(_torch().cuda.current_stream().cuda_stream)

    def inp(self, a):
        if a is None:
            return None
        if self.dev:
            t = _torch()
            a = a.to(t.float32).contiguous()
            self.keep.append(a)
            return C.c_void_p(a.data_ptr())
        a = np.ascontiguousarray(a, dtype=np.float32)
        self.keep.append(a)
        return C.c_void_p(a.ctypes.data)

    def out(self, shape, like=None):
        if self.dev:
            t = _torch()
            o = t.empty(shape, dtype=t.float32, device=like.device if like is not None else "cuda")
            return o, C.c_void_p(o.data_ptr())
        o = np.empty(shape, np.float32)
        return o, C.c_void_p(o.ctypes.data)


def version():
    return lib().geo_version().decode()


def launch_count():
    """Kernel launches issued by the library since it was loaded."""
    return int(lib().geo_launch_count())


def fd2d_shot(v, e, d, *, npd, nt, dx, dz, dt, favg, fs, zs, pfac=10.0, ds=0.0, is_=1, variant="cpu", sv=0,
              wtype=1, rec_iz=None, rec_scale=None, mute_tt=0, snap_every=0):
    """One 2D shot; returns the record (nx, nt) [and padded P snapshots].

    variant: "cpu" (CPU_vti2dfd), "gpu" (GPU_vti2dfd) or "mpi" (the MPI
    RTM program's forward modelling)."""
    b = _Bufs(v, e, d)
    nx, nz = v.shape
    var = _VARIANTS[variant] if isinstance(variant, str) else int(variant)
    desc = FD2DDesc(nx=nx, nz=nz, npd=npd, nt=nt, dx=dx, dz=dz, dt=dt, favg=favg, pfac=pfac, wtype=wtype,
                    fs=fs, ds=ds, zs=zs, is_=is_, variant=var, sv=sv,
                    rec_iz=npd if rec_iz is None else rec_iz,
                    rec_scale=(2.0 if var == GEO_VARIANT_CPU else 1.0) if rec_scale is None else rec_scale,
                    mute_tt=mute_tt)
    pv, pe, pd = b.inp(v), b.inp(e), b.inp(d)
    shot, ps = b.out((nx, nt), v)
    snaps, psn = (None, None)
    if snap_every:
        snaps, psn = b.out(((nt - 1) // snap_every + 1, nx + 2 * npd, nz + 2 * npd), v)
    check(lib().geo_fd2d_shot(C.byref(desc), pv, pe, pd, ps, psn, snap_every, b.mem, b.stream()), "geo_fd2d_shot")
    return (shot, snaps) if snap_every else shot


def tti2d_shot(v, e, d, theta, *, npd, nt, dx, dz, dt, favg, fs, zs, pfac=10.0, ds=0.0, is_=1, sv=0, wtype=1,
               rec_iz=None, snap_every=0):
    """One 2D TTI shot (the GPU TTI program's semantics); theta in degrees,
    all arrays (nx, nz).  Returns the record (nx, nt) [and padded P
    snapshots at it = snap_every, 2*snap_every, ...]."""
    b = _Bufs(v, e, d, theta)
    nx, nz = v.shape
    desc = FD2DDesc(nx=nx, nz=nz, npd=npd, nt=nt, dx=dx, dz=dz, dt=dt, favg=favg, pfac=pfac, wtype=wtype,
                    fs=fs, ds=ds, zs=zs, is_=is_, variant=GEO_VARIANT_GPU, sv=sv,
                    rec_iz=npd if rec_iz is None else rec_iz, rec_scale=1.0, mute_tt=0)
    pv, pe, pd, pt = b.inp(v), b.inp(e), b.inp(d), b.inp(theta)
    shot, ps = b.out((nx, nt), v)
    snaps, psn = (None, None)
    if snap_every:
        snaps, psn = b.out(((nt - 1) // snap_every, nx + 2 * npd, nz + 2 * npd), v)
    check(lib().geo_tti2d_shot(C.byref(desc), pv, pe, pd, pt, ps, psn, snap_every, b.mem, b.stream()),
          "geo_tti2d_shot")
    return (shot, snaps) if snap_every else shot


class FD3DPlan:
    """Device state for repeated 3D shots on one grid (geo_fd3d_plan_*)."""

    def __init__(self, *, nx, ny, nz, npd, nt, dx, dy, dz, dt, favg, fsx, fsy, fsz, pfac=10.0, wtype=1, sv=0,
                 mode="fast", dsx=0, dsy=0, dsz=0, rec_iz=None, rx0=0, drx=1, nrx=None, ry0=0, dry=1, nry=None,
                 mute_tt=0):
        self.desc = FD3DDesc(nx=nx, ny=ny, nz=nz, npd=npd, nt=nt, dx=dx, dy=dy, dz=dz, dt=dt, favg=favg, pfac=pfac,
                             wtype=wtype, sv=sv, mode=_MODES[mode] if isinstance(mode, str) else int(mode),
                             fsx=fsx, fsy=fsy, fsz=fsz, dsx=dsx, dsy=dsy, dsz=dsz,
                             rec_iz=npd if rec_iz is None else rec_iz, rx0=rx0, drx=drx,
                             nrx=nx if nrx is None else nrx, ry0=ry0, dry=dry, nry=ny if nry is None else nry,
                             mute_tt=mute_tt)
        self._p = C.c_void_p()
        check(lib().geo_fd3d_plan_create(C.byref(self._p), C.byref(self.desc)), "geo_fd3d_plan_create")
        self.padded = (ny + 2 * npd, nx + 2 * npd, nz + 2 * npd)

    def set_model(self, v, e, d):
        b = _Bufs(v, e, d)
        check(lib().geo_fd3d_set_model(self._p, b.inp(v), b.inp(e), b.inp(d), b.mem, b.stream()),
              "geo_fd3d_set_model")

    def set_tilt(self, theta, phi):
        """3D TTI medium: tilt from the vertical and azimuth in degrees,
        shaped like the model and smooth in space (geo_fd3d_set_tilt); the
        plan must use mode "fast"."""
        b = _Bufs(theta, phi)
        check(lib().geo_fd3d_set_tilt(self._p, b.inp(theta), b.inp(phi), b.mem, b.stream()), "geo_fd3d_set_tilt")

    def run_shot(self, is_=0, device=None, out=None):
        """Shot `is_` (0-based); returns (nry, nrx, nt), on the GPU if device;
        `out` (host float32 array of that shape, e.g. a view of pinned
        memory) receives the record instead of a new array."""
        D = self.desc
        shape = (D.nry, D.nrx, D.nt)
        if out is not None:
            if out.shape != shape or out.dtype != np.float32 or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float32 array of shape %s" % (shape,))
            check(lib().geo_fd3d_run_shot(self._p, is_, C.c_void_p(out.ctypes.data), GEO_MEM_HOST, None),
                  "geo_fd3d_run_shot")
            return out
        if device:
            t = _torch()
            out = t.empty(shape, dtype=t.float32, device=device)
            check(lib().geo_fd3d_run_shot(self._p, is_, C.c_void_p(out.data_ptr()), GEO_MEM_DEVICE,
                                          C.c_void_p(t.cuda.current_stream().cuda_stream)), "geo_fd3d_run_shot")
            return out
        out = np.empty(shape, np.float32)
        check(lib().geo_fd3d_run_shot(self._p, is_, C.c_void_p(out.ctypes.data), GEO_MEM_HOST, None),
              "geo_fd3d_run_shot")
        return out

    def time_steps(self, n, stream=None):
        """Device time (ms) of n bare time steps on the current state."""
        ms = C.c_float()
        check(lib().geo_fd3d_time_steps(self._p, n, C.byref(ms), stream), "geo_fd3d_time_steps")
        return ms.value

    def fields(self):
        P = np.empty(self.padded, np.float32)
        Q = np.empty(self.padded, np.float32)
        check(lib().geo_fd3d_get_fields(self._p, C.c_void_p(P.ctypes.data), C.c_void_p(Q.ctypes.data),
                                        GEO_MEM_HOST, None), "geo_fd3d_get_fields")
        return P, Q

    def close(self):
        if self._p:
            lib().geo_fd3d_plan_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fd3d_shot(v, e, d, is_=0, theta=None, phi=None, **kw):
    """One-call 3D shot (create plan, set model, run, destroy); with theta
    and phi (degrees) on the 3D TTI medium."""
    ny, nx, nz = v.shape
    plan = FD3DPlan(nx=nx, ny=ny, nz=nz, **kw)
    try:
        plan.set_model(v, e, d)
        if theta is not None:
            plan.set_tilt(theta, phi)
        return plan.run_shot(is_, device=v.device if _is_dev(v) else None)
    finally:
        plan.close()


_RTM = {"boundary": GEO_RTM_BOUNDARY, "snapshot": GEO_RTM_SNAPSHOT, "learned": GEO_RTM_LEARNED,
        "checkpoint": GEO_RTM_CHECKPOINT}


def rtm3d(v, e, d, *, npd, nt, dx, dy, dz, dt, favg, fsx, fsy, fsz, ns=1, dsx=0, dsy=0, dsz=0, mute_tt=70,
          pfac=10.0, wtype=1, sv=0, mode="fast", laplace=True, illum=False, method="boundary", snap_every=4,
          codec=None, adcig=None, theta=None, phi=None, ckpt_every=0, receivers=None):
    """3D RTM over shots 0..ns-1; v,e,d shaped (ny, nx, nz); theta, phi
    (degrees, same shape): the 3D TTI medium (mode "fast", no gathers).

    method "boundary": the 3D GPU RTM program's boundary-saving recompute;
    "snapshot": source P kept every snap_every steps (fp32);
    "learned": the same snapshots through `codec` (a trained Codec);
    "checkpoint": exact recompute from full wavefields saved every
    ckpt_every steps (0: the interval minimising states plus segment
    snapshots); same image as "snapshot" in bounded memory.
    adcig = (na, da, dcdp) (boundary method): also the Poynting angle
    gathers, shaped (ny//dcdp, nx//dcdp, na, nz), illumination-divided.
    receivers = (rx0, drx, nrx, ry0, dry, nry): only that surface grid
    records and takes the record back (default: every surface node, the
    program's receivers).
    Returns the illumination-divided image, then the Laplacian-filtered image
    if `laplace`, then the illumination if `illum`, then the gathers."""
    b = _Bufs(v, e, d, theta, phi)
    ny, nx, nz = v.shape
    fd = FD3DDesc(nx=nx, ny=ny, nz=nz, npd=npd, nt=nt, dx=dx, dy=dy, dz=dz, dt=dt, favg=favg, pfac=pfac,
                  wtype=wtype, sv=sv, mode=_MODES[mode] if isinstance(mode, str) else int(mode),
                  fsx=fsx, fsy=fsy, fsz=fsz, dsx=dsx, dsy=dsy, dsz=dsz, rec_iz=npd, rx0=0, drx=1, nrx=nx,
                  ry0=0, dry=1, nry=ny, mute_tt=0)
    if receivers is not None:
        fd.rx0, fd.drx, fd.nrx, fd.ry0, fd.dry, fd.nry = (int(x) for x in receivers)
    na, da, dcdp = adcig if adcig is not None else (0, 0, 0)
    desc = RTM3DDesc(fd=fd, ns=ns, mute_tt=mute_tt, method=_RTM[method] if isinstance(method, str) else int(method),
                     snap_every=snap_every, ae=codec._p if codec is not None else None, na=na, da=da, dcdp=dcdp,
                     ckpt_every=ckpt_every, rec_grid=1 if receivers is not None else 0)
    pv, pe, pd = b.inp(v), b.inp(e), b.inp(d)
    if theta is not None:
        desc.theta, desc.phi = b.inp(theta), b.inp(phi)
    mig, pm = b.out((ny, nx, nz), v)
    lap, pl = b.out((ny, nx, nz), v) if laplace else (None, None)
    ill, pi = b.out((ny, nx, nz), v) if illum else (None, None)
    ag, pa = b.out((ny // dcdp, nx // dcdp, na, nz), v) if adcig is not None else (None, None)
    check(lib().geo_rtm3d_adcig(C.byref(desc), pv, pe, pd, pm, pl, pi, pa, b.mem, b.stream()), "geo_rtm3d_adcig")
    out = [mig] + ([lap] if laplace else []) + ([ill] if illum else []) + ([ag] if adcig is not None else [])
    return out[0] if len(out) == 1 else tuple(out)


def rtm2d_gpu(v, e, d, *, npml, nt, dx, dz, dt, favg, ns=1, fs=1, ds=0, zs=1, pfac=10.0, wtype=1, mute_tt=20,
              nangle=70, dangle=1, obs=None):
    """2D RTM with the 2D GPU RTM program's semantics (full-model shots,
    ring saving, Poynting angle gathers).  Returns a dict: "mig_lap" (nx,nz),
    "illum", "adcigs" (nx,nangle,nz), "stk_lap", "shots" (ns,nx,nt)."""
    b = _Bufs(v, e, d, obs)
    nx, nz = v.shape
    desc = RTM2DGpuDesc(nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dz, dt=dt, favg=favg, pfac=pfac, wtype=wtype,
                        ns=ns, fs=fs, ds=ds, zs=zs, mute_tt=mute_tt, nangle=nangle, dangle=dangle)
    pv, pe, pd, po = b.inp(v), b.inp(e), b.inp(d), b.inp(obs)
    out = {}
    ptrs = []
    for name, shape in (("mig_lap", (nx, nz)), ("illum", (nx, nz)), ("adcigs", (nx, nangle, nz)),
                        ("stk_lap", (nx, nz)), ("shots", (ns, nx, nt))):
        out[name], p = b.out(shape, v)
        ptrs.append(p)
    check(lib().geo_rtm2d_gpu(C.byref(desc), pv, pe, pd, po, *ptrs, b.mem, b.stream()), "geo_rtm2d_gpu")
    return out


def rtm2d_tti(v, e, d, theta, *, npml, nt, dx, dz, dt, favg, ns=1, fs=1, ds=0, zs=1, pfac=10.0, wtype=1,
              mute_tt=30, nangle=65, dangle=1, dcdp=1, obs=None):
    """2D TTI RTM with the 2D TTI GPU RTM program's semantics; theta is the
    tilt in degrees.  Returns a dict: "mig_lap" (nx,nz), "illum", "adcigs"
    (nx//dcdp, nangle, nz), "shots" (ns,nx,nt)."""
    b = _Bufs(v, e, d, theta, obs)
    nx, nz = v.shape
    desc = RTM2DGpuDesc(nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dz, dt=dt, favg=favg, pfac=pfac, wtype=wtype,
                        ns=ns, fs=fs, ds=ds, zs=zs, mute_tt=mute_tt, nangle=nangle, dangle=dangle, dcdp=dcdp)
    pv, pe, pd, pt, po = b.inp(v), b.inp(e), b.inp(d), b.inp(theta), b.inp(obs)
    out = {}
    ptrs = []
    for name, shape in (("mig_lap", (nx, nz)), ("illum", (nx, nz)), ("adcigs", (nx // dcdp, nangle, nz)),
                        ("shots", (ns, nx, nt))):
        out[name], p = b.out(shape, v)
        ptrs.append(p)
    check(lib().geo_rtm2d_tti(C.byref(desc), pv, pe, pd, pt, po, *ptrs, b.mem, b.stream()), "geo_rtm2d_tti")
    return out


def _inplace_copy(b, a):
    """A float32 contiguous copy of `a` on the same side, and its pointer."""
    if b.dev:
        c = a.to(_torch().float32).contiguous().clone()
        return c, C.c_void_p(c.data_ptr())
    c = np.array(a, dtype=np.float32, order="C", copy=True)
    return c, C.c_void_p(c.ctypes.data)


def smooth2d(v, rx, rz):
    """smooth2float of the MPI RTM program on v (nx, nz): rx 3-point passes
    along x, then rz along z.  Returns a new array."""
    b = _Bufs(v)
    nx, nz = v.shape
    out, p = _inplace_copy(b, v)
    check(lib().geo_smooth2d(nx, rx, nz, rz, p, b.mem, b.stream()), "geo_smooth2d")
    return out


def adcig_smooth_stack(adcig, passes=10):
    """The MPI RTM program's smoothed angle gathers and their stack: adcig
    shaped (na, nx, nz) as rtm2d_batch(adcig=True) returns it.  Returns
    (smoothed gathers, stack (nx, nz))."""
    b = _Bufs(adcig)
    na, nx, nz = adcig.shape
    g, pg = _inplace_copy(b, adcig)
    stk, ps = b.out((nx, nz), adcig)
    check(lib().geo_adcig_smooth_stack(nx, nz, na, passes, pg, ps, b.mem, b.stream()), "geo_adcig_smooth_stack")
    return g, stk


def mute_direct(shot, *, dt, favg, dx, dz, fs, ds, zs, is_, vp, epsilon=0.0, tt=190):
    """The direct-wave mute utility on one trace-major record shot (nx, nt);
    returns a new array."""
    b = _Bufs(shot)
    nx, nt = shot.shape
    out, p = _inplace_copy(b, shot)
    check(lib().geo_mute_direct(nx, nt, dt, favg, dx, dz, fs, ds, zs, is_, vp, epsilon, tt, p, b.mem, b.stream()),
          "geo_mute_direct")
    return out


def smooth_model3d(v, passes=20, mmz=20):
    """The 3D model smoother utility on v shaped (ny, nx, nz); returns a new
    array (host sweep, see geo_smooth_model3d)."""
    b = _Bufs(v)
    ny, nx, nz = v.shape
    out, p = _inplace_copy(b, v)
    check(lib().geo_smooth_model3d(nx, ny, nz, passes, mmz, p, b.mem, b.stream()), "geo_smooth_model3d")
    return out


def smooth_model2d(v, passes=100, z0=31):
    """The 2D model smoother utility on v shaped (nx, nz), rows z >= z0;
    returns a new array."""
    b = _Bufs(v)
    nx, nz = v.shape
    out, p = _inplace_copy(b, v)
    check(lib().geo_smooth_model2d(nx, nz, z0, passes, p, b.mem, b.stream()), "geo_smooth_model2d")
    return out


def morton_order():
    """perm[m] = natural index (z + 16*x + 256*y) of Morton index m of a
    16^3 block (bit 3l = z bit l, 3l+1 = x bit l, 3l+2 = y bit l)."""
    m = np.arange(4096)
    z = sum(((m >> (3 * l)) & 1) << l for l in range(4))
    x = sum(((m >> (3 * l + 1)) & 1) << l for l in range(4))
    y = sum(((m >> (3 * l + 2)) & 1) << l for l in range(4))
    return z + 16 * x + 256 * y


class Codec:
    """The learned snapshot codec (geo_ae_*): a 4-level convolutional
    autoencoder over 16^3 blocks trained on the GPU."""

    def __init__(self, seed=1):
        self._p = C.c_void_p()
        check(lib().geo_ae_create(C.byref(self._p), C.c_ulonglong(seed)), "geo_ae_create")

    @staticmethod
    def num_params():
        return int(lib().geo_ae_num_params())

    def params(self):
        out = np.empty(self.num_params(), np.float32)
        check(lib().geo_ae_get_params(self._p, C.c_void_p(out.ctypes.data)), "geo_ae_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().geo_ae_set_params(self._p, C.c_void_p(p.ctypes.data)), "geo_ae_set_params")

    def reserve(self, max_blocks):
        check(lib().geo_ae_reserve(self._p, int(max_blocks)), "geo_ae_reserve")

    def num_blocks(self):
        return int(lib().geo_ae_num_blocks(self._p))

    def add_blocks(self, blocks):
        b = _Bufs(blocks)
        n = blocks.shape[0]
        check(lib().geo_ae_add_blocks(self._p, b.inp(blocks), n, b.mem), "geo_ae_add_blocks")

    def add_shot(self, plan, is_=0, snap_every=10, t_first=0, rel=1e-3):
        check(lib().geo_ae_add_shot(self._p, plan._p, is_, snap_every, t_first, C.c_float(rel), None),
              "geo_ae_add_shot")

    def train(self, iters, batch=256, lr=1e-3):
        loss = np.zeros(iters, np.float32)
        check(lib().geo_ae_train(self._p, iters, batch, C.c_float(lr), C.c_void_p(loss.ctypes.data), None),
              "geo_ae_train")
        return loss

    def eval(self, blocks, grad=True):
        """(recon, loss, grad) on nb (multiple of 128) blocks (nb, 4096)."""
        b = _Bufs(blocks)
        nb = blocks.shape[0]
        rec, pr = b.out((nb, 4096), blocks)
        g, pg = b.out((self.num_params(),), blocks) if grad else (None, None)
        loss = C.c_double()
        check(lib().geo_ae_eval(self._p, b.inp(blocks), nb, pr, C.byref(loss), pg, b.mem, b.stream()), "geo_ae_eval")
        return rec, loss.value, g

    def roundtrip(self, vol, escape=False):
        """Encode + decode a (ny, nx, nz) CUDA tensor; returns the
        reconstruction (and the number of escaped blocks if `escape`)."""
        t = _torch()
        vol = vol.to(t.float32).contiguous()
        ny, nx, nz = vol.shape
        out = t.empty_like(vol)
        ne = C.c_int(0)
        check(lib().geo_ae_roundtrip(self._p, nx, ny, nz, C.c_void_p(vol.data_ptr()), C.c_void_p(out.data_ptr()),
                                     1 if escape else 0, C.byref(ne),
                                     C.c_void_p(t.cuda.current_stream().cuda_stream)), "geo_ae_roundtrip")
        return (out, ne.value) if escape else out

    def set_escape(self, tau=0.05, frac=0.03):
        """Per snapshot, keep bf16 residuals of the (at most frac of the)
        blocks with the largest decoding error above tau times their norm."""
        check(lib().geo_ae_set_escape(self._p, C.c_float(tau), C.c_float(frac)), "geo_ae_set_escape")

    def stats(self):
        """(blocks coded, blocks escaped) over the learned RTM shots so far."""
        b, e = C.c_longlong(), C.c_longlong()
        check(lib().geo_ae_stats(self._p, C.byref(b), C.byref(e)), "geo_ae_stats")
        return b.value, e.value

    def close(self):
        if self._p:
            lib().geo_ae_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tc_gemm_bf16(A, B, bias=None, act=False, out_f32=True):
    """out = A @ B^T (+bias) (leaky ReLU) with the codec's tcgen05 GEMM;
    A (M, K), B (N, K) bf16 CUDA tensors."""
    t = _torch()
    M, K = A.shape
    N = B.shape[0]
    out = t.empty((M, N), dtype=t.float32 if out_f32 else t.bfloat16, device=A.device)
    bp = C.c_void_p(bias.data_ptr()) if bias is not None else None
    check(lib().geo_tc_gemm_bf16(M, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), bp, 1 if act else 0,
                                 C.c_void_p(out.data_ptr()), 1 if out_f32 else 0,
                                 C.c_void_p(t.cuda.current_stream().cuda_stream)), "geo_tc_gemm_bf16")
    return out


def rtm2d_batch(v, e, d, *, npd, nt, dx, dz, dt_ms, favg, pfac, zs, shot_x, shot_nxs, laplace=True,
                per_shot=False, tile_x=0, adcig=False, mode="exact"):
    """Batched 2D RTM with the MPI program's semantics; returns the stacked
    (Laplacian-filtered) image (nx, nz) [and the per-shot images] [and the
    Poynting angle gathers (90, nx, nz) when `adcig`].  mode "exact" is the
    program's arithmetic bit for bit; "fast" forms its double-precision
    chains (two stress terms and the illumination sum) in FP32."""
    b = _Bufs(v, e, d)
    nx, nz = v.shape
    ns = len(shot_x)
    sx = (C.c_int * ns)(*[int(k) for k in shot_x])
    sw = (C.c_int * ns)(*[int(k) for k in shot_nxs])
    desc = RTM2DDesc(nx=nx, nz=nz, npd=npd, nt=nt, dx=dx, dz=dz, dt_ms=dt_ms, favg=favg, pfac=pfac, zs=zs, ns=ns,
                     shot_x=sx, shot_nxs=sw, laplace=1 if laplace else 0, tile_z=0, tile_x=tile_x,
                     mode=_MODES[mode] if isinstance(mode, str) else int(mode))
    pv, pe, pd = b.inp(v), b.inp(e), b.inp(d)
    img, pi = b.out((nx, nz), v)
    shots = pshots = None
    if per_shot:
        shots, pshots = b.out((int(sum(int(w) for w in shot_nxs)) * nz,), v)
    gathers = pg = None
    if adcig:
        gathers, pg = b.out((90, nx, nz), v)
    check(lib().geo_rtm2d_batch_adcig(C.byref(desc), pv, pe, pd, pi, pshots, pg, b.mem, b.stream()),
          "geo_rtm2d_batch")
    res = [img]
    if per_shot:
        out, o = [], 0
        for w in shot_nxs:
            out.append(shots[o:o + int(w) * nz].reshape(int(w), nz))
            o += int(w) * nz
        res.append(out)
    if adcig:
        res.append(gathers)
    return res[0] if len(res) == 1 else tuple(res)


def laplace2d(img):
    """Adjoint first-difference Laplacian (laplac2_lop adj=1) of (nx, nz)."""
    b = _Bufs(img)
    nx, nz = img.shape
    pi = b.inp(img)
    out, po = b.out((nx, nz), img)
    check(lib().geo_laplace2d(nx, nz, pi, po, b.mem, b.stream()), "geo_laplace2d")
    return out


def laplace3d(img):
    """3D adjoint first-difference Laplacian of (ny, nx, nz)."""
    b = _Bufs(img)
    ny, nx, nz = img.shape
    pi = b.inp(img)
    out, po = b.out((ny, nx, nz), img)
    check(lib().geo_laplace3d(nx, ny, nz, pi, po, b.mem, b.stream()), "geo_laplace3d")
    return out


def _s(x):
    return x.encode() if isinstance(x, str) else x


def GPU_vti2dfd(nx, nz, dx, dz, npd, SV, FNv, FNe, FNd, favg, ns, fs, ds, zs, FNshot, FNsnap, nt, dt, run_count=1):
    """Drop-in for GPU_vti2dfd_kernels.cu:301 (files in, files out)."""
    lib().GPU_vti2dfd(nx, nz, dx, dz, npd, SV, _s(FNv), _s(FNe), _s(FNd), favg, ns, fs, ds, zs, _s(FNshot),
                      _s(FNsnap), nt, dt, run_count)


def CPU_vti2dfd(nx, nz, dx, dz, npd, SV, FNv, FNe, FNd, favg, ns, fs, ds, zs, FNshot, FNsnap, nt, dt, run_count=1):
    """Drop-in for CPU_vti2dfd_kernels.c:366 (CPU semantics, computed on the GPU)."""
    lib().CPU_vti2dfd(nx, nz, dx, dz, npd, SV, _s(FNv), _s(FNe), _s(FNd), favg, ns, fs, ds, zs, _s(FNshot),
                      _s(FNsnap), nt, dt, run_count)


def GPU_vti3dfd(nx, ny, nz, dx, dy, dz, npml, SV, FNv, FNe, FNd, favg, ns, fsx, dsx, fsy, dsy, fsz, dsz, FNshot,
                FNsnap, nt, dt, run_count=1):
    """Drop-in for GPU_vti3dfd_kernels.cu:371."""
    lib().GPU_vti3dfd(nx, ny, nz, dx, dy, dz, npml, SV, _s(FNv), _s(FNe), _s(FNd), favg, ns, fsx, dsx, fsy, dsy,
                      fsz, dsz, _s(FNshot), _s(FNsnap), nt, dt, run_count)


def su_read(path, ntr, ns, big_endian=True, headers=False):
    """ntr traces of ns samples -> (ntr, ns) float32 [and (ntr, 240) uint8 headers]."""
    data = np.empty((ntr, ns), np.float32)
    hdr = np.empty((ntr, 240), np.uint8) if headers else None
    check(lib().geo_su_read(_s(path), ntr, ns, 1 if big_endian else 0, C.c_void_p(data.ctypes.data),
                            C.c_void_p(hdr.ctypes.data) if headers else None), "geo_su_read")
    return (data, hdr) if headers else data


def su_write(path, data, dt_us=1000.0, big_endian=True, headers=None):
    """Write (ntr, ns) traces with generated (or given (ntr, 240)) headers."""
    data = np.ascontiguousarray(data, np.float32)
    ntr, ns = data.shape
    h = None if headers is None else np.ascontiguousarray(headers, np.uint8)
    check(lib().geo_su_write(_s(path), ntr, ns, C.c_float(dt_us), 1 if big_endian else 0,
                             C.c_void_p(data.ctypes.data), C.c_void_p(h.ctypes.data) if h is not None else None),
          "geo_su_write")


def su_replace_data(template, raw, out, ntr, ns):
    """The binary2segy utility: template headers + byte-swapped raw samples."""
    check(lib().geo_su_replace_data(_s(template), _s(raw), _s(out), ntr, ns), "geo_su_replace_data")


class Par:
    """A `key= value` par file read by geo_par_load."""

    def __init__(self, path):
        self._p = C.c_void_p()
        check(lib().geo_par_load(_s(path), C.byref(self._p)), "geo_par_load")

    def int(self, key):
        x = C.c_int()
        check(lib().geo_par_get_int(self._p, _s(key), C.byref(x)), "geo_par_get_int")
        return x.value

    def float(self, key):
        x = C.c_float()
        check(lib().geo_par_get_float(self._p, _s(key), C.byref(x)), "geo_par_get_float")
        return x.value

    def str(self, key):
        buf = C.create_string_buffer(1024)
        check(lib().geo_par_get_string(self._p, _s(key), buf, 1024), "geo_par_get_string")
        return buf.value.decode()

    def __del__(self):
        try:
            if self._p:
                lib().geo_par_free(self._p)
        except Exception:
            pass


def read_par(path):
    return Par(path)


def _par_run(fn, path, out_shape, device, like):
    """geo_fd2d / geo_fd3d / geo_rtm2d on a par file; with out_shape, also
    into a fresh CUDA tensor of that shape (returned)."""
    par = Par(path)
    out, ptr, stream = None, None, None
    if out_shape is not None:
        t = _torch()
        out = t.empty(out_shape, dtype=t.float32, device="cuda" if like is None else like)
        ptr, stream = C.c_void_p(out.data_ptr()), C.c_void_p(t.cuda.current_stream().cuda_stream)
    check(getattr(lib(), fn)(par._p, device, ptr, stream), fn)
    return out


def fd2d_par(path, device=-1, out_shape=None):
    """The shots of GPU_vti2dfd / CPU_vti2dfd from a par file (see geo_fd2d)."""
    return _par_run("geo_fd2d", path, out_shape, device, None)


def fd3d_par(path, device=-1, out_shape=None):
    """The shots of GPU_vti3dfd from a par file (see geo_fd3d)."""
    return _par_run("geo_fd3d", path, out_shape, device, None)


def rtm2d_par(path, device=-1, out_shape=None):
    """The MPI RTM program from a par file (see geo_rtm2d)."""
    return _par_run("geo_rtm2d", path, out_shape, device, None)
