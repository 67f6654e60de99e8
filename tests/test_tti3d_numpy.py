"""An independent restatement of the 3D TTI step in vectorised numpy (FP64)
against the oracle's FP64 build.  The 3D TTI scheme has no reference
program, so this is the check on the oracle's transcription of it:

  u <- k2 u - k1 dP/dx',  v <- k2 v - k1 dP/dy',  w <- k2 w - k1 dQ/dz'
  P <- k2 P - k1 (A a + B b),  Q <- k2 Q - k1 (B a + C b)

with x' = (cos t cos f, cos t sin f, -sin t), y' = (-sin f, cos f, 0),
z' = (sin t cos f, sin t sin f, cos t), a = du/dx' + dv/dy', b = dw/dz',
forward-staggered axis derivatives for the velocities and backward ones
for the stresses, the product sponge, and the source added to P,Q before
the velocity update only.  The sponge profiles, d0 and source amplitudes
come from the oracle's helpers shared with the VTI path (pinned there)."""
import ctypes as C

import numpy as np

from tests.util import random_model_3d, rel_l2, smooth_angles

C8 = np.array([1.196289, -0.0797526, 0.009570313, -0.0006975447], np.float32).astype(np.float64)


def dfwd(f, axis, lo, hi):
    """sum_m c_m (f[i+m+1] - f[i-m]) along axis for i in [lo, hi)."""
    out = 0.0
    for m in range(4):
        out = out + C8[m] * (np.take(f, range(lo + m + 1, hi + m + 1), axis) - np.take(f, range(lo - m, hi - m), axis))
    return out


def dbwd(f, axis, lo, hi):
    """sum_m c_m (f[i+m] - f[i-m-1]) along axis for i in [lo, hi)."""
    out = 0.0
    for m in range(4):
        out = out + C8[m] * (np.take(f, range(lo + m, hi + m), axis) - np.take(f, range(lo - m - 1, hi - m - 1), axis))
    return out


def numpy_tti3d(orc, v, e, d, th, ph, *, npd, nt, dx, dy, dz, dt, favg, pfac, fsx, fsy, fsz):
    ny, nx, nz = v.shape
    pad = lambda a: np.pad(a.astype(np.float64), npd, mode="edge")
    V, E, D, T, F = (pad(a) for a in (v, e, d, th, ph))
    nny, nnx, nnz = V.shape
    A = V * V * (1 + 2 * E)
    B = V * V * np.sqrt(1 + 2 * D)
    Cm = V * V
    ct, st = np.cos(T * (np.pi / 180)), np.sin(T * (np.pi / 180))
    cp, sp = np.cos(F * (np.pi / 180)), np.sin(F * (np.pi / 180))
    L = orc.lib(64)
    L.orc_d0.restype = C.c_float
    L.orc_d0.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float]
    d0 = L.orc_d0(1, 3, 0.0, float(V.reshape(-1)[V.size // 2]), npd, dx, dy, dz)
    prof = {}
    for ax, n in (("x", nx), ("y", ny), ("z", nz)):
        p = [np.zeros(n + 2 * npd, np.float32) for _ in range(4)]
        L.orc_sponge.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float] + [C.POINTER(C.c_float)] * 4
        L.orc_sponge(1, n, npd, dt, d0, *[q.ctypes.data_as(C.POINTER(C.c_float)) for q in p])
        prof[ax] = [q.astype(np.float64) for q in p]      # coff1, coff2, acoff1, acoff2
    amp = np.zeros(nt, np.float32)
    act = np.zeros(nt, np.uint8)
    L.orc_source_amp.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                 C.POINTER(C.c_float), C.POINTER(C.c_ubyte)]
    L.orc_source_amp(1, nt, dt, favg, pfac, 1, amp.ctypes.data_as(C.POINTER(C.c_float)),
                     act.ctypes.data_as(C.POINTER(C.c_ubyte)))
    dtx, dty, dtz = (np.float64(np.float32(dt) / np.float32(h)) for h in (dx, dy, dz))
    u, vv, w, P, Q = (np.zeros(V.shape) for _ in range(5))
    sy, sx, sz = slice(4, nny - 4), slice(4, nnx - 4), slice(4, nnz - 4)
    inner = (sy, sx, sz)
    src = (fsy + npd - 1, fsx + npd - 1, fsz + npd - 1)
    rec = np.zeros((ny, nx, nt))
    a, b, c, s = ct[inner], st[inner], cp[inner], sp[inner]
    for it in range(nt):
        p0, q0 = P[src], Q[src]
        if act[it]:
            P[src] += amp[it]
            Q[src] += amp[it]
        # velocities: k = cx*cy*cz in that order
        k2 = prof["x"][1][sx][None, :, None] * prof["y"][1][sy][:, None, None] * prof["z"][1][sz][None, None, :]
        k1 = prof["x"][0][sx][None, :, None] * prof["y"][0][sy][:, None, None] * prof["z"][0][sz][None, None, :]
        Px, Py, Pz = dfwd(P, 1, 4, nnx - 4)[sy, :, sz], dfwd(P, 0, 4, nny - 4)[:, sx, sz], dfwd(P, 2, 4, nnz - 4)[sy, sx, :]
        Qx, Qy, Qz = dfwd(Q, 1, 4, nnx - 4)[sy, :, sz], dfwd(Q, 0, 4, nny - 4)[:, sx, sz], dfwd(Q, 2, 4, nnz - 4)[sy, sx, :]
        u[inner] = k2 * u[inner] - k1 * (a * c * dtx * Px + a * s * dty * Py - b * dtz * Pz)
        vv[inner] = k2 * vv[inner] - k1 * (c * dty * Py - s * dtx * Px)
        w[inner] = k2 * w[inner] - k1 * (b * c * dtx * Qx + b * s * dty * Qy + a * dtz * Qz)
        # stresses from the new velocities and P,Q before the source
        P[src], Q[src] = p0, q0
        k2 = prof["x"][3][sx][None, :, None] * prof["y"][3][sy][:, None, None] * prof["z"][3][sz][None, None, :]
        k1 = prof["x"][2][sx][None, :, None] * prof["y"][2][sy][:, None, None] * prof["z"][2][sz][None, None, :]
        ux, uy, uz = dbwd(u, 1, 4, nnx - 4)[sy, :, sz], dbwd(u, 0, 4, nny - 4)[:, sx, sz], dbwd(u, 2, 4, nnz - 4)[sy, sx, :]
        vx, vy = dbwd(vv, 1, 4, nnx - 4)[sy, :, sz], dbwd(vv, 0, 4, nny - 4)[:, sx, sz]
        wx, wy, wz = dbwd(w, 1, 4, nnx - 4)[sy, :, sz], dbwd(w, 0, 4, nny - 4)[:, sx, sz], dbwd(w, 2, 4, nnz - 4)[sy, sx, :]
        ha = (a * c * dtx * ux + a * s * dty * uy - b * dtz * uz) + (c * dty * vy - s * dtx * vx)
        hb = b * c * dtx * wx + b * s * dty * wy + a * dtz * wz
        Pn = k2 * P[inner] - k1 * (A[inner] * ha + B[inner] * hb)
        Qn = k2 * Q[inner] - k1 * (B[inner] * ha + Cm[inner] * hb)
        P[inner], Q[inner] = Pn, Qn
        rec[:, :, it] = P[npd:npd + ny, npd:npd + nx, npd]
    return rec


def test_tti3d_numpy_restatement_matches_oracle(orc):
    v, e, d = random_model_3d(12, 11, 13, seed=21)
    th, ph = smooth_angles(v.shape, seed=22)
    kw = dict(npd=6, nt=60, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, fsx=6, fsy=5,
              fsz=3)
    want = orc.fd3d(v, e, d, theta=th, phi=ph, prec=64, rec_iz=6, **kw)
    got = numpy_tti3d(orc, v, e, d, th, ph, **kw)
    assert np.abs(want).max() > 0
    # the oracle hands back FP32 records: the floor is their rounding (measured 2.6e-8)
    assert rel_l2(got, want) < 1e-7
