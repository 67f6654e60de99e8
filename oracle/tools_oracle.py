"""CPU restatement of the post-processing tools -- test infrastructure only,
never called by the library.

smooth1 / smooth2d: smooth1float and smooth2float of the MPI RTM program
(2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:1607-1664); adcig_smooth_stack: its
smoothed gathers and angle stack (:416-437); mute_direct: the direct-wave
mute utility (2D-vti-fd+rtm-cuda/functions/shot_muteDirect.c:11-33).  Pinned
against the reference's own smooth2float and mute_directwave, compiled from
its sources into oracle/_ref (tests/test_tools_oracle.py).
"""
import math

import numpy as np

_f = np.float32


def smooth1(v, r):
    """r Jacobi passes of 3-point averaging along the last axis (float32 sums
    in the programs' order, divided in double, stored float32)."""
    v0 = np.array(v, dtype=_f, copy=True)
    n = v0.shape[-1]
    for _ in range(r):
        out = np.empty_like(v0)
        s = (v0[..., :-2] + v0[..., 1:-1]) + v0[..., 2:]
        out[..., 1:-1] = (s.astype(np.float64) / 3.0).astype(_f)
        out[..., 0] = ((v0[..., 0] + v0[..., 1]).astype(np.float64) / 2.0).astype(_f)
        out[..., n - 1] = ((v0[..., n - 1] + v0[..., n - 2]).astype(np.float64) / 2.0).astype(_f)
        v0 = out
    return v0


def smooth2d(v, rx, rz):
    """v shaped (nx, nz): rx passes along x for every z, then rz along z."""
    a = smooth1(np.asarray(v, _f).T, rx).T
    return smooth1(a, rz)


def adcig_smooth_stack(adcig, passes=10):
    """adcig (na, nx, nz): smoothed along the angle axis; stack over angles
    in order from 0."""
    g = np.moveaxis(smooth1(np.moveaxis(np.asarray(adcig, _f), 0, -1), passes), -1, 0)
    stk = np.zeros(g.shape[1:], _f)
    for ia in range(g.shape[0]):
        stk = (stk + g[ia]).astype(_f)
    return np.ascontiguousarray(g), stk


def mute_direct(shot, *, dt, favg, dx, dz, fs, ds, zs, is_, vp, epsilon=0.0, tt=190):
    """shot (nx, nt) trace-major; returns the muted copy."""
    out = np.array(shot, dtype=_f, copy=True)
    nx, nt = out.shape
    dt, favg, dx, dz, vp, epsilon = (_f(x) for x in (dt, favg, dx, dz, vp, epsilon))
    for ix in range(nx):
        mu_x = _f(dx * _f(abs(ix - fs - (is_ - 1) * ds)))
        mu_z = _f(dz * _f(zs))
        den = float(_f(vp * np.sqrt(_f(_f(1) + _f(2) * epsilon))))
        mu_t0 = _f(math.sqrt(float(mu_x) ** 2 + float(mu_z) ** 2) / den)
        mu_t = int(2.0 / float(_f(dt * favg)))
        t0 = int(_f(mu_t0 / dt))
        mu_nt = t0 + mu_t + tt
        for it in range(nt):
            if it > t0 - tt and it < mu_nt:
                out[ix, it] = 0.0
    return out


def smooth_model2d(v, z0, passes):
    """The 2D in-place model smoother (utils-3D-smooth-f95/smooth.f95:44-70)
    on v (nx, nz), rows z >= z0 (the program's nzs - 1), in its visiting
    order with float32 arithmetic.  Parity unpinned: no Fortran compiler here."""
    a = np.array(v, dtype=_f, copy=True)
    nx, nz = a.shape
    X, Z = nx - 1, nz - 1
    two, four = _f(2), _f(4)

    def s(*t):
        acc = t[0]
        for x in t[1:]:
            acc = _f(acc + x)
        return acc

    for _ in range(passes):
        P = a
        P[0, z0] = s(two * P[1, z0], two * P[0, z0 + 1], P[1, z0 + 1], four * P[0, z0]) / _f(9)
        P[0, Z] = s(two * P[0, Z - 1], two * P[1, Z], P[1, Z - 1], four * P[0, Z]) / _f(9)
        P[X, z0] = s(two * P[X - 1, z0], P[X - 1, z0 + 1], two * P[X, z0 + 1], four * P[X, z0]) / _f(9)
        P[X, Z] = s(P[X - 1, Z - 1], two * P[X, Z - 1], two * P[X - 1, Z], four * P[X, Z]) / _f(9)
        for i in range(1, X):
            P[i, z0] = s(two * P[i - 1, z0], P[i - 1, z0 + 1], two * P[i, z0 + 1], P[i + 1, z0 + 1],
                         two * P[i + 1, z0], four * P[i, z0]) / _f(12)
            P[i, Z] = s(two * P[i - 1, Z], P[i - 1, Z - 1], two * P[i, Z - 1], P[i + 1, Z - 1], two * P[i + 1, Z],
                        four * P[i, Z]) / _f(12)
        for j in range(z0 + 1, Z):
            P[0, j] = s(two * P[0, j - 1], P[1, j - 1], two * P[1, j], P[1, j + 1], two * P[0, j + 1],
                        four * P[0, j]) / _f(12)
            P[X, j] = s(two * P[X, j - 1], P[X - 1, j - 1], two * P[X - 1, j], P[X - 1, j + 1], two * P[X, j + 1],
                        four * P[X, j]) / _f(12)
        for i in range(1, X):
            for j in range(z0 + 1, Z):
                P[i, j] = s(P[i - 1, j - 1], P[i, j - 1] * two, P[i + 1, j - 1], P[i - 1, j] * two, P[i, j] * four,
                            P[i + 1, j] * two, P[i - 1, j + 1], P[i, j + 1] * two, P[i + 1, j + 1]) / _f(16)
    return a
