"""Synthetic VTI media: seeded smooth random fields with dipping interfaces.

The reference builds its test media with small C generators
(utils-getBinaryMedia-c/Toa_vtiMedia.c: layers and anticlines) and ships no
model files; this generator makes the random-field media the benchmarks and
the codec's training set use: a Gaussian random field of the given
correlation length (FFT-filtered white noise), mapped to vp in [vlo, vhi),
plus planar dipping interfaces that each add a velocity jump, with
eps = emax*(vp-vlo)/(vhi-vlo) and del = dmax*(vp-vlo)/(vhi-vlo) (so
del <= eps everywhere).  Arrays are (ny, nx, nz), z fastest: the reference's
binary layout iz + nz*(ix + nx*iy).
"""
import numpy as np


def random_vti(nx, ny, nz, seed=0, corr=40.0, vlo=1500.0, vhi=4500.0, jump=300.0, interfaces=3, emax=0.3,
               dmax=0.15):
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((ny, nx, nz)).astype(np.float32)
    sig = corr / 2.0
    fy = np.fft.fftfreq(ny)[:, None, None]
    fx = np.fft.fftfreq(nx)[None, :, None]
    fz = np.fft.rfftfreq(nz)[None, None, :]
    filt = np.exp(-2.0 * np.pi ** 2 * sig ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    G = np.fft.irfftn(np.fft.rfftn(noise) * filt, s=(ny, nx, nz))
    G = (G - G.min()) / max(G.max() - G.min(), 1e-30)
    span = vhi - vlo - interfaces * jump
    vp = vlo + span * G
    iy = np.arange(ny, dtype=np.float64)[:, None, None]
    ix = np.arange(nx, dtype=np.float64)[None, :, None]
    iz = np.arange(nz, dtype=np.float64)[None, None, :]
    for k in range(interfaces):
        z0 = nz * (k + 1) / (interfaces + 1) + rng.uniform(-0.05, 0.05) * nz
        ax, ay = rng.uniform(-0.12, 0.12, 2)
        vp = vp + jump * (iz > z0 + ax * (ix - nx / 2) + ay * (iy - ny / 2))
    frac = (vp - vlo) / (vhi - vlo)
    return (vp.astype(np.float32), (emax * frac).astype(np.float32), (dmax * frac).astype(np.float32))


def layered_vti(nx, nz, seed=1, nlayers=5, vlo=2000.0, vhi=4000.0, emax=0.25, dmax=0.1):
    """Flat layers (2D, shape (nx, nz), z fastest): per-layer vp, eps, del
    drawn from a seeded generator, velocities sorted to grow with depth and
    del <= eps in every layer (the pseudo-acoustic VTI system is unstable
    where del > eps, in the reference as much as here)."""
    rng = np.random.default_rng(seed)
    vp = np.sort(rng.uniform(vlo, vhi, nlayers))
    ep = rng.uniform(0.0, emax, nlayers)
    de = np.minimum(rng.uniform(0.0, dmax, nlayers), ep)
    bounds = np.linspace(0, nz, nlayers + 1).astype(int)
    v = np.empty((nx, nz), np.float32)
    e = np.empty((nx, nz), np.float32)
    d = np.empty((nx, nz), np.float32)
    for k in range(nlayers):
        v[:, bounds[k]:bounds[k + 1]] = vp[k]
        e[:, bounds[k]:bounds[k + 1]] = ep[k]
        d[:, bounds[k]:bounds[k + 1]] = de[k]
    return v, e, d


def layered_random_vti(nx, nz, seed=3, corr=40.0, amp=0.05, **kw):
    """`layered_vti` times (1 + amp * G) with G a zero-mean unit-max Gaussian
    random field of correlation `corr` cells; eps and del scale with it."""
    v, e, d = layered_vti(nx, nz, seed=seed, **kw)
    rng = np.random.default_rng(seed + 1000)
    noise = rng.standard_normal((nx, nz))
    sig = corr / 2.0
    fx = np.fft.fftfreq(nx)[:, None]
    fz = np.fft.rfftfreq(nz)[None, :]
    G = np.fft.irfft2(np.fft.rfft2(noise) * np.exp(-2.0 * np.pi ** 2 * sig ** 2 * (fx ** 2 + fz ** 2)), s=(nx, nz))
    G = G / max(np.abs(G).max(), 1e-30)
    f = (1.0 + amp * G).astype(np.float32)
    return (v * f).astype(np.float32), (e * f).astype(np.float32), (d * f).astype(np.float32)
