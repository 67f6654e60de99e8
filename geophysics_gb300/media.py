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
