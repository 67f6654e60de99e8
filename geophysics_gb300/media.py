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
    G = np.fft.irfftn(np.fft.rfftn(noise) * filt, s=(ny, nx, nz), axes=(0, 1, 2))
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


def interface_model(nx, nz, tops, values, base, ny=None):
    """Layered medium by interfaces, the rule of the reference's generators
    (utils-getBinaryMedia-c/Toa_vtiMedia.c:27-60, 3D-vti-fd+rtm-cuda/
    Toa_vel3.c:37-51): a cell takes `base`, then values[k] for every
    interface k (in order, later ones win) whose depth it lies strictly below
    (iz > top).  tops[k] is a depth in cells, or an array over x (a curved
    interface such as `anticline_profile`).  Returns float32 (nx, nz), or
    (ny, nx, nz) when ny is given (interfaces constant along y)."""
    iz = np.arange(nz)[None, :]
    a = np.full((nx, nz), base, np.float32)
    for top, val in zip(tops, values):
        t = np.broadcast_to(np.asarray(top, np.float64).reshape(-1, 1) if np.ndim(top) else top, (nx, 1))
        a = np.where(iz > t, np.float32(val), a)
    a = a.astype(np.float32)
    return a if ny is None else np.ascontiguousarray(np.broadcast_to(a, (ny, nx, nz)))


def anticline_profile(nx, x0, x1, x2, x3, z_flank, z_crest):
    """Depth of an anticline-shaped interface over x, as the generators'
    `layer` arrays (utils-getBinaryMedia-c/Toa_vel.c:27-34: 150 / rising
    0.5 per cell / 200 / falling / 150 with breaks at x = 150, 250, 350,
    450; Toa_vel3.c:29-35 the same at 25, 75, 125, 175 from 100 to 125):
    z_flank before x0 and from x3 on, a linear ramp from x0 to x1 and back
    down from x2 to x3, z_crest between x1 and x2.  float32 (nx,)."""
    k = np.arange(nx, dtype=np.float64)
    up = (z_crest - z_flank) / float(x1 - x0)
    down = (z_crest - z_flank) / float(x3 - x2)
    z = np.full(nx, float(z_flank))
    z = np.where((k >= x0) & (k < x1), up * (k - x0) + z_flank, z)
    z = np.where((k >= x1) & (k < x2), z_crest, z)
    z = np.where((k >= x2) & (k < x3), -down * (k - x2) + z_crest, z)
    return z.astype(np.float32)


def vti_layers_media(nx, nz=2500):
    """The VTI media generator's model (Toa_vtiMedia.c, 10000 x 2500 there):
    interfaces below rows 500, 1000, 1500, 2000; vp 2000/2600/3300/3800/4500,
    eps 0/0.07/0.12/0.19/0.25, del 0/0.02/0.05/0.08/0.1.  Returns v, e, d (nx, nz)."""
    tops = (500, 1000, 1500, 2000)
    return (interface_model(nx, nz, tops, (2600, 3300, 3800, 4500), 2000.0),
            interface_model(nx, nz, tops, (0.07, 0.12, 0.19, 0.25), 0.0),
            interface_model(nx, nz, tops, (0.02, 0.05, 0.08, 0.1), 0.0))
