"""Shared helpers for the tests: seeded models and error measures."""
import numpy as np


def layered_model(nx, nz, seed=1, nlayers=5, vlo=2000.0, vhi=4000.0, emax=0.25, dmax=0.1):
    """Flat layers with per-layer vp/eps/del drawn from a seeded generator,
    sorted so velocity grows with depth."""
    rng = np.random.default_rng(seed)
    vp = np.sort(rng.uniform(vlo, vhi, nlayers))
    ep = rng.uniform(0.0, emax, nlayers)
    # delta <= eps per layer: the pseudo-acoustic VTI system is unstable
    # where delta > eps, in the reference as much as here
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


def random_model_3d(nx, ny, nz, seed=2, vlo=1800.0, vhi=3200.0):
    rng = np.random.default_rng(seed)
    base = rng.uniform(0, 1, (ny, nx, nz)).astype(np.float32)
    # a little smoothing so the field is not white noise
    for ax in range(3):
        base = (np.roll(base, 1, ax) + base + np.roll(base, -1, ax)) / 3
    base = (base - base.min()) / (base.max() - base.min())
    v = (vlo + (vhi - vlo) * base).astype(np.float32)
    e = (0.2 * base).astype(np.float32)
    d = (0.1 * base).astype(np.float32)
    return v, e, d


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def to_np(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(x)


def wave_blocks(nb, seed):
    """Band-limited random 16^3 blocks in Morton order (sums of plane waves
    under a Gaussian envelope, amplitudes over two decades)."""
    from oracle import ae_oracle as A
    rng = np.random.default_rng(seed)
    z, x, y = np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij")
    out = np.zeros((nb, 4096), np.float32)
    perm = A.morton_order()
    zz, xx, yy = perm % 16, (perm // 16) % 16, perm // 256
    for b in range(nb):
        f = np.zeros((16, 16, 16))
        for _ in range(3):
            k = rng.normal(0, 0.6, 3)
            f += rng.normal() * np.cos(k[0] * z + k[1] * x + k[2] * y + rng.uniform(0, 6.28))
        f *= np.exp(-((z - 8) ** 2 + (x - 8) ** 2 + (y - 8) ** 2) / rng.uniform(20, 80))
        out[b] = (rng.uniform(0.1, 10) * f)[zz, xx, yy]
    return out


def smooth_angles(shape, seed=0):
    """Smooth tilt 2.5-42.5 deg and azimuth 10-350 deg fields (ny, nx, nz)."""
    ny, nx, nz = shape
    rng = np.random.default_rng(seed)
    a, b, c = rng.uniform(5, 12, 3)
    Y, X, Z = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
    theta = 22.5 + 20.0 * np.sin(X / a + Y / b) * np.cos(Z / c)
    phi = 180.0 + 170.0 * np.sin(X / c - Y / a + Z / b)
    return theta.astype(np.float32), phi.astype(np.float32)
