"""The codec's CPU oracle: backward formulas against finite differences, and
the Morton block layout (CPU only)."""
import numpy as np

from oracle import ae_oracle as A
from tests.util import wave_blocks as _wave_blocks


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = A.init_params(1).astype(np.float64) * 0.5
    blocks = _wave_blocks(2, 4).astype(np.float64)
    loss, g = A.backward(p, blocks, emulate=False)
    offs, P = A.offsets()
    idx = []
    for (ow, ob), (N, K, _, _) in zip(offs, A.LAYERS):
        idx += list(rng.integers(ow, ow + N * K, 3)) + list(rng.integers(ob, ob + N, 2))
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = A.forward(q, blocks, emulate=False)["loss"]
        q[i] -= 2 * h
        lm = A.forward(q, blocks, emulate=False)["loss"]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])


def test_emulated_close_to_exact():
    p = A.init_params(2)
    blocks = _wave_blocks(4, 5)
    l32, g32 = A.backward(p, blocks, emulate=True)
    l64, g64 = A.backward(p.astype(np.float64), blocks.astype(np.float64), emulate=False)
    assert abs(l32 - l64) <= 0.05 * l64
    assert np.linalg.norm(g32 - g64) <= 0.1 * np.linalg.norm(g64)


def test_morton_blocks_of_volume():
    rng = np.random.default_rng(0)
    vol = rng.normal(size=(32, 16, 48)).astype(np.float32)   # (ny, nx, nz)
    b = A.blocks_of_volume(vol)
    assert b.shape == (3 * 1 * 2, 4096)
    perm = A.morton_order()
    assert sorted(perm) == list(range(4096))
    # block (bz=2, bx=0, by=1), Morton index 5 -> z bit0=1, y bit0=1
    m = 5
    z, x, y = perm[m] % 16, (perm[m] // 16) % 16, perm[m] // 256
    assert (z, x, y) == (1, 0, 1)
    assert b[2 + 3 * (0 + 1 * 1), m] == vol[16 + y, x, 32 + z]
