"""CPU oracle of the learned snapshot codec -- test infrastructure only.

The codec has no counterpart in the reference (it is the learned part added
to 3D RTM); this restates its arithmetic in numpy so the GPU forward and
backward kernels can be checked:

  * `emulate=True` follows the GPU's rounding points: bf16 weights, bf16
    activations after every level (round to nearest even), fp32 block
    scaling, E1 and D1 summed in fp32 in the kernels' order, the GEMM levels
    accumulated exactly (float64) and rounded to fp32 -- the tensor cores'
    fp32 accumulation order is not specified, so GPU and oracle agree to
    rounding, not bit for bit;
  * `emulate=False` is the same network in float64 without rounding, for
    checking the backward formulas against finite differences.

Blocks are 16^3 points in Morton order (bit 3l = z bit l, 3l+1 = x bit l,
3l+2 = y bit l).  Levels (out N, in K, rows per block, activation):
E1 16<-8, E2 64<-128, E3 256<-512, E4 512<-2048 (linear), D4 2048<-512,
D3 512<-256, D2 128<-64, D1 8<-16 (linear); leaky ReLU slope 0.1.
"""
import numpy as np

LAYERS = [(16, 8, 512, 1), (64, 128, 64, 1), (256, 512, 8, 1), (512, 2048, 1, 0),
          (2048, 512, 1, 1), (512, 256, 8, 1), (128, 64, 64, 1), (8, 16, 512, 0)]
LEAK = 0.1
TINY = 1e-30


def offsets():
    """[(w_offset, b_offset)] per level in the flat parameter vector."""
    out, p = [], 0
    for N, K, _, _ in LAYERS:
        out.append((p, p + N * K))
        p += N * K + N
    return out, p


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32)


def morton_order():
    m = np.arange(4096)
    z = sum(((m >> (3 * l)) & 1) << l for l in range(4))
    x = sum(((m >> (3 * l + 1)) & 1) << l for l in range(4))
    y = sum(((m >> (3 * l + 2)) & 1) << l for l in range(4))
    return z + 16 * x + 256 * y


def blocks_of_volume(vol):
    """(ny, nx, nz) volume with multiple-of-16 extents -> (nb, 4096) Morton
    blocks, block index bz + nbz*(bx + nbx*by)."""
    ny, nx, nz = vol.shape
    b = vol.reshape(ny // 16, 16, nx // 16, 16, nz // 16, 16).transpose(0, 2, 4, 1, 3, 5)
    b = b.reshape(-1, 4096)                     # natural order y, x, z within the block
    perm = morton_order()                       # natural index z + 16x + 256y
    zz, xx, yy = perm % 16, (perm // 16) % 16, perm // 256
    return np.ascontiguousarray(b[:, yy * 256 + xx * 16 + zz])


def _leaky(v):
    return np.where(v > 0, v, v * (np.float32(LEAK) if v.dtype == np.float32 else LEAK))


def _weights(params, emulate):
    offs, _ = offsets()
    Ws, bs = [], []
    for (N, K, _, _), (ow, ob) in zip(LAYERS, offs):
        W = params[ow:ow + N * K].reshape(N, K)
        b = params[ob:ob + N]
        if emulate:
            Ws.append(bf16(W.astype(np.float32)))
            bs.append(b.astype(np.float32))
        else:
            Ws.append(W.astype(np.float64))
            bs.append(b.astype(np.float64))
    return Ws, bs


def _seq_dot(W, X):
    """fp32 sum over the last axis in index order: out[r, c] = sum_j W[c, j] X[r, j]."""
    acc = np.zeros((X.shape[0], W.shape[0]), np.float32)
    for j in range(W.shape[1]):
        acc = (acc + (X[:, j:j + 1] * W[None, :, j]).astype(np.float32)).astype(np.float32)
    return acc


def forward(params, blocks, emulate=True):
    """Returns a dict of the activations, 'recon' (normalized) and 'loss'."""
    f = np.float32 if emulate else np.float64
    Ws, bs = _weights(params, emulate)
    x = np.asarray(blocks, f)
    B = x.shape[0]
    s = np.abs(x).max(axis=1)
    s = np.where(s >= TINY, s, 0)        # blocks below TINY are coded as zero
    if emulate:
        inv = np.where(s > 0, np.float32(1) / np.where(s > 0, s, 1).astype(np.float32), 0).astype(np.float32)
        xn = (x * inv[:, None]).astype(np.float32)
        x8 = bf16(xn).reshape(B * 512, 8)
        h = _seq_dot(Ws[0], x8)
        h = bf16(_leaky((h + bs[0]).astype(np.float32)))
    else:
        inv = np.where(s > 0, 1.0 / np.where(s > 0, s, 1), 0)
        xn = x * inv[:, None]
        x8 = xn.reshape(B * 512, 8)
        h = _leaky(x8 @ Ws[0].T + bs[0])
    acts = {"xn": xn, "x8": x8, "scale": s, "a0": h}
    a = h
    for l in range(1, 7):
        N, K, rows, act = LAYERS[l]
        A = a.reshape(B * rows, K)
        if emulate:
            o = (A.astype(np.float64) @ Ws[l].T.astype(np.float64)).astype(np.float32)
            o = (o + bs[l]).astype(np.float32)
            if act:
                o = _leaky(o)
            o = bf16(o)
        else:
            o = A @ Ws[l].T + bs[l]
            if act:
                o = _leaky(o)
        acts["in%d" % l] = A
        acts["a%d" % l] = o
        a = o
    g = a.reshape(B * 512, 16)
    if emulate:
        y = (_seq_dot(Ws[7], g) + bs[7]).astype(np.float32)
    else:
        y = g @ Ws[7].T + bs[7]
    acts["g1"] = g
    recon = y.reshape(B, 4096)
    acts["recon"] = recon
    d = recon - xn
    acts["loss"] = float(np.sum(d.astype(np.float64) ** 2) / d.size)
    return acts


def backward(params, blocks, emulate=True):
    """(loss, grad) with grad = d loss / d params (flat, float64)."""
    acts = forward(params, blocks, emulate)
    Ws, _ = _weights(params, emulate)
    offs, P = offsets()
    grad = np.zeros(P, np.float64)
    B = blocks.shape[0]
    count = B * 4096
    if emulate:
        dy = (np.float32(2) * (acts["recon"] - acts["xn"]).astype(np.float32) * np.float32(1.0 / count)).astype(
            np.float32).reshape(B * 512, 8)
    else:
        dy = (2.0 * (acts["recon"] - acts["xn"]) / count).reshape(B * 512, 8)
    g = acts["g1"]
    grad[offs[7][0]:offs[7][1]] = (dy.astype(np.float64).T @ g.astype(np.float64)).ravel()
    grad[offs[7][1]:offs[7][1] + 8] = dy.astype(np.float64).sum(axis=0)
    if emulate:
        dg = _seq_dot(Ws[7].T.copy(), dy)
        dout = bf16(np.where(g > 0, dg, np.float32(LEAK) * dg).astype(np.float32))
    else:
        dg = dy @ Ws[7]
        dout = np.where(g > 0, dg, LEAK * dg)
    # dout: gradient at the output of level 6 (D2), shape (B*512, 16)
    for l in range(6, 0, -1):
        N, K, rows, act = LAYERS[l]
        D = dout.reshape(B * rows, N)
        A = acts["in%d" % l]
        grad[offs[l][0]:offs[l][1]] = (D.astype(np.float64).T @ A.astype(np.float64)).ravel()
        grad[offs[l][1]:offs[l][1] + N] = D.astype(np.float64).sum(axis=0)
        prev_act = LAYERS[l - 1][3]
        if emulate:
            dA = (D.astype(np.float64) @ Ws[l].astype(np.float64)).astype(np.float32)
            if prev_act:
                dA = np.where(A > 0, dA, np.float32(LEAK) * dA).astype(np.float32)
            dout = bf16(dA)
        else:
            dA = D @ Ws[l]
            if prev_act:
                dA = np.where(A > 0, dA, LEAK * dA)
            dout = dA
    D = dout.reshape(B * 512, 16)
    x8 = acts["x8"]
    grad[offs[0][0]:offs[0][1]] = (D.astype(np.float64).T @ x8.astype(np.float64)).ravel()
    grad[offs[0][1]:offs[0][1] + 16] = D.astype(np.float64).sum(axis=0)
    return acts["loss"], grad


def init_params(seed=0):
    """He-normal weights, zero biases (numpy generator; not the library's)."""
    rng = np.random.default_rng(seed)
    offs, P = offsets()
    p = np.zeros(P, np.float32)
    for (N, K, _, act), (ow, _) in zip(LAYERS, offs):
        p[ow:ow + N * K] = rng.normal(0, np.sqrt(2.0 / K), N * K)
    return p
