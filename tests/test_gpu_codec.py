"""The learned snapshot codec on the GPU: the tcgen05 GEMM against torch,
forward and gradients against the CPU oracle, training on solver snapshots,
and 3D RTM with stored / coded snapshots."""
import numpy as np
import pytest

from tests.util import random_model_3d, rel_l2, wave_blocks

pytestmark = pytest.mark.gpu


# tile widths 64/128/256 with every stage count (stages = K/64 up to the
# width's ring: 4/3/2), including one-slice tiles whose bf16 output tile is
# larger than their ring
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 64, 128), (256, 64, 192), (128, 64, 256),
                                   (128, 128, 64), (256, 128, 128), (128, 128, 192),
                                   (256, 256, 64), (384, 256, 512), (128, 512, 2048), (256, 2048, 512)])
def test_tc_gemm_matches_torch(geo, M, N, K):
    import torch
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    ref = A.float() @ B.float().T   # fp32 reference of the same bf16 operands
    out = geo.tc_gemm_bf16(A, B)
    assert (out - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
    bias = torch.randn(N, generator=g).cuda()
    outb = geo.tc_gemm_bf16(A, B, bias=bias, act=True, out_f32=False).float()
    r = ref + bias
    r = torch.where(r > 0, r, 0.1 * r)
    # bf16 output: within one bf16 ulp of the fp32 reference (rounding may
    # fall either side when the fp32 sums differ in the last place)
    bad = ((outb - r).abs() > r.abs() * 2.0 ** -7 + 1e-6).float().mean().item()
    assert bad < 1e-3


def test_codec_forward_and_gradients_match_oracle(geo):
    from oracle import ae_oracle as A
    codec = geo.Codec(seed=3)
    p = codec.params()
    blocks = wave_blocks(128, 7)
    blocks[5] *= 1e-35          # below the zero-block threshold
    rec, loss, g = codec.eval(blocks)
    acts = A.forward(p, blocks)
    lo, go = A.backward(p, blocks)
    assert np.isfinite(rec).all()
    # bf16 activations: GPU and oracle agree to rounding (the tensor cores'
    # fp32 accumulation order is not specified); measured about 1e-3
    tol = 3e-3
    assert rel_l2(rec, acts["recon"]) < tol, rel_l2(rec, acts["recon"])
    assert abs(loss - lo) <= tol * lo, (loss, lo)
    offs, _ = A.offsets()
    worst = 0.0
    for l, (ow, ob) in enumerate(offs):
        N, K, _, _ = A.LAYERS[l]
        rw, rb = rel_l2(g[ow:ow + N * K], go[ow:ow + N * K]), rel_l2(g[ob:ob + N], go[ob:ob + N])
        worst = max(worst, rw, rb)
        assert rw < tol and rb < tol, (l, rw, rb)
    print("codec gradient worst rel-L2 per tensor: %.3g" % worst)


@pytest.mark.parametrize("mode", [0, 1])
def test_rtm3d_snapshot_method_bit_exact(geo, orc, mode):
    v, e, d = random_model_3d(20, 17, 23, seed=11)
    kw = dict(npd=8, nt=150, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, fsx=6, fsy=8,
              fsz=2, dsx=7, ns=2, mute_tt=20)
    mo, io, _ = orc.rtm3d(v, e, d, mode=mode, snap_every=4, **kw)
    mg, ig = geo.rtm3d(v, e, d, mode=mode, laplace=False, illum=True, method="snapshot", snap_every=4, **kw)
    assert np.abs(mo).max() > 0
    assert np.array_equal(ig, io)
    assert np.array_equal(mg, mo)


N3 = 64
FD = dict(npd=16, dx=10.0, dy=10.0, dz=10.0, dt=8e-4, favg=15.0, fsz=1, mode="fast", sv=1)


@pytest.fixture(scope="module")
def trained(geo):
    """A codec trained on snapshots of 6 seeded random media."""
    from geophysics_gb300 import media
    codec = geo.Codec(seed=1)
    codec.reserve(40000)
    rng = np.random.default_rng(1)
    for s in range(6):
        v, e, d = media.random_vti(N3, N3, N3, seed=100 + s, corr=float(rng.uniform(8, 30)))
        plan = geo.FD3DPlan(nx=N3, ny=N3, nz=N3, nt=360, fsx=int(rng.integers(12, N3 - 12)),
                            fsy=int(rng.integers(12, N3 - 12)), **FD)
        plan.set_model(v, e, d)
        codec.add_shot(plan, 0, snap_every=8, t_first=16)
        plan.close()
    assert codec.num_blocks() > 1000
    loss = codec.train(2000, batch=256, lr=2e-3)
    return codec, loss


def test_codec_training_reduces_loss(trained):
    _, loss = trained
    assert np.isfinite(loss).all()
    assert loss[-20:].mean() < 0.05 * loss[:20].mean()


def test_learned_rtm_gains_over_untrained(geo, trained):
    """The trained codec's image is far closer to the stored-snapshot image
    than an untrained codec's, with 16x less snapshot memory."""
    from geophysics_gb300 import media
    codec, _ = trained
    v, e, d = media.random_vti(N3, N3, N3, seed=7, corr=20.0)
    kw = dict(FD, nt=360, fsx=25, fsy=35, mute_tt=40, laplace=False)
    ref = geo.rtm3d(v, e, d, method="snapshot", snap_every=4, **kw)
    got = geo.rtm3d(v, e, d, method="learned", snap_every=4, codec=codec, **kw)
    raw = geo.rtm3d(v, e, d, method="learned", snap_every=4, codec=geo.Codec(seed=5), **kw)
    assert np.isfinite(got).all()
    e_trained, e_untrained = rel_l2(got, ref), rel_l2(raw, ref)
    assert e_trained < 0.25 * e_untrained, (e_trained, e_untrained)


def test_learned_rtm_with_every_block_escaped_matches_snapshots(geo, trained):
    """With every block keeping its bf16 residual the coded snapshots equal
    the stored ones up to bf16 rounding of the residual."""
    from geophysics_gb300 import media
    codec, _ = trained
    v, e, d = media.random_vti(N3, N3, N3, seed=8, corr=15.0)
    kw = dict(FD, nt=240, fsx=30, fsy=30, mute_tt=40, laplace=False)
    ref = geo.rtm3d(v, e, d, method="snapshot", snap_every=4, **kw)
    codec.set_escape(0.0, 1.0)
    b0, e0 = codec.stats()
    got = geo.rtm3d(v, e, d, method="learned", snap_every=4, codec=codec, **kw)
    b1, e1 = codec.stats()
    codec.set_escape()
    assert e1 - e0 > 0.5 * (b1 - b0)
    assert rel_l2(got, ref) < 2e-3


def test_codec_roundtrip_escape_budget(geo, trained):
    import torch
    codec, _ = trained
    rng = np.random.default_rng(2)
    vol = torch.from_numpy(rng.normal(size=(32, 48, 40)).astype(np.float32)).cuda()   # ragged z blocks
    codec.set_escape(0.0, 0.25)
    out, ne = codec.roundtrip(vol, escape=True)
    codec.set_escape()
    nb = 2 * 3 * 3
    assert ne == int(np.ceil(0.25 * nb))
    base = codec.roundtrip(vol)
    assert rel_l2(out.cpu().numpy(), vol.cpu().numpy()) < rel_l2(base.cpu().numpy(), vol.cpu().numpy())
