"""2D TTI on the GPU against the oracle (bit-exact).  The GPU TTI programs
form cos and sin of their tilt on the device; the oracle is given the
device's values (oracle.refgpu.cuda_trig) and restates the rest."""
import numpy as np
import pytest

from oracle.refgpu import cuda_angle_tables, cuda_trig
from tests.util import layered_model, rel_l2

pytestmark = pytest.mark.gpu

KW = dict(npd=20, nt=300, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=40, zs=10)


def _model(nx=90, nz=67, seed=3):
    v, e, d = layered_model(nx, nz, seed=seed)
    x, z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    theta = (25 + 20 * np.sin(x / 13.0) * np.cos(z / 9.0)).astype(np.float32)
    return v, e, d, theta


@pytest.mark.parametrize("sv", [0, 1])
def test_tti2d_bit_exact(geo, orc, sv):
    v, e, d, th = _model()
    ref, rs = orc.tti2d(v, e, d, th, sv=sv, snap_every=100, trig=cuda_trig(th), **KW)
    out, snaps = geo.tti2d_shot(v, e, d, th, sv=sv, snap_every=100, **KW)
    assert np.abs(ref).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)
    assert snaps.shape == rs.shape == (2, 130, 107)
    assert np.array_equal(snaps, rs)


def test_tti2d_device_buffers_and_second_shot(geo, orc):
    import torch
    v, e, d, th = _model(seed=4)
    kw = dict(KW, ds=7.0, is_=2, rec_iz=22)
    ref = orc.tti2d(v, e, d, th, trig=cuda_trig(th), **kw)
    t = [torch.from_numpy(a).cuda() for a in (v, e, d, th)]
    out = geo.tti2d_shot(*t, **kw)
    assert out.is_cuda
    assert np.array_equal(out.cpu().numpy(), ref)


def test_tti2d_source_on_receiver_row_large_grid(geo, orc):
    """The record row through the source cell (the step's source reaches the
    velocity taps only, never the recorded P), snapshots every 7 steps, and
    a grid of more points than one wave of resident threads, so each thread
    of the persistent launch strides over several points."""
    v, e, d, th = _model(nx=1100, nz=1000, seed=5)
    kw = dict(KW, nt=60, rec_iz=29)          # source cell row: (int)(zs + 0.5) + npd - 1
    ref, rs = orc.tti2d(v, e, d, th, snap_every=7, trig=cuda_trig(th), **kw)
    out, snaps = geo.tti2d_shot(v, e, d, th, snap_every=7, **kw)
    assert np.abs(ref).max() > 0
    assert np.array_equal(out, ref), rel_l2(out, ref)
    assert snaps.shape == rs.shape == (8, 1140, 1040)
    assert np.array_equal(snaps, rs)


def test_tti2d_receiver_row_outside_updated_band(geo, orc):
    v, e, d, th = _model(seed=6)
    kw = dict(KW, nt=40, rec_iz=2)
    ref = orc.tti2d(v, e, d, th, trig=cuda_trig(th), **kw)
    out = geo.tti2d_shot(v, e, d, th, **kw)
    assert np.array_equal(out, ref)
    assert not out.any()


def test_tti2d_rejects_bad_input(geo):
    v, e, d, th = _model()
    th[3, 4] = np.nan
    with pytest.raises(geo.GeoError):
        geo.tti2d_shot(v, e, d, th, **KW)


TKW = dict(npml=20, nt=600, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, ns=2, fs=30, ds=30, zs=2,
           mute_tt=30, nangle=65, dangle=1)


@pytest.mark.parametrize("dcdp", [1, 3])
def test_rtm2d_tti_program_bit_exact(geo, orc, dcdp):
    """The 2D TTI GPU RTM program (TTI stencil, ring saving, forward-stepped
    reconstruction, Poynting gathers at every dcdp-th CDP; nx = 91 is not a
    multiple of 3): image, illumination, gathers and records equal the
    oracle's."""
    v, e, d, th = _model(nx=91, nz=60, seed=5)
    mig, ill, ag, shots = orc.rtm2d_tti(v, e, d, th, dcdp=dcdp, trig=cuda_trig(th),
                                        **cuda_angle_tables(TKW["dangle"]), **TKW)
    out = geo.rtm2d_tti(v, e, d, th, dcdp=dcdp, **TKW)
    assert np.abs(ill).max() > 0 and np.abs(ag).max() > 0
    assert out["adcigs"].shape == (91 // dcdp, 65, 60)
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["illum"], ill)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag), rel_l2(out["adcigs"], ag)


def test_rtm2d_tti_program_thin_sponge_large_grid(geo, orc):
    """As the VTI program's case: npml = 5 (ring cells outside the updated
    band) on a grid larger than one wave of resident threads."""
    v, e, d, th = _model(nx=700, nz=400, seed=8)
    kw = dict(TKW, npml=5, ns=1, nt=150, fs=350)
    mig, ill, ag, shots = orc.rtm2d_tti(v, e, d, th, trig=cuda_trig(th), **cuda_angle_tables(kw["dangle"]), **kw)
    out = geo.rtm2d_tti(v, e, d, th, **kw)
    assert np.abs(ill).max() > 0
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["illum"], ill)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag), rel_l2(out["adcigs"], ag)


@pytest.mark.parametrize("every", ["0", "7", "1"])
def test_2d_programs_independent_of_launch_segments(geo, orc, monkeypatch, every):
    """The persistent launches end at every watchdog scan (GEO_WATCH_EVERY
    steps; 0: one launch per pass, 1: one launch per step), and a backward
    launch opens with the ring restore and record injection of its first
    step: the results are the oracle's whatever the segmentation."""
    monkeypatch.setenv("GEO_WATCH_EVERY", every)
    v, e, d, th = _model(nx=70, nz=50, seed=9)
    kw = dict(TKW, ns=1, nt=120)
    mig, ill, ag, shots = orc.rtm2d_tti(v, e, d, th, trig=cuda_trig(th), **cuda_angle_tables(kw["dangle"]), **kw)
    out = geo.rtm2d_tti(v, e, d, th, **kw)
    assert np.array_equal(out["shots"], shots)
    assert np.array_equal(out["mig_lap"], orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"], ag)
    ref, rs = orc.tti2d(v, e, d, th, snap_every=9, trig=cuda_trig(th), **dict(KW, nt=100))
    got, gs = geo.tti2d_shot(v, e, d, th, snap_every=9, **dict(KW, nt=100))
    assert np.array_equal(got, ref) and np.array_equal(gs, rs)


def test_rtm2d_tti_program_observed_shots_device(geo, orc):
    import torch
    v, e, d, th = _model(nx=80, nz=50, seed=6)
    kw = dict(TKW, ns=1, nt=400)
    obs = np.random.default_rng(7).standard_normal((1, 80, 400)).astype(np.float32) * 1e-3
    mig, ill, ag, _ = orc.rtm2d_tti(v, e, d, th, obs=obs, trig=cuda_trig(th), **cuda_angle_tables(kw["dangle"]), **kw)
    t = [torch.from_numpy(a).cuda() for a in (v, e, d, th, obs)]
    out = geo.rtm2d_tti(*t[:4], obs=t[4], **kw)
    assert out["mig_lap"].is_cuda
    assert np.array_equal(out["mig_lap"].cpu().numpy(), orc.laplace2d_adj(mig))
    assert np.array_equal(out["adcigs"].cpu().numpy(), ag)
