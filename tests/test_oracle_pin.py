"""The oracle against the reference's own CPU code (compiled unmodified into
oracle/_ref) and against the golden fixtures made from it.  CPU only."""
import os

import numpy as np
import pytest

from tests.util import layered_model

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _need_ref(orc):
    if not orc.ref_available():
        pytest.skip("reference tree not present (oracle/_ref not built)")


@pytest.mark.parametrize("sv", [0, 1])
def test_fd2d_cpu_variant_bit_exact_vs_CPU_vti2dfd(orc, sv):
    _need_ref(orc)
    v, e, d = layered_model(61, 51, seed=1)
    kw = dict(npd=20, nt=250, dx=10, dz=10, favg=20, fs=30, zs=5)
    ref, snaps = orc.ref_cpu_vti2dfd(v, e, d, dt_us=1000, sv=sv, **kw)
    mine, ms = orc.fd2d(v, e, d, dt=np.float32(1000 / 1e6), pfac=10.0, sv=sv, snap_every=50,
                        **{k: float(x) for k, x in kw.items() if k not in ("npd", "nt")}, npd=20, nt=250)
    assert np.array_equal(ref[0], mine)
    assert np.array_equal(snaps, ms)
    assert np.abs(mine).max() > 0.1


def test_fd2d_cpu_variant_two_shots(orc):
    _need_ref(orc)
    v, e, d = layered_model(71, 41, seed=4)
    ref, _ = orc.ref_cpu_vti2dfd(v, e, d, npd=12, nt=120, dx=10, dz=10, dt_us=1000, favg=25, fs=20, zs=3,
                                 ns=2, ds=15)
    for is_ in (1, 2):
        mine = orc.fd2d(v, e, d, npd=12, nt=120, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0,
                        fs=20.0, ds=15.0, zs=3.0, is_=is_)
        assert np.array_equal(ref[is_ - 1], mine)


def test_rtm2d_mpi_bit_exact_vs_reference(orc):
    _need_ref(orc)
    rng = np.random.default_rng(3)
    nx, nz = 101, 50
    v, e, d = layered_model(nx, nz, seed=3, vlo=2000, vhi=2600)
    v += rng.uniform(0, 40, v.shape).astype(np.float32)
    accr = np.zeros((nx, nz), np.float32)
    acco = np.zeros((nx, nz), np.float32)
    agr = np.zeros((90, nx, nz), np.float32)
    ago = np.zeros((90, nx, nz), np.float32)
    for is_, nxs in ((1, 41), (2, 53)):
        kw = dict(npd=15, nt=650, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0, fs_sxd=35, ds_sxd=20,
                  zs_sxd=1, is_=is_, nxs=nxs)
        mr, pr = orc.ref_rtm_mpi_shot(v, e, d, accr, adcig_acc=agr, **kw)
        mo, off, po, ag = orc.rtm2d_mpi_shot(v, e, d, adcig=True, **kw)
        orc.stack2d(acco, mo, off)
        for ia in range(90):
            orc.stack2d(ago[ia], ag[ia], off)
        assert np.array_equal(pr, po)
        assert np.array_equal(mr, mo)
    assert np.array_equal(accr, acco)
    # Poynting angle gathers (flag_adcig = 1): every angle plane bit-exact
    assert np.abs(agr).max() > 0 and (np.abs(agr).reshape(90, -1).max(axis=1) > 0).sum() > 10
    assert np.array_equal(agr, ago)
    assert np.array_equal(orc.ref_laplace2d_adj(accr), orc.laplace2d_adj(acco))


def test_laplace2d_vs_reference(orc):
    _need_ref(orc)
    img = np.random.default_rng(7).standard_normal((37, 23)).astype(np.float32)
    assert np.array_equal(orc.ref_laplace2d_adj(img), orc.laplace2d_adj(img))


def test_oracle_matches_golden_fixtures(orc):
    """Pins that hold without the reference tree (e.g. on the GPU machine)."""
    g = np.load(os.path.join(GOLD, "golden_fd2d_cpu.npz"))
    mine = orc.fd2d(g["v"], g["e"], g["d"], npd=int(g["npd"]), nt=int(g["nt"]), dx=10.0, dz=10.0,
                    dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=float(g["fs"]), zs=float(g["zs"]), sv=int(g["sv"]))
    # bit-exact on the machine that made them; libm may differ in the last
    # bit of the sponge profiles elsewhere, hence the tolerance
    assert np.abs(mine - g["shot"]).max() <= 1e-6 * np.abs(g["shot"]).max()
    r = np.load(os.path.join(GOLD, "golden_rtm2d_mpi.npz"))
    acc = np.zeros(r["v"].shape, np.float32)
    for is_, nxs in zip(r["shots"], r["widths"]):
        mo, off, _ = orc.rtm2d_mpi_shot(r["v"], r["e"], r["d"], npd=int(r["npd"]), nt=int(r["nt"]), dx=10.0, dz=10.0,
                                        dt_ms=1.0, favg=20.0, pfac=1000.0, fs_sxd=int(r["fs"]), ds_sxd=int(r["ds"]),
                                        zs_sxd=1, is_=int(is_), nxs=int(nxs))
        orc.stack2d(acc, mo, off)
    lap = orc.laplace2d_adj(acc)
    assert np.abs(lap - r["image"]).max() <= 1e-5 * np.abs(r["image"]).max()


def test_fp64_oracle_close_to_fp32(orc):
    v, e, d = layered_model(61, 51, seed=1)
    kw = dict(npd=20, nt=300, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=30.0, zs=5.0)
    a = orc.fd2d(v, e, d, prec=32, **kw)
    b = orc.fd2d(v, e, d, prec=64, **kw)
    err = np.linalg.norm(a - b) / np.linalg.norm(b)
    assert 0 < err < 1e-4


def test_fd3d_oracle_fast_vs_exact(orc):
    from tests.util import random_model_3d, rel_l2
    v, e, d = random_model_3d(20, 18, 22, seed=5)
    kw = dict(npd=8, nt=120, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0,
              fsx=10, fsy=9, fsz=3)
    a = orc.fd3d(v, e, d, mode=0, **kw)
    b = orc.fd3d(v, e, d, mode=1, **kw)
    assert np.abs(a).max() > 0
    assert rel_l2(b, a) < 1e-5
