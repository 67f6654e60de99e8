"""Failure detection during propagation: the wavefield watchdog and the
stability checks of the reference's set-up code.

Divergence is made on the host side of the physics, never by a fault: a
pseudo-acoustic VTI medium with delta > epsilon is unstable (in the
reference as much as here) and overflows to Inf within a few hundred
steps.  The watchdog sees it at its next scan, the run stops queueing
steps and returns GEO_ERR_NAN; the context stays usable."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEO_ERR_CFL, GEO_ERR_NAN = 5, 8


def _unstable3d(n=24):
    v = np.full((n, n, n), 2500.0, np.float32)
    return v, np.zeros_like(v), np.full_like(v, 0.4)


def _step_of(err):
    m = re.search(r"by time step (\d+)", str(err))
    return int(m.group(1)) if m else None


KW3 = dict(npd=8, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0, fsx=12, fsy=12, fsz=3)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_fd3d_watchdog_stops_a_diverging_shot(geo, mode):
    v, e, d = _unstable3d()
    with pytest.raises(geo.GeoError) as ei:
        geo.fd3d_shot(v, e, d, nt=2000, mode=mode, **KW3)
    assert ei.value.status == GEO_ERR_NAN, str(ei.value)
    assert _step_of(ei.value) in (100, 200, 300), str(ei.value)
    # the context and the library still compute correctly afterwards
    from tests.util import random_model_3d
    vs, es, ds = random_model_3d(24, 24, 24, seed=1)
    out = geo.fd3d_shot(vs, es, ds, nt=150, mode=mode, **KW3)
    assert np.isfinite(out).all() and np.abs(out).max() > 0


def test_fd3d_watchdog_interval_and_off(geo, monkeypatch):
    v, e, d = _unstable3d()
    monkeypatch.setenv("GEO_WATCH_EVERY", "50")
    with pytest.raises(geo.GeoError) as ei:
        geo.fd3d_shot(v, e, d, nt=1000, mode="fast", **KW3)
    assert ei.value.status == GEO_ERR_NAN and _step_of(ei.value) % 50 == 0
    # off: the run completes as the reference's would, with non-finite values
    monkeypatch.setenv("GEO_WATCH_EVERY", "0")
    out = geo.fd3d_shot(v, e, d, nt=600, mode="fast", **KW3)
    assert not np.isfinite(out).all()


def test_fd3d_watchdog_checks_the_last_step(geo):
    """nt not a multiple of the interval: the last step is scanned too."""
    v, e, d = _unstable3d()
    with pytest.raises(geo.GeoError) as ei:
        geo.fd3d_shot(v, e, d, nt=399, mode="fast", **KW3)
    assert ei.value.status == GEO_ERR_NAN


def test_rtm3d_watchdog(geo):
    v, e, d = _unstable3d(20)
    kw = dict(KW3, fsx=10, fsy=10)
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm3d(v, e, d, nt=700, method="boundary", **kw)
    assert ei.value.status == GEO_ERR_NAN


def _unstable2d(nx=48, nz=48):
    v = np.full((nx, nz), 2500.0, np.float32)
    return v, np.zeros_like(v), np.full_like(v, 0.4)


KW2 = dict(npd=10, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=24.0, zs=5.0)


@pytest.mark.parametrize("variant", ["cpu", "gpu", "mpi"])
@pytest.mark.parametrize("snap_every", [0, 50])
def test_fd2d_watchdog(geo, variant, snap_every):
    v, e, d = _unstable2d()
    with pytest.raises(geo.GeoError) as ei:
        geo.fd2d_shot(v, e, d, nt=1200, variant=variant, snap_every=snap_every, **KW2)
    assert ei.value.status == GEO_ERR_NAN, str(ei.value)


def test_tti2d_watchdog(geo):
    v, e, d = _unstable2d()
    th = np.full_like(v, 20.0)
    with pytest.raises(geo.GeoError) as ei:
        geo.tti2d_shot(v, e, d, th, nt=1200, **KW2)
    assert ei.value.status == GEO_ERR_NAN


def test_rtm2d_batch_watchdog(geo):
    nx, nz = 121, 40
    v = np.full((nx, nz), 2500.0, np.float32)
    e, d = np.zeros_like(v), np.full_like(v, 0.4)
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm2d_batch(v, e, d, npd=12, nt=900, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=1000.0, zs=1,
                        shot_x=[41, 81], shot_nxs=[41, 51])
    assert ei.value.status == GEO_ERR_NAN, str(ei.value)
    assert "forward" in str(ei.value)


def test_rtm2d_gpu_watchdog(geo):
    v, e, d = _unstable2d(60, 40)
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm2d_gpu(v, e, d, npml=15, nt=900, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, fs=30, zs=2)
    assert ei.value.status == GEO_ERR_NAN, str(ei.value)


def test_stability_condition_refused_everywhere(geo):
    """dt*vmax*sqrt(sum 1/d^2) >= 0.777 (the set-up code's limit for the
    8th-order operator) is refused with GEO_ERR_CFL before any step."""
    from tests.util import layered_model, random_model_3d
    v3, e3, d3 = random_model_3d(20, 20, 20, seed=2, vlo=2000, vhi=4500)
    with pytest.raises(geo.GeoError) as ei:       # 0.002*4500*sqrt(3)/10 = 1.56
        geo.fd3d_shot(v3, e3, d3, nt=20, **dict(KW3, dt=np.float32(2e-3), fsx=10, fsy=10))
    assert ei.value.status == GEO_ERR_CFL
    v, e, d = layered_model(50, 40, seed=1)        # vp up to 4000: 0.002*4000*sqrt(2)/10 = 1.13
    for variant in ("cpu", "gpu", "mpi"):
        with pytest.raises(geo.GeoError) as ei:
            geo.fd2d_shot(v, e, d, nt=20, variant=variant, **dict(KW2, dt=np.float32(2e-3)))
        assert ei.value.status == GEO_ERR_CFL
    with pytest.raises(geo.GeoError) as ei:
        geo.rtm2d_batch(v, e, d, npd=12, nt=20, dx=10.0, dz=10.0, dt_ms=2.0, favg=20.0, pfac=1000.0, zs=1,
                        shot_x=[25], shot_nxs=[21])
    assert ei.value.status == GEO_ERR_CFL
    with pytest.raises(geo.GeoError) as ei:
        geo.tti2d_shot(v, e, d, np.full_like(v, 10.0), nt=20, **dict(KW2, dt=np.float32(2e-3)))
    assert ei.value.status == GEO_ERR_CFL


def test_cpu_program_limits(geo):
    """CPU_vti2dfd's get_constant limits (spacing above vmin/favg*0.2, dt
    above 0.5*min(d)/vmax) are refused for the CPU form only: the program
    leaves its sponge constant undefined there; the GPU programs have no
    such check."""
    from tests.util import layered_model
    v, e, d = layered_model(50, 40, seed=1)        # vmin >= 2000: 2000/150*0.2 = 2.7 < 10
    with pytest.raises(geo.GeoError) as ei:
        geo.fd2d_shot(v, e, d, nt=20, variant="cpu", **dict(KW2, favg=150.0))
    assert ei.value.status == GEO_ERR_CFL
    out = geo.fd2d_shot(v, e, d, nt=20, variant="gpu", **dict(KW2, favg=150.0))
    assert np.isfinite(out).all()
