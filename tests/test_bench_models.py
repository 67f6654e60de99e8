"""The synthetic media of the bench workloads have the properties their
descriptions state (built on the CPU here, at small sizes)."""
import numpy as np


def test_tti_model_ranges_and_stability_condition():
    import bench
    v, e, d, th, ph = (a.numpy() for a in bench.tti_model((40, 36, 30), device="cpu"))
    assert 1500 <= v.min() and v.max() <= 4500 + 1e-3
    assert 0 <= e.min() and e.max() <= 0.3 + 1e-6
    assert -0.05 - 1e-6 <= d.min() and d.max() <= 0.15 + 1e-6
    assert (d < e).all()                      # the pseudo-acoustic TTI scheme needs del < eps
    assert 0 <= th.min() and th.max() <= 45 and 0 <= ph.min() and ph.max() <= 360
    # smooth: neighbouring tilt values differ by a small fraction of the range
    assert np.abs(np.diff(th, axis=2)).max() < 5.0


def test_vti_model_ranges():
    import bench
    v, e, d = (a.numpy() for a in bench.make_model(shape=(32, 30, 28), device="cpu"))
    assert 1500 <= v.min() and v.max() <= 4500 + 1e-3
    assert (d <= e + 1e-7).all()
