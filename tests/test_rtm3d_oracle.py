"""CPU checks of the oracle's 3D RTM angle gathers (Poynting_Adcigs and
adcigs_illum of 3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu)."""
import math

import numpy as np
import pytest

from tests.util import random_model_3d

KW = dict(npd=8, nt=120, dx=10.0, dy=10.0, dz=10.0, dt=np.float32(1e-3), favg=25.0, pfac=10.0,
          fsx=6, fsy=7, fsz=2, ns=1, mute_tt=20)


@pytest.fixture(scope="module")
def runs(orc):
    v, e, d = random_model_3d(14, 13, 15, seed=21)
    full = orc.rtm3d(v, e, d, adcig=(90, 1, 1), **KW)
    dec = orc.rtm3d(v, e, d, adcig=(90, 1, 2), **KW)
    return full, dec


def test_gathers_leave_image_and_illumination_alone(orc, runs):
    v, e, d = random_model_3d(14, 13, 15, seed=21)
    mig, ill, rec = orc.rtm3d(v, e, d, **KW)
    full, _ = runs
    assert np.array_equal(full[0], mig) and np.array_equal(full[1], ill) and np.array_equal(full[2], rec)


def test_cdp_decimation_samples_the_full_gathers(runs):
    """dcdp = 2 keeps the gathers of every second CDP in x and y, unchanged
    (the illumination divisor is taken at the same points)."""
    (_, _, _, ag1), (_, _, _, ag2) = runs
    assert ag2.shape == (13 // 2, 14 // 2, 90, 15)
    assert np.abs(ag1).max() > 0
    assert np.array_equal(ag2, ag1[0:2 * (13 // 2):2, 0:2 * (14 // 2):2])


def test_opening_angle_range(runs):
    """Half opening angles lie in [0, 90) degrees; with na = 90 and da = 1
    the bins past 45 degrees are reached only by waves meeting head-on, and
    the near-normal bins carry energy."""
    (_, _, _, ag1), _ = runs
    per_bin = np.abs(ag1).sum(axis=(0, 1, 3))
    assert per_bin[:10].sum() > 0
    assert np.count_nonzero(per_bin) >= 10


def test_bin_function_restatement():
    """The program's bin, (int)((float)(0.5*acosf(a)*180/pi)/da), is
    non-increasing in the cosine a -- the property the GPU's threshold
    search relies on -- sampled over [-1, 1] in float."""
    pi = 3.141592653
    a = np.linspace(-1, 1, 20001, dtype=np.float32)
    for da in (1, 2, 3):
        b = np.array([int(np.float32(0.5 * math.acos(float(x)) * 180.0 / pi) / (da * 1.0)) for x in a])
        assert np.all(np.diff(b) <= 0)
        assert b[0] == int(90 / da) and b[-1] == 0
