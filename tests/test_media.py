"""Model generators (host-side numpy) against the reference generators'
rules, read from utils-getBinaryMedia-c and 3D-vti-fd+rtm-cuda/Toa_vel3.c."""
import numpy as np

from geophysics_gb300 import media


def test_vti_layers_media():
    v, e, d = media.vti_layers_media(3)
    assert v.shape == (3, 2500) and v.dtype == np.float32
    assert v[0, 500] == 2000 and v[0, 501] == 2600 and v[0, 1001] == 3300 and v[0, 2001] == 4500
    assert e[2, 1501] == np.float32(0.19) and d[1, 2499] == np.float32(0.1) and d[0, 0] == 0


def test_anticline_profiles():
    z = media.anticline_profile(601, 150, 250, 350, 450, 150, 200)
    assert z[0] == 150 and z[149] == 150 and z[200] == 175 and z[250] == 200 and z[349] == 200
    assert z[400] == 175 and z[450] == 150 and z[600] == 150
    z3 = media.anticline_profile(201, 25, 75, 125, 175, 100, 125)
    assert z3[25] == 100 and z3[50] == np.float32(112.5) and z3[75] == 125 and z3[150] == np.float32(112.5)


def test_interface_model_curved_and_3d():
    top = media.anticline_profile(40, 10, 15, 25, 30, 20, 10)
    a = media.interface_model(40, 35, (top, 30), (2.0, 3.0), 1.0, ny=4)
    assert a.shape == (4, 40, 35)
    assert a[0, 0, 20] == 1.0 and a[0, 0, 21] == 2.0 and a[3, 20, 11] == 2.0 and a[3, 20, 31] == 3.0
    assert np.array_equal(a[0], a[3])
