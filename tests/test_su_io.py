"""SU / SEG-Y trace files: round trips, header fields, the MPI program's
trace layout, and the binary2segy utility pinned against the reference's
own build (CPU)."""
import os
import subprocess

import numpy as np
import pytest

REF_B2S = os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "binary2segy")


@pytest.mark.parametrize("big", [True, False])
def test_su_roundtrip_and_header(geo, tmp_path, big):
    rng = np.random.default_rng(1)
    data = rng.standard_normal((7, 33)).astype(np.float32)
    p = str(tmp_path / "a.su")
    geo.su_write(p, data, dt_us=500.0, big_endian=big)
    raw = open(p, "rb").read()
    assert len(raw) == 7 * (240 + 33 * 4)
    order = ">" if big else "<"
    h = raw[240 + 33 * 4: 2 * 240 + 33 * 4]          # second trace header
    assert np.frombuffer(h[0:4], order + "i4")[0] == 2
    assert np.frombuffer(h[114:116], order + "u2")[0] == 33
    assert np.frombuffer(h[116:118], order + "u2")[0] == 500
    # trace i of ns samples starts at (i+1)*240 + i*ns*4 (read_v_e_d_r, seismic == 2)
    i = 4
    o = (i + 1) * 240 + i * 33 * 4
    assert np.array_equal(np.frombuffer(raw[o:o + 33 * 4], order + "f4"), data[i])
    back, hdr = geo.su_read(p, 7, 33, big_endian=big, headers=True)
    assert np.array_equal(back, data)
    q = str(tmp_path / "b.su")
    geo.su_write(q, data * 2, big_endian=big, headers=hdr)
    assert np.array_equal(geo.su_read(q, 7, 33, big_endian=big), data * 2)
    assert open(q, "rb").read()[:240] == raw[:240]


def test_su_errors(geo, tmp_path):
    with pytest.raises(geo.GeoError):
        geo.su_read(str(tmp_path / "missing.su"), 3, 10)
    p = str(tmp_path / "short.su")
    geo.su_write(p, np.zeros((2, 10), np.float32))
    with pytest.raises(geo.GeoError):
        geo.su_read(p, 3, 10)


@pytest.mark.skipif(not os.path.exists(REF_B2S), reason="reference utility not built (no reference tree)")
def test_replace_data_matches_reference_binary2segy(geo, tmp_path):
    ntr, ns = 1700, 601                   # the utility's fixed sizes
    rng = np.random.default_rng(2)
    hdr = rng.integers(0, 256, (ntr, 240), dtype=np.uint8)
    tmpl = np.concatenate([hdr, rng.standard_normal((ntr, ns)).astype(">f4").view(np.uint8)], axis=1)
    tmpl.tofile(tmp_path / "v1.su")
    rng.standard_normal((ntr, ns)).astype(np.float32).tofile(tmp_path / "v2.dat")
    # the utility's main() is void: its exit status means nothing, its output does
    subprocess.run([os.path.abspath(REF_B2S)], cwd=tmp_path, capture_output=True)
    ref = (tmp_path / "v2.su").read_bytes()
    geo.su_replace_data(str(tmp_path / "v1.su"), str(tmp_path / "v2.dat"), str(tmp_path / "mine.su"), ntr, ns)
    assert (tmp_path / "mine.su").read_bytes() == ref
