"""C ABI: the library loads on a machine without a GPU and exports every
entry point include/geofd.h declares; host-only pieces (par file, status
strings) work without a GPU."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "geofd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "sizeof", "defined")))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("GPU_vti2dfd", "CPU_vti2dfd", "GPU_vti3dfd", "geo_fd2d_shot", "geo_fd3d_plan_create",
              "geo_rtm2d_batch", "geo_laplace2d", "geo_par_load"):
        assert n in names


def test_library_exports_every_declared_symbol(geo):
    L = geo.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(geo):
    L = geo.lib()
    assert L.geo_strerror(0) == b"ok"
    assert b"window" in L.geo_strerror(6)
    assert b"sm_103a" in L.geo_version()


def test_par_file(geo, tmp_path):
    p = tmp_path / "fd.par"
    p.write_text("        nx=   401\n  dx=  10.0\n# comment\nFNvelocity=   vel.dat  # trailing\n"
                 "  xstart,xend=  17751  59640\n")
    par = geo.read_par(str(p))
    assert par.int("nx") == 401
    assert abs(par.float("dx") - 10.0) < 1e-6
    assert par.str("FNvelocity") == "vel.dat"
    assert par.str("xstart,xend") == "17751  59640"
    import pytest
    with pytest.raises(geo.GeoError):
        par.int("nz")


def test_missing_file_is_an_io_error(geo, tmp_path):
    with __import__("pytest").raises(geo.GeoError) as ei:
        geo.read_par(str(tmp_path / "nope.par"))
    assert ei.value.status == 3


def test_par_runs_reject_incomplete_par_files(geo, tmp_path):
    """geo_fd2d / geo_fd3d / geo_rtm2d check their keys before touching a
    GPU: a missing key or an output nowhere to go is GEO_ERR_ARG."""
    import pytest
    p = tmp_path / "a.par"
    p.write_text("nx= 10\nnz= 10\n")
    for fn in (geo.fd2d_par, geo.fd3d_par, geo.rtm2d_par):
        with pytest.raises(geo.GeoError) as ei:
            fn(str(p))
        assert ei.value.status == 1
    q = tmp_path / "b.par"
    q.write_text("nx= 10\nnz= 10\ndx= 10\ndz= 10\nnpd= 20\nnt= 10\ndt= 1000\nfavg= 20\nns= 1\nfs= 5\nds= 0\n"
                 "zs= 1\nFNv= v\nFNe= e\nFNd= d\n")
    with pytest.raises(geo.GeoError) as ei:
        geo.fd2d_par(str(q))          # no FNshot and no device buffer
    assert ei.value.status == 1
