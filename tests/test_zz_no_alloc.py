"""geo_fd2d_shot_noalloc, the entry point for callers that cannot allocate
GPU memory (their device memory is reserved by their own pool, or their
framework forbids allocation outside its allocator).

It must give the same record as geo_fd2d_shot, bit for bit like every 2D
parity test here, on two calls in a row (the shared static work array keeps
the previous call's contents, so the second call checks that state is
cleared), and it must not change the device's free memory.

This file sorts last so a run that stops at the first failure has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest

from tests.util import layered_model

pytestmark = pytest.mark.gpu


def _desc(G, nx, nz, **kw):
    from geophysics_gb300._lib import FD2DDesc
    base = dict(nx=nx, nz=nz, npd=16, nt=220, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, wtype=1,
                fs=nx / 2, ds=0.0, zs=4.0, is_=1, variant=0, sv=0, rec_iz=16, rec_scale=2.0, mute_tt=0)
    base.update(kw)
    return FD2DDesc(**base)


def _run_noalloc(G, desc, tv, te, td, out):
    import torch
    st = torch.cuda.current_stream().cuda_stream
    return G.lib().geo_fd2d_shot_noalloc(C.byref(desc), C.c_void_p(tv.data_ptr()), C.c_void_p(te.data_ptr()),
                                         C.c_void_p(td.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(st))


def _run_existing(G, desc, tv, te, td, out):
    import torch
    st = torch.cuda.current_stream().cuda_stream
    return G.lib().geo_fd2d_shot(C.byref(desc), C.c_void_p(tv.data_ptr()), C.c_void_p(te.data_ptr()),
                                 C.c_void_p(td.data_ptr()), C.c_void_p(out.data_ptr()), None, 0, 1, C.c_void_p(st))


def test_noalloc_matches_existing_entry_point_twice(geo):
    import torch
    G = geo
    cases = [
        # CPU_vti2dfd semantics with the SV taper
        (layered_model(64, 52, seed=11), dict(variant=0, sv=1, rec_scale=2.0)),
        # GPU_vti2dfd semantics with the direct-wave mute, a different grid
        (layered_model(57, 40, seed=12), dict(variant=1, sv=1, rec_scale=1.0, mute_tt=100, npd=12, rec_iz=12,
                                             nt=180, fs=20.0, zs=5.0)),
    ]
    bufs = []
    for (v, e, d), kw in cases:
        nx, nz = v.shape
        desc = _desc(G, nx, nz, **kw)
        tv, te, td = (torch.from_numpy(a).cuda() for a in (v, e, d))
        ref = torch.empty((nx, desc.nt), dtype=torch.float32, device="cuda")
        out = torch.full((nx, desc.nt), 7.0, dtype=torch.float32, device="cuda")
        bufs.append((desc, tv, te, td, ref, out))
    for desc, tv, te, td, ref, _ in bufs:
        assert _run_existing(G, desc, tv, te, td, ref) == 0
    torch.cuda.synchronize()
    for k, (desc, tv, te, td, ref, out) in enumerate(bufs):
        free0 = torch.cuda.mem_get_info()[0]
        assert _run_noalloc(G, desc, tv, te, td, out) == 0, G.lib().geo_last_error()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.abs(b).max() > 0
        assert np.array_equal(a, b), "call %d differs" % k
        if k > 0:
            # modules are loaded by now: the call itself must not allocate
            assert free1 == free0
    # a repeat of the first case after the second (stale contents cleared)
    desc, tv, te, td, ref, out = bufs[0]
    assert _run_noalloc(G, desc, tv, te, td, out) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_rejects_sizes_beyond_the_limit(geo):
    import torch
    G = geo
    limit = G.lib().geo_fd2d_noalloc_limit()
    assert limit == 32 << 20
    nx, nz = 1200, 1200   # 11 full fields of ~1.27M points: > 32 MiB
    desc = _desc(G, nx, nz, nt=10)
    t = torch.ones((nx, nz), dtype=torch.float32, device="cuda")
    out = torch.empty((nx, 10), dtype=torch.float32, device="cuda")
    rc = _run_noalloc(G, desc, t, t, t, out)
    assert rc == 1
    assert b"limit" in G.lib().geo_last_error()
