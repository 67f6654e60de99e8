"""Shot-parallel 2D RTM host logic on two gloo ranks (CPU): round-robin
dealing, rank-ordered image sum, Laplacian on rank 0, and a rank that dies
before the exchange is reported rather than waited for."""
import datetime
import socket

import numpy as np
import pytest

from tests.util import layered_model, rel_l2

NX, NZ, NPD, NT = 120, 60, 20, 700   # the MPI-form mute spans ~300 samples
SHOT_X = [41, 52, 63, 74, 85]
WIDTHS = [41, 51, 45, 61, 41]
KW = dict(npd=NPD, nt=NT, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=10.0, zs_sxd=5)


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _partial(orc, v, e, d, idx):
    full = np.zeros((NX, NZ), np.float32)
    for i in idx:
        mig, off, _ = orc.rtm2d_mpi_shot(v, e, d, fs_sxd=SHOT_X[i], ds_sxd=0, is_=1, nxs=WIDTHS[i], **KW)
        orc.stack2d(full, mig, off)
    return full


def _worker(rank, world, port, q, fail_rank):
    import torch.distributed as dist

    from geophysics_gb300.shots import rtm2d_sharded
    from oracle import orc
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    v, e, d = layered_model(NX, NZ, seed=7)
    if rank == fail_rank:
        raise SystemExit(3)        # leaves before the image exchange
    try:
        img = rtm2d_sharded(v, e, d, shot_x=SHOT_X, shot_nxs=WIDTHS,
                            compute=lambda ii: _partial(orc, v, e, d, ii), laplace_fn=orc.laplace2d_adj)
        if rank == 0:
            q.put(("ok", img))
    except Exception as exc:   # reported to the test, not waited for
        if rank == 0:
            q.put(("error", repr(exc)))
    dist.destroy_process_group()


def _run(fail_rank):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, fail_rank)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    return out, [p.exitcode for p in procs]


def test_round_robin_dealing():
    from geophysics_gb300.shots import rank_shots
    assert rank_shots(5, 0, 2) == [0, 2, 4]
    assert rank_shots(5, 1, 2) == [1, 3]
    assert rank_shots(2, 3, 4) == []
    assert sorted(sum((rank_shots(7, r, 3) for r in range(3)), [])) == list(range(7))


def test_two_ranks_match_rank_ordered_sum(orc):
    (kind, img), codes = _run(fail_rank=-1)
    assert kind == "ok" and codes == [0, 0]
    v, e, d = layered_model(NX, NZ, seed=7)
    r0 = _partial(orc, v, e, d, [0, 2, 4])
    r1 = _partial(orc, v, e, d, [1, 3])
    assert np.array_equal(img, orc.laplace2d_adj(r0 + r1))
    one = _partial(orc, v, e, d, range(5))
    assert np.abs(one).max() > 0
    assert rel_l2(img, orc.laplace2d_adj(one)) < 1e-5


def test_dead_rank_is_reported(orc):
    (kind, msg), codes = _run(fail_rank=1)
    assert kind == "error", msg
    assert codes[1] == 3
