"""Shot-parallel RTM over ranks, one GPU per rank (torch.distributed).

The MPI RTM program deals shots round-robin (`for(is=1+myid; is<=ns;
is+=numprocs)`, 2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:295), stacks its
shots' images in shot order on every rank and sums the partial stacks on
rank 0 (`MPI_Reduce(..., MPI_SUM, 0, ...)`, :396-399).  Here each rank runs
its shots as one batched launch, the partial stacks are all-gathered and
rank 0 adds them in rank order (r0 + r1 + ...: deterministic, and for two
ranks the same sum any reduction order gives), then applies the adjoint
Laplacian.  The image sum is the only exchange; there is no collective in the
time loop.
"""
import numpy as np


def rank_shots(ns, rank, world):
    """0-based indices of the shots rank `rank` of `world` runs."""
    return list(range(rank, ns, world))


def reduce_images(partial, group=None, dst=0):
    """Sum the ranks' partial stacks in rank order on rank `dst` (returns
    the sum there, None elsewhere).  `partial`: numpy array or tensor."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    t = partial if isinstance(partial, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(partial))
    bufs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(bufs, t.contiguous(), group=group)
    if rank != dst:
        return None
    out = bufs[0].clone()
    for b in bufs[1:]:
        out += b
    return out


def rtm2d_sharded(v, e, d, *, shot_x, shot_nxs, laplace=True, group=None, compute=None, laplace_fn=None, **kw):
    """Batched 2D RTM (MPI-program semantics) with the shots dealt over the
    ranks of `group`; returns the stacked (Laplacian-filtered) image on rank
    0 and None elsewhere.

    compute(indices) -> partial stack of those shots, in shot order
    (default: `rtm2d_batch` on this rank's GPU); laplace_fn(image) -> the
    adjoint Laplacian (default: `laplace2d` on the GPU)."""
    import torch.distributed as dist
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    idx = rank_shots(len(shot_x), rank, world)
    if compute is None:
        from .api import laplace2d, rtm2d_batch

        def compute(ii):
            if not ii:
                return np.zeros(np.shape(v), np.float32)
            img = rtm2d_batch(v, e, d, shot_x=[shot_x[i] for i in ii], shot_nxs=[shot_nxs[i] for i in ii],
                              laplace=False, **kw)
            return img.cpu().numpy() if hasattr(img, "cpu") else img
        if laplace_fn is None:
            laplace_fn = laplace2d
    part = compute(idx)
    img = reduce_images(part, group=group)
    if img is None:
        return None
    img = img.numpy()
    if laplace:
        img = laplace_fn(img)
    return img
