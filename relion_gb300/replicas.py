"""Data-parallel E-step replicas: particle partitioning and the one exchange
step of an iteration.

Particles are independent given the model, so each rank (one GPU) runs the
E-step on a contiguous particle range with its own bundle and accumulates
its own FP64 weighted sums and backprojected volumes.  The only exchange is
the sum of those accumulators over the ranks of a half-set, after the
E-step: MlOptimiserMpi::combineAllWeightedSums (src/ml_optimiser_mpi.cpp:
2028-2100) packs wsum_model into one double vector and MPI_Allreduce-sums
it over the followers of each random half (node->splitC) or all followers
(node->followerC).  Here the packed vector is one torch.distributed
all_reduce (SUM) over the process group of the half-set: gloo with host
tensors, or NCCL with device tensors.
"""
import numpy as np


def divide_equally(n, size, rank):
    """[first, last] particle range of `rank` among `size` ranks, the first
    n % size ranks taking one extra (divide_equally, src/parallel.cpp:156-171)."""
    per, rest = divmod(int(n), int(size))
    if rank < rest:
        first = rank * (per + 1)
        last = first + per
    else:
        first = rank * per + rest
        last = first + per - 1
    return first, last


def half_set_ranks(world, do_split_random_halves):
    """Ranks of each half-set: odd/even split as the reference's followers
    (rank parity decides the random half), or one group of all ranks."""
    if not do_split_random_halves or world < 2:
        return [list(range(world))]
    return [list(range(0, world, 2)), list(range(1, world, 2))]


def _pack(wsum, volumes):
    parts, layout = [], []
    for k in sorted(wsum):
        a = np.asarray(wsum[k], dtype=np.float64)
        layout.append(("wsum", k, a.shape))
        parts.append(a.ravel())
    for i, (data, weight) in enumerate(volumes):
        d = np.asarray(data)
        layout.append(("data", i, d.shape))
        parts.append(np.ascontiguousarray(d, dtype=np.complex128).view(np.float64).ravel())
        w = np.asarray(weight, dtype=np.float64)
        layout.append(("weight", i, w.shape))
        parts.append(w.ravel())
    return np.concatenate(parts) if parts else np.zeros(0), layout


def _unpack(vec, layout):
    wsum, vols, pos = {}, {}, 0
    for kind, key, shape in layout:
        m = int(np.prod(shape)) if len(shape) else 1
        if kind == "data":
            a = vec[pos:pos + 2 * m].view(np.complex128).reshape(shape)
            pos += 2 * m
        else:
            a = vec[pos:pos + m].reshape(shape)
            pos += m
        if kind == "wsum":
            wsum[key] = float(a) if len(shape) == 0 else a.copy()
        else:
            vols.setdefault(key, [None, None])[0 if kind == "data" else 1] = a.copy()
    return wsum, [tuple(vols[i]) for i in sorted(vols)]


def combine_weighted_sums(wsum, volumes, group=None, device=None):
    """Sum the weighted sums (dict of scalars / arrays, as
    MlDeviceBundle.get_wsum returns) and the per-class (data, weight)
    volumes over the ranks of `group`.  Returns the summed (wsum, volumes);
    every rank of the group receives the same result.  `device`: torch
    device of the reduction buffer (a CUDA device for NCCL, None = host)."""
    import torch
    import torch.distributed as dist
    vec, layout = _pack(wsum, volumes)
    t = torch.from_numpy(vec)
    if device is not None:
        t = t.to(device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return _unpack(t.cpu().numpy().copy(), layout)


def max_over_ranks(values, device=None):
    """Element-wise maximum of a list of floats over all ranks (timing)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]
