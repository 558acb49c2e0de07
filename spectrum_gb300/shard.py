"""One job over several GPUs: one process per GPU, shards by trajectory id, one sum at the end.

Trajectories are independent, and their random streams are keyed by (seed, trajectory id,
problem id). Run k of a context draws the trajectory ids k * n_traj ... k * n_traj + n_traj - 1 of
each problem. A job of R runs per rank is therefore split exactly: rank r starts at run index
r * R (``SPX_OPT_RUN_INDEX``). The union of the ranks' trajectories is the trajectory set of one
context running W * R runs. No data moves while the kernels run. The only exchange is the sum of
the histograms afterwards, the analogue of the reference's reduction of its workers'
distributions (src/simulation.cc:173-177, DistributionTemplated::operator+=,
src/distribution_templated.cc:280-288).
"""
from __future__ import annotations

from . import capi


def first_run_index(rank: int, runs_per_rank: int) -> int:
    """Run index at which rank ``rank`` starts when every rank makes ``runs_per_rank`` runs."""
    if rank < 0 or runs_per_rank < 1:
        raise ValueError("rank >= 0 and runs_per_rank >= 1 required")
    return rank * runs_per_rank


def assign(sim, rank: int, runs_per_rank: int) -> None:
    """Point a context (SimulationGPU) at this rank's shard of trajectory ids."""
    sim.ctx.set_option(capi.SPX_OPT_RUN_INDEX, first_run_index(rank, runs_per_rank))


def combine_distributions(distros, group=None):
    """Sum per-rank distributions over all ranks (torch.distributed; every rank gets the sum).

    ``distros`` is a list over problems of lists over distributions of (counts, sums, n_events)
    tuples as ``Context.distribution`` returns them. Counts are summed as int64 (exact), sums as
    float64, event counts as int64."""
    import numpy as np
    import torch
    import torch.distributed as dist
    flat_c = [np.asarray(c, dtype=np.int64).ravel() for row in distros for c, _, _ in row]
    flat_s = [np.asarray(s, dtype=np.float64).ravel() for row in distros for _, s, _ in row]
    ne = np.array([n for row in distros for _, _, n in row], dtype=np.int64)
    c_t = torch.from_numpy(np.concatenate(flat_c) if flat_c else np.zeros(0, np.int64))
    s_t = torch.from_numpy(np.concatenate(flat_s) if flat_s else np.zeros(0, np.float64))
    n_t = torch.from_numpy(ne)
    backend_device = None
    if dist.get_backend(group) == "nccl":
        backend_device = torch.device("cuda", torch.cuda.current_device())
    for t in (c_t, s_t, n_t):
        tt = t.to(backend_device) if backend_device is not None else t
        dist.all_reduce(tt, op=dist.ReduceOp.SUM, group=group)
        if backend_device is not None:
            t.copy_(tt.cpu())
    out, oc, os_, k = [], 0, 0, 0
    for row in distros:
        r = []
        for c, s, _ in row:
            nb = np.asarray(c).size
            shape = np.asarray(s).shape
            ns = int(np.prod(shape))
            r.append((c_t[oc:oc + nb].numpy().copy(), s_t[os_:os_ + ns].numpy().reshape(shape).copy(),
                      int(n_t[k].item())))
            oc += nb
            os_ += ns
            k += 1
        out.append(r)
    return out


def max_over_ranks(value: float, group=None) -> float:
    """The maximum of a per-rank scalar (e.g. device seconds of the timed region)."""
    import torch
    import torch.distributed as dist
    dev = None
    if dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
