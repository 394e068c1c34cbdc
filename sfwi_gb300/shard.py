"""Shots over several GPUs: one process per GPU, each advancing its share of
the shots in one batch, then one sum of the gradients and the misfit.

This replaces the reference's MPI task farm (sfwi-stage1/main.cpp:534-635,
the master hands shots to workers one at a time) and its reduction of the
gradient buffers (main.cpp:637-666).  Shots are independent, so the only
exchange is the final sum: `partition` splits the shot list by cost (padded
cells x time steps, largest first onto the least-loaded rank) and
`allreduce_gradients` sums the per-rank FP64 gradients and misfits with
torch.distributed (NCCL between GPUs, gloo on the host).
"""
import numpy as np


def shot_cost(shot, pml, nzpml, nt):
    """Work of one shot-gradient: padded cells times time steps."""
    return (int(shot["nx"]) + 2 * pml) * nzpml * nt


def partition(costs, world):
    """Assign shots to ranks, largest first onto the least-loaded rank;
    returns per-rank lists of shot indices in ascending order."""
    if world < 1:
        raise ValueError("world size must be positive")
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(v) for v in out]


def allreduce_gradients(arrays, misfit, group=None):
    """Sum FP64 arrays and the misfit over the ranks of `group` in place
    (one collective: the values are packed into one buffer); returns the
    summed misfit."""
    import torch
    import torch.distributed as dist
    flat = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in arrays]
    buf = torch.from_numpy(np.concatenate(flat + [np.array([misfit], np.float64)]))
    if dist.get_backend(group) == "nccl":
        buf = buf.cuda()
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    buf = buf.cpu().numpy()
    o = 0
    for a, f in zip(arrays, flat):
        a.reshape(-1)[:] = buf[o:o + f.size]
        o += f.size
    return float(buf[o])


def run_sharded(fd, shots, rank, world, group=None):
    """One gradient pass over `shots` (dicts with the enqueue_shot fields and
    records) on this rank's engine `fd`: enqueue this rank's share, run, then
    sum the FP64 gradients and the misfit over the ranks.  Returns
    (misfit, (grad_pp, grad_ps, illum)), identical on every rank."""
    pml, nzpml, nt = fd.pml, fd.nzpml, fd.nt
    mine = partition([shot_cost(d, pml, nzpml, nt) for d in shots], world)[rank]
    for i in mine:
        d = shots[i]
        fd.enqueue_shot(d["nx"], d["isx"], d["isz"], d["igz"], d["ngx_left"], d["delta_left"], 0, d["gc"],
                        d["obs_z"], d["obs_x"])
    m = 0.0
    if mine:
        m, _ = fd.run()
    grads = [np.array(g, dtype=np.float64) for g in fd.read_gradients_f64()]
    fd.imagebuffer_resettozero()
    total = allreduce_gradients(grads, m, group)
    return total, tuple(grads)
