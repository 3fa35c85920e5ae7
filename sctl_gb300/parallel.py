"""Multi-rank forms of the direct sum (one process per GPU).

`eval_direct` restates ParticleFMM::EvalDirect (fmm-wrapper.txx:551-623) over
torch.distributed: targets and sources are partitioned evenly by global count
(:565-571), source blocks travel round a ring of np steps (:598-617) and each
rank adds every visiting block's contribution to its own targets with the
local evaluator (the GPU library by default).  `partition_blocks` shards a
near list's independent blocks across ranks (longest-processing-time first by
interactions, no data exchange: each block owns its targets).  `max_over_ranks`
is the timing reduction bench.py uses for replicas.  Covered on CPU with the
gloo backend.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def partition_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's share of n items (fmm-wrapper.txx:565-569)."""
    return n * rank // world, n * (rank + 1) // world


def partition_blocks(blocks, world: int):
    """Indices of the near blocks (rows of (src_begin, src_count, trg_begin, trg_count)) each of
    `world` ranks evaluates: largest first (Ns x Nt interactions), each to the least-loaded rank
    so far; every rank's list in ascending block order.  Deterministic (ties to the lower rank)."""
    import heapq

    import numpy as np
    b = np.asarray(blocks, dtype=np.int64).reshape(-1, 4)
    cost = b[:, 1] * b[:, 3]
    order = np.argsort(-cost, kind="stable")
    heap = [(0, r) for r in range(world)]
    own = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        own[r].append(int(i))
        heapq.heappush(heap, (load + int(cost[i]), r))
    return [np.array(sorted(o), dtype=np.int64) for o in own]


def max_over_ranks(x: float, group=None) -> float:
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def _send_recv(x: torch.Tensor, offset: int, group=None) -> torch.Tensor:
    """Send x to rank+offset, receive the block of rank-offset (counts first, as :584-597)."""
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    if offset % world == 0:
        return x
    dst, src = (rank + offset) % world, (rank - offset) % world
    cnt_out = torch.tensor([x.numel()], dtype=torch.int64, device=x.device)
    cnt_in = torch.zeros(1, dtype=torch.int64, device=x.device)
    reqs = [dist.isend(cnt_out, dst, group=group, tag=2 * offset), dist.irecv(cnt_in, src, group=group, tag=2 * offset)]
    for r in reqs:
        r.wait()
    y = torch.empty(int(cnt_in.item()), dtype=x.dtype, device=x.device)
    reqs = [dist.isend(x.contiguous(), dst, group=group, tag=2 * offset + 1),
            dist.irecv(y, src, group=group, tag=2 * offset + 1)]
    for r in reqs:
        r.wait()
    return y


def eval_direct(evaluator, r_trg: torch.Tensor, r_src: torch.Tensor, n_src: torch.Tensor, v_src: torch.Tensor,
                trg_dim: int, group=None) -> torch.Tensor:
    """Distributed direct sum over a ring of ranks.  Each rank passes its local
    targets and its local share of the sources; returns this rank's potentials.
    `evaluator(v_trg, r_trg, r_src, n_src, v_src)` adds into v_trg (the
    reference's Eval contract, e.g. sctl_gb300.Laplace3D_DxU.Eval)."""
    world = dist.get_world_size(group)
    v = torch.zeros(r_trg.numel() // 3 * trg_dim, dtype=r_trg.dtype, device=r_trg.device)
    for i in range(world):
        xs, xn, f = (_send_recv(t.reshape(-1), i, group) for t in (r_src, n_src, v_src))
        if xs.numel():
            evaluator(v, r_trg, xs, xn, f)
    return v
