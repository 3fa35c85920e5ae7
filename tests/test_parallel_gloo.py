"""World-size-2 gloo runs of the multi-rank direct sum (ring over ranks, as
ParticleFMM::EvalDirect), of near blocks sharded across ranks, and of the
max-over-ranks timing reduction, on CPU with the oracle as the per-rank
evaluator."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, kernel, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from sctl_gb300 import parallel as P
        from sctl_gb300 import workloads as W
        d = W.sphere_ball(701, 333, kernel, seed=5)
        nd, sd, td = O.DIMS[kernel]
        t0, t1 = P.partition_range(333, rank, world)
        s0, s1 = P.partition_range(701, rank, world)
        tt = lambda a: torch.from_numpy(np.ascontiguousarray(a))  # noqa: E731

        def evaluator(v, xt, xs, xn, f):
            res = O.eval(kernel, xt.numpy(), xs.numpy(), xn.numpy() if nd else None, f.numpy(),
                         v_trg=v.numpy().copy())
            v.copy_(torch.from_numpy(res))

        v = P.eval_direct(evaluator, tt(d["r_trg"][t0:t1]), tt(d["r_src"][s0:s1]),
                          tt(d["n_src"][s0:s1] if nd else np.zeros((0, 3))), tt(d["v_src"][s0:s1]), td)
        ref = O.eval(kernel, d["r_trg"][t0:t1], d["r_src"], d["n_src"], d["v_src"])
        m = P.max_over_ranks(float(rank + 1))
        out_q.put((rank, float(O.rel_l2(v.numpy(), ref)), m))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kernel", [1, 2])
def test_ring_eval_direct_world2(kernel):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, kernel, q)) for r in range(2)]
    [p.start() for p in procs]
    res = [q.get(timeout=120) for _ in range(2)]
    [p.join(timeout=60) for p in procs]
    assert all(p.exitcode == 0 for p in procs)
    for rank, err, m in res:
        assert err < 1e-13, (rank, err)
        assert m == 2.0


def test_partition_range_matches_reference_rule():
    from sctl_gb300.parallel import partition_range
    n, world = 1001, 7
    parts = [partition_range(n, r, world) for r in range(world)]
    assert parts[0][0] == 0 and parts[-1][1] == n
    assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
    assert max(b - a for a, b in parts) - min(b - a for a, b in parts) <= 1


def _blocks_worker(rank, world, port, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from sctl_gb300 import parallel as P
        from sctl_gb300 import workloads as W
        d = W.near_blocks(40, 1, seed=9)
        nt = d["r_trg"].shape[0]
        mine = P.partition_blocks(d["blocks"], world)[rank]
        v = np.zeros(nt)
        for s0, n, t0, m in d["blocks"][mine]:  # this rank's blocks, evaluated locally
            v[t0:t0 + m] = O.eval(1, d["r_trg"][t0:t0 + m], d["r_src"][s0:s0 + n], d["n_src"][s0:s0 + n],
                                  d["v_src"][s0:s0 + n])
        tot = torch.from_numpy(v)
        dist.all_reduce(tot)  # only to compare: the blocks' targets are disjoint, so this is a gather
        ref = np.zeros(nt)
        for s0, n, t0, m in d["blocks"]:
            ref[t0:t0 + m] = O.eval(1, d["r_trg"][t0:t0 + m], d["r_src"][s0:s0 + n], d["n_src"][s0:s0 + n],
                                    d["v_src"][s0:s0 + n])
        out_q.put((rank, float(np.abs(tot.numpy() - ref).max()), len(mine)))
    finally:
        dist.destroy_process_group()


def test_near_blocks_sharded_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_blocks_worker, args=(r, 2, port, q)) for r in range(2)]
    [p.start() for p in procs]
    res = [q.get(timeout=120) for _ in range(2)]
    [p.join(timeout=60) for p in procs]
    assert all(p.exitcode == 0 for p in procs)
    assert sum(n for _, _, n in res) == 40
    for rank, err, _ in res:
        assert err == 0.0, (rank, err)


def test_partition_blocks_covers_and_balances():
    from sctl_gb300 import workloads as W
    from sctl_gb300.parallel import partition_blocks
    b = W.near_blocks(4096, 1, seed=0)["blocks"]
    cost = b[:, 1] * b[:, 3]
    for world in (1, 2, 3, 8):
        parts = partition_blocks(b, world)
        allidx = np.concatenate(parts)
        assert np.array_equal(np.sort(allidx), np.arange(len(b)))
        loads = np.array([cost[p].sum() for p in parts])
        assert loads.max() <= 1.01 * loads.mean() + cost.max()
        assert all(np.all(np.diff(p) > 0) for p in parts)
    assert [p.tolist() for p in partition_blocks(b[:50], 4)] == [p.tolist() for p in partition_blocks(b[:50], 4)]



def _dying_worker(rank, world, port, out_q):
    import datetime
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    if rank == 1:  # this rank fails between steps, before the ring starts, and exits
        out_q.put((rank, "died"))
        out_q.close()
        out_q.join_thread()
        os._exit(3)
    try:
        from sctl_gb300 import parallel as P
        x = torch.zeros(6, dtype=torch.float64)
        P.eval_direct(lambda *a: None, x, x, x, torch.zeros(2, dtype=torch.float64), 1)
        out_q.put((rank, "no error"))
    except Exception as e:  # the peer's loss surfaces as an error on the ring, not a hang
        out_q.put((rank, "error: " + type(e).__name__))


def test_ring_reports_a_lost_rank():
    """A rank that dies before the ring makes the other rank's exchange fail with an error within
    the process-group timeout instead of hanging (failure detected on the host)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_dying_worker, args=(r, 2, port, q)) for r in range(2)]
    [p.start() for p in procs]
    try:
        res = dict(q.get(timeout=120) for _ in range(2))
        [p.join(timeout=60) for p in procs]
    finally:
        for p in procs:  # never leave a rank behind, whatever happened
            if p.is_alive():
                p.terminate()
    assert res[1] == "died" and procs[1].exitcode == 3
    assert res[0].startswith("error"), res[0]
