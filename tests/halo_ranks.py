"""Rank coupling for the subdomain tests: what MPI does for T-FlowS, done
with torch.distributed (gloo, host memory) between spawned processes.

exchange(sd)  -> phi -> None: swaps each connected neighbour's segment of
                 PHI(-NB:-1) with that rank in place, as MPI_SENDRECV_REPLACE
                 does in Parallel/Double/Exchng.f90:46-60.
glosum()      -> v -> sum over ranks (Parallel/Double/GloSum.f90).
run_ranks(fn, world, *args) spawns `world` processes that join a gloo group
on 127.0.0.1, run fn(rank, world, *args) and return its results by rank.
"""
import os
import socket
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def exchange(sd):
    import torch
    import torch.distributed as dist
    segs = sd.segments()

    def fn(phi):
        reqs, recv = [], []
        for q, lo, hi in segs:
            out = torch.from_numpy(phi[lo:hi].copy())
            into = torch.empty(hi - lo, dtype=torch.float64)
            reqs.append(dist.isend(out, q))
            reqs.append(dist.irecv(into, q))
            recv.append((lo, hi, into))
        for r in reqs:
            r.wait()
        for lo, hi, into in recv:
            phi[lo:hi] = into.numpy()
    return fn


def glosum():
    import torch
    import torch.distributed as dist

    def fn(v):
        t = torch.tensor([v], dtype=torch.float64)
        dist.all_reduce(t)
        return float(t.item())
    return fn


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _entry(rank, world, port, q, fn, args):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, fn(rank, world, *args)))
    except Exception as e:  # reported to the parent, which fails the test
        import traceback
        q.put((rank, RuntimeError(f"rank {rank}: {e}\n{traceback.format_exc()}")))
    finally:
        dist.destroy_process_group()


def run_ranks(fn, world, *args, timeout=600):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_entry, args=(r, world, port, q, fn, args)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=timeout) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    for r in range(world):
        if isinstance(got[r], Exception):
            raise got[r]
    for p in procs:
        assert p.exitcode == 0
    return [got[r] for r in range(world)]
