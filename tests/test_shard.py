"""Formula sharding over two ranks (gloo on CPU, emulation build): every formula is
taken by exactly one rank, shares balance, and the gathered results equal one
batched round over the whole batch."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from parafrost_gb300 import cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.shard import run_sharded, shard_formulas


def forms():
    return [cnfgen.aig_unrolled(num_gates=50 + 13 * i, steps=2 + i % 3, seed=70 + i) for i in range(9)] + \
           [cnfgen.random_ksat(num_vars=150, num_clauses=600, k=3, seed=80 + i) for i in range(5)]


def test_shard_partition():
    f = forms()
    for world in (1, 2, 3):
        shares = shard_formulas(f, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(f)))
        assert all(s == sorted(s) for s in shares)
    loads = [sum(f[i][2].size for i in s) for s in shard_formulas(f, 2)]
    assert max(loads) < 1.5 * min(loads)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, lib, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = run_sharded(forms(), Options(all=1), rank, world, library=lib)
        if rank == 0:
            q.put([rd.canonical_result(st, r if st == 0 else None) for st, _, r in res])
    finally:
        dist.destroy_process_group()


def test_shard_two_ranks_gloo(built):
    lib = built["emu"]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, lib, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    whole = run_sharded(forms(), Options(all=1), 0, 1, library=lib)
    assert got == [rd.canonical_result(st, r if st == 0 else None) for st, _, r in whole]
