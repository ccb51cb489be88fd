"""Photon-range sharding across ranks (world size 2, gloo, CPU).

Each rank propagates a contiguous photon range of every source (the same split
bench.py uses for N GPUs); gathering the hit tables over the process group must
give exactly the single-process run, because photon i always draws the same
Philox stream.  The CPU oracle stands in for the device on this host."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard(sources, rank, world, pp, scaling):
    import copy
    out = []
    for s in sources:
        n = pp.source_photons(s.photons, scaling)
        lo, hi = n * rank // world, n * (rank + 1) // world
        c = copy.copy(s)
        c.photons = hi - lo
        c.first_photon = lo
        out.append(c)
    return out


def _setup(pp):
    """Two sources near one module: an isotropic point and a cascade."""
    s = pp.workloads.c0_setup(120_000)
    s.sources.append(pp.ExtendedCherenkovEmitter(
        [0.0, 0.0, 4.0], [0.0, 0.6, 0.8], 0.0, 80_000,
        pp.LongitudinalParameterisation(2.0, 0.63, 0.36)))
    return s


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pp = entry.load()
    orc = entry.load_oracle()
    setup = _setup(pp)
    setup.sources = _shard(setup.sources, rank, world, pp, setup.photon_scaling)
    hits, sim, steps = orc.Run.from_setup(setup).propagate_all(nthreads=2)
    keys = np.stack([hits["source_index"], hits["photon_index"]], 1).astype(np.int64)
    gathered = [None] * world
    dist.all_gather_object(gathered, (keys, hits["position"], int(sim)))
    if rank == 0:
        q.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_union_equals_single_run(orc, pp):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    keys = np.concatenate([g[0] for g in gathered])
    pos = np.concatenate([g[1] for g in gathered])
    sim = sum(g[2] for g in gathered)

    full = _setup(pp)
    ref, ref_sim, _ = orc.Run.from_setup(full).propagate_all(nthreads=2)
    assert sim == ref_sim
    rkeys = np.stack([ref["source_index"], ref["photon_index"]], 1).astype(np.int64)
    assert len(ref) > 0
    o1 = np.lexsort((keys[:, 1], keys[:, 0]))
    o2 = np.lexsort((rkeys[:, 1], rkeys[:, 0]))
    np.testing.assert_array_equal(keys[o1], rkeys[o2])
    np.testing.assert_array_equal(pos[o1], ref["position"][o2])
