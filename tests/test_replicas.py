"""Multi-GPU replica path on the host: two gloo ranks on CPU (no GPU needed).

The bench's N > 1 launch runs one rank per GPU, each with its own seeds and no
collective in the sweep; the whole-job time is the maximum over ranks, and the
only data exchange is the per-bin mean of the observables over walkers
(observables_mod.F90:824-834).  Here each of two gloo ranks runs its own Markov
chain (the CPU oracle stands in for a rank's GPU), forms its scalar bins, and the
ranks merge them with bins.mean_over_ranks; the merged bins must equal the mean of
the same two chains run in one process.
"""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

import oracle
from alf_gb300 import bins, model as mdl, replicas, rng


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [1.0 + rank, 10.0 - rank]  # rank 1 is slower in the first entry
        out[rank] = replicas.max_over_ranks(local)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0] == out[1] == [2.0, 10.0]
    assert replicas.whole_job_rate(world, 3, 5, 2.0) == 15.0


def test_replica_seeds_are_distinct():
    seeds = {replicas.replica_seed(7, r, c) for r in range(8) for c in range(128)}
    assert len(seeds) == 8 * 128
    # the base seed is part of the packing: neighbouring runs share no chain seed
    a = {replicas.replica_seed(b, r, c) for b in (1, 1001) for r in range(2) for c in range(1001)}
    assert len(a) == 2 * 2 * 1001
    assert replicas.replica_seed(1, 1, 0) != replicas.replica_seed(1001, 0, 0)
    assert replicas.replica_seed(1, 1, 0) != replicas.replica_seed(1, 0, 1000)


_RING = dict(lattice="n_leg_ladder", L1=4, L2=1, U=4.0, beta=2.0, dtau=0.1, nwrap=10)
_BINS, _SWEEPS = 3, 5


def _chain_bins(seed: int):
    """Scalar bins of one oracle chain on the 4-site ring, seeded from `seed`."""
    m = mdl.hubbard(_RING["lattice"], _RING["L1"], _RING["L2"], U=_RING["U"], beta=_RING["beta"],
                    dtau=_RING["dtau"], nwrap=_RING["nwrap"])
    o = oracle.Oracle(m)
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    H = mdl.hopping_matrix(_RING["lattice"], _RING["L1"], _RING["L2"]).real
    o.set_scalar_obs(np.stack([H, H]), np.full(m.ndim, _RING["U"]))
    out, sweep = [], 0
    for _ in range(_BINS):
        for _ in range(_SWEEPS):
            o.sweep(rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, sweep))
            sweep += 1
        out.append(bins.walker_mean([bins.bin_from_sums(o.scalar_obs(reset=True))]))
    return out


def _chain_rank(rank, world, port, base, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        own = _chain_bins(replicas.replica_seed(base, rank, 0))
        merged = [bins.mean_over_ranks(ov, sg) for ov, sg in own]
        out[rank] = ([(list(ov), sg) for ov, sg in own], [(list(ov), sg) for ov, sg in merged])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_run_their_own_chains_and_merge_the_bins():
    base, world = 11, 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_chain_rank, args=(world, _free_port(), base, out), nprocs=world, join=True)
    own = [out[r][0] for r in range(world)]
    # the ranks ran different chains (their own seeds) ...
    assert any(not np.allclose(own[0][b][0], own[1][b][0]) for b in range(_BINS))
    # ... each rank's chain is the chain a single process gets from that rank's seed ...
    for r in range(world):
        ref = _chain_bins(replicas.replica_seed(base, r, 0))
        for b in range(_BINS):
            np.testing.assert_allclose(own[r][b][0], ref[b][0], rtol=0, atol=1e-13)
            assert abs(own[r][b][1] - ref[b][1]) < 1e-13
    # ... and every rank holds the walker mean of both ranks' bins
    for b in range(_BINS):
        want = np.mean([np.asarray(own[r][b][0]) for r in range(world)], axis=0)
        want_s = np.mean([own[r][b][1] for r in range(world)])
        for r in range(world):
            ov, sg = out[r][1][b]
            np.testing.assert_allclose(ov, want, rtol=0, atol=1e-13)
            assert abs(sg - want_s) < 1e-13
