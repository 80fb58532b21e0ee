"""Replica sharding and the exact tally reduction on world_size-2 gloo ranks
(CPU).  Each rank walks its photon-id share with the CPU oracle standing in
for its GPU; the reduced tally must equal one walk of the whole range."""
import os
import socket

import numpy as np
import pytest


def test_shard_covers_range_without_overlap():
    from tiny_mc_gb300.replicas import shard
    for n, world in [(10, 3), (7, 8), (1 << 20, 4), (0, 2)]:
        got = [shard(n, world, r, base=100) for r in range(world)]
        at = 100
        for start, count in got:
            assert start == at
            at += count
        assert at == 100 + n


def test_add128_carries():
    from tiny_mc_gb300 import TALLY_DTYPE
    from tiny_mc_gb300.replicas import add128
    a = np.zeros(2, TALLY_DTYPE)
    b = np.zeros(2, TALLY_DTYPE)
    a["w_lo"] = [2 ** 64 - 1, 5]
    b["w_lo"] = [2, 7]
    a["w2_hi"] = [3, 0]
    b["w2_lo"] = [2 ** 63, 2 ** 63]
    a["w2_lo"] = [2 ** 63, 0]
    c = add128(a, b)
    assert list(c["w_lo"]) == [1, 12] and list(c["w_hi"]) == [1, 0]
    assert list(c["w2_lo"]) == [0, 2 ** 63] and list(c["w2_hi"]) == [4, 0]


def _rank(rank, world, port, n, out_dir):
    import torch.distributed as dist

    from oracle import oracle
    from tiny_mc_gb300 import TALLY_DTYPE
    from tiny_mc_gb300.replicas import reduce_tallies, shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    base, count = shard(n, world, rank, base=12345)
    t, _, _ = oracle.walk_fx(oracle.cfg("params_h", seed=3), count, id_base=base, nthreads=2)
    local = t.reshape(-1).view(TALLY_DTYPE).copy()
    total = reduce_tallies(local)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), total)
    dist.destroy_process_group()


def test_gloo_two_ranks_match_single_walk(tmp_path, oracle_mod):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    n = 6000
    mp.start_processes(_rank, args=(2, port, n, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    ref, _, _ = oracle_mod.walk_fx(oracle_mod.cfg("params_h", seed=3), n, id_base=12345)
    for r in range(2):
        got = np.load(tmp_path / f"rank{r}.npy")
        got = np.stack([got["w_lo"], got["w_hi"], got["w2_lo"], got["w2_hi"]], axis=1)
        assert np.array_equal(got, ref)
