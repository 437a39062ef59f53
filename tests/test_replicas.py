"""The replica (multi-GPU) host logic with world_size 2 gloo ranks on CPU: each
rank takes its share of random vectors, computes their moments (with the oracle
standing in for the GPU), and one all-reduce gives the same averaged moments,
and the same DOS, as a single process."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_path):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from minijclsquant_gb300 import lattice, replicas
    from minijclsquant_gb300.observables import random_vector_generator
    from minijclsquant_gb300.modifiers import modifier_bounds
    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        H = lattice.honeycomb(6, 5, t=-2.7, W=0.6, seed=2)
        d = modifier_bounds(H)
        R_total, M = 5, 40
        local = np.zeros(M, dtype=np.complex128)
        for seed in replicas.vector_seeds(R_total, rank, world):
            local += oracle.rec_A_tab(M, d, H.indices, H.len_row, random_vector_generator(H.shape[0], seed), threads=1)
        mu = replicas.mean_moments(local, R_total)
        t = replicas.max_over_ranks(0.1 * (rank + 1))
        if rank == 0:
            np.save(out_path, np.concatenate([mu, [t]]))
    finally:
        dist.destroy_process_group()


def test_replicas_two_gloo_ranks_match_single_process(tmp_path):
    from minijclsquant_gb300 import lattice, replicas
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator
    from oracle import oracle

    out = str(tmp_path / "mu.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    mu, t = got[:-1], got[-1].real
    H = lattice.honeycomb(6, 5, t=-2.7, W=0.6, seed=2)
    d = modifier_bounds(H)
    ref = np.mean([oracle.rec_A_tab(40, d, H.indices, H.len_row, random_vector_generator(H.shape[0], 1000 + i),
                                    threads=1) for i in range(5)], axis=0)
    assert np.allclose(mu, ref, rtol=1e-13, atol=1e-12)
    assert t == pytest.approx(0.2)


def test_split_range_covers_units_once():
    from minijclsquant_gb300 import replicas

    for n in (0, 1, 7, 256):
        for w in (1, 2, 3, 8):
            parts = [replicas.split_range(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))
            assert max(b - a for a, b in parts) - min(b - a for a, b in parts) <= 1
