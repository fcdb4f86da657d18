"""Replica parallelism (xitils_gb300.replicas) on CPU ranks: two gloo processes
render disjoint sample ranges of the same film and add their films; the sum
equals one process rendering every sample (FP32 sums in another order), and the
job's time is the slower rank's. The renders here are the CPU oracle's, standing
in for each rank's GPU (the exchange is host-side either way)."""
import os
import socket
import tempfile

import numpy as np
import pytest

from xitils_gb300 import replicas


def test_sample_ranges_partition_the_samples():
    for spp in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            ranges = [replicas.sample_range(r, world, spp, first=5) for r in range(world)]
            assert sum(c for _, c in ranges) == spp
            assert ranges[0][0] == 5
            for (b0, c0), (b1, _) in zip(ranges, ranges[1:]):
                assert b0 + c0 == b1
            assert max(c for _, c in ranges) - min(c for _, c in ranges) <= 1
    with pytest.raises(ValueError):
        replicas.sample_range(2, 2, 4)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from oracle.bindings import load_scene
    from xitils_gb300 import scenes
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        desc = scenes.cornell(32, 24, 6)
        chk = load_scene(desc, "port")
        film = replicas.render_replica(lambda b, c: chk.render_pcg(desc, spp_begin=b, spp_count=c, nthreads=1),
                                       rank, world, desc.spp)
        slowest = replicas.max_over_ranks(1.0 + rank)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), film=film, slowest=slowest)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_single_render():
    import torch.multiprocessing as mp

    from oracle.bindings import load_scene
    from xitils_gb300 import scenes
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(2, _free_port(), d), nprocs=2, join=True, start_method="spawn")
        r0, r1 = np.load(os.path.join(d, "rank0.npz")), np.load(os.path.join(d, "rank1.npz"))
    desc = scenes.cornell(32, 24, 6)
    full = load_scene(desc, "port").render_pcg(desc)
    np.testing.assert_array_equal(r0["film"], r1["film"])  # every rank receives the sum
    np.testing.assert_allclose(r0["film"], full, rtol=1e-5, atol=1e-5)
    assert float(r0["slowest"]) == 2.0 and float(r1["slowest"]) == 2.0
