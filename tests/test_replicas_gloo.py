"""Multi-process replica path of bench.py on CPU (gloo, world size 2): per-rank seeds, max-over-ranks
timing and whole-job throughput.  Each rank renders a tiny frame with the CPU oracle (a stand-in for
its GPU; the replica logic is what is under test)."""
import os
import socket
import time

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from lambda_gb300 import configs
    from oracle.oracle import Oracle
    sb, cam, opts = configs.cornell(8, 8, 2)
    opts.seed = bench.replica_seed(rank)
    t0 = time.perf_counter()
    film = Oracle(sb).render(cam, opts, threads=1)
    ms = (time.perf_counter() - t0) * 1e3 + 10.0 * rank      # ranks finish at different times
    (ms_max,) = bench.max_over_ranks([ms], dist, "cpu")
    np.save(os.path.join(out_dir, "film%d.npy" % rank), film)
    np.save(os.path.join(out_dir, "ms%d.npy" % rank), np.array([ms, ms_max]))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_two_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    from oracle import oracle
    oracle.build()
    world, port = 2, _free_port()
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    f0, f1 = np.load(tmp_path / "film0.npy"), np.load(tmp_path / "film1.npy")
    m0, m1 = np.load(tmp_path / "ms0.npy"), np.load(tmp_path / "ms1.npy")
    # every rank did the full per-rank work (weak scaling) with its own random numbers
    assert np.all(f0[..., 3] == 2) and np.all(f1[..., 3] == 2)
    assert not np.array_equal(f0[..., :3], f1[..., :3])
    # both ranks agree on the slowest rank's time
    assert m0[1] == m1[1] == max(m0[0], m1[0])
    import bench
    v = bench.job_throughput(8 * 8 * 2, 1, world, m0[1])
    assert abs(v - world * 128 / (m0[1] / 1e3) / 1e6) < 1e-9
