"""Multi-rank sharding on CPU: two gloo ranks each trace their own primary range with the FP64
oracle (the Philox streams are keyed by the global primary index), sum their histograms with one
all-reduce, and the result equals the unsharded run.  This is the host-side logic of a multi-GPU
job (one rank per GPU, replicas over primary ranges), exercised without a GPU."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, n, out_path):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from pachydermacoustic_universal_gb300 import rooms

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    w = rooms.shoebox_c1()
    per = n // world
    begin = rank * per
    cnt = per if rank < world - 1 else n - begin
    h, st = O.trace(w, rays=cnt, ray_begin=begin, seed=11, threads=2)
    t = torch.from_numpy(np.concatenate([h["energy"].ravel(), h["analysis"].ravel()]))
    seg = torch.tensor([float(st["segments"])], dtype=torch.float64)
    dist.all_reduce(t)
    dist.all_reduce(seg)
    if rank == 0:
        np.save(out_path, np.concatenate([t.numpy(), seg.numpy()]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_unsharded_run(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import oracle as O
    from pachydermacoustic_universal_gb300 import rooms

    n = 40
    out = str(tmp_path / "sum.npy")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, n, out), nprocs=2, join=True)
    got = np.load(out)
    w = rooms.shoebox_c1()
    h, st = O.trace(w, rays=n, ray_begin=0, seed=11, threads=2)
    ref = np.concatenate([h["energy"].ravel(), h["analysis"].ravel()])
    np.testing.assert_allclose(got[:-1], ref, rtol=1e-12, atol=1e-300)
    assert got[-1] == st["segments"]
