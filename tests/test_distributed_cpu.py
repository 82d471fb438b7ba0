"""CPU, two gloo ranks: the row-sharded SpMM path (each rank owns a
contiguous, nnz-balanced range of whole block rows, B is replicated, no data
exchange) reassembles the full product, and the max-over-ranks timing
reduction the benchmark uses gives the slowest rank. GPU kernels are not
involved; each rank checks its shard with the oracle."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "sptc-smat_gb300"))
    sys.path.insert(0, os.path.join(root, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as O
    import smat
    from smat import generators as G
    A = G.rmat(10, 8000, seed=11)
    B = np.random.default_rng(1).standard_normal((A.cols, 8))
    r0, r1 = smat.partition_rows(A, world)[rank]
    S = smat.row_slice(A, r0, r1)
    Cs = O.spmm_f64(S.row_ptr, S.col_idx, S.values.astype(np.float64), B)
    parts = [None] * world
    dist.all_gather_object(parts, (r0, r1, Cs))
    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        full = O.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), B)
        got = np.zeros_like(full)
        for a, b, c in parts:
            got[a:b] = c
        np.save(os.path.join(out_dir, "ok.npy"), np.array([np.array_equal(got, full), float(t[0])]))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_rows_reassemble_full_product(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    ok, tmax = np.load(tmp_path / "ok.npy")
    assert ok == 1.0
    assert tmax == float(world)
