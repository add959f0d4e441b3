"""Instance sharding (``pyqed_gb300.shard``): the partition, the gather order
and a two-rank ``gloo`` run on the CPU whose gathered result is bitwise the
single-rank one.  The per-rank engine inside the two-rank test is the oracle
(test infrastructure), standing in for one GPU per rank."""
import os
import socket
import tempfile

import numpy as np
import pytest

from oracle import lindblad_oracle as O
from pyqed_gb300 import shard as S
from pyqed_gb300 import workloads as W


def test_partition_covers_every_instance_once_and_balances_n3():
    dims = W.exciton_dims()  # the exciton batch: N = n + 1, n ~ U{8..64}
    cost = S.instance_cost(dims)
    for world in (1, 2, 3, 4, 8):
        parts = S.partition(dims, world)
        allidx = np.concatenate(parts)
        assert np.array_equal(np.sort(allidx), np.arange(dims.size))
        assert all(np.all(np.diff(p) > 0) for p in parts)  # each rank keeps batch order
        loads = np.array([cost[p].sum() for p in parts])
        # greedy LPT: no two ranks differ by more than one instance's cost
        assert loads.max() - loads.min() <= cost.max()
        assert loads.max() / loads.mean() < 1.001


def test_partition_is_deterministic_and_rank_selection():
    dims = np.array([9, 65, 33, 17, 65, 40, 12, 64])
    a = S.partition(dims, 3)
    assert all(np.array_equal(x, y) for x, y in zip(a, S.partition(dims, 3)))
    for r in range(3):
        assert np.array_equal(S.shard_indices(dims, r, 3), a[r])
    with pytest.raises(ValueError):
        S.shard_indices(dims, 3, 3)
    # more ranks than instances: the extra ranks get nothing
    p = S.partition(dims[:2], 4)
    assert sorted(len(x) for x in p) == [0, 0, 1, 1]


def test_gather_restores_batch_order_and_checks_coverage():
    parts = [(np.array([0, 3]), ["a", "d"]), (np.array([1, 2]), ["b", "c"])]
    assert S.gather(parts, 4) == ["a", "b", "c", "d"]
    with pytest.raises(ValueError):
        S.gather(parts[:1], 4)
    with pytest.raises(ValueError):
        S.gather(parts + [(np.array([2]), ["x"])], 4)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case():
    return W.exciton_batch(indices=[0, 1, 2, 3, 4, 5, 6, 313, 100, 200], nt=12)


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        ex = _case()
        dims = [h.shape[0] for h in ex["H"]]
        idx = S.shard_indices(dims, rank, world)
        local = [O.propagate_diag_correlation(ex["H"][b], ex["mu"][b], ex["rho_g"][b], ex["c_diag"][b],
                                              ex["dt"], ex["nt"]) for b in idx]
        full = S.gather_to_rank0(idx, local, len(dims))
        if rank == 0:
            np.save(out_path, np.stack(full))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_gather_is_bitwise_single_rank():
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "gathered.npy")
        mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True,
                           start_method="spawn")
        got = np.load(out)
    ex = _case()
    ref = np.stack([O.propagate_diag_correlation(ex["H"][b], ex["mu"][b], ex["rho_g"][b], ex["c_diag"][b],
                                                 ex["dt"], ex["nt"]) for b in range(len(ex["H"]))])
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


def test_batch_api_shard_argument_selects_the_rank_share():
    # the batched API's shard= path up to the engine call (no GPU): the
    # selection helper returns this rank's instances in batch order
    from pyqed_gb300.batch import _select
    ex = _case()
    dims = [h.shape[0] for h in ex["H"]]
    cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
    seen = []
    for r in range(3):
        idx, H, c, r0, e, d_ops, drv = _select((r, 3), ex["H"], cops, ex["rho_g"], None, None, None)
        assert np.array_equal(idx, S.shard_indices(dims, r, 3))
        assert all(H[k] is ex["H"][b] for k, b in enumerate(idx))
        assert e is None and d_ops is None and drv is None
        seen.extend(idx.tolist())
    assert sorted(seen) == list(range(len(dims)))
