"""World-size-2 host logic of the replica path, on CPU with the gloo backend.

Each rank takes its n^3-balanced shard of one mixed-size batch, "solves" it
(the oracle's FP64 restatement stands in for the GPU replica here: no GPU is
needed and the oracle is only the checker), gathers the per-matrix scalars and
the max-over-ranks step time.  Rank 0 then checks that the gathered results
equal a one-process pass over the whole batch, that the shards partition it,
and that the bench's whole-job throughput uses the slowest rank.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "skewlinearalgebra.jl_gb300"))

from skewgpu import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sizes():
    rng = np.random.default_rng(42)
    return [int(x) for x in rng.integers(1, 97, 40)] + [128, 2, 3]


def _mat(n, k):
    rng = np.random.default_rng(1000 + k)
    B = rng.standard_normal((n, n)) / np.sqrt(n)
    return (B - B.T) / 2


def _worker(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "skewlinearalgebra.jl_gb300"))
    from oracle import oracle as O
    from skewgpu import replicas as R

    w, r, _, dist = R.init_from_env("gloo")
    assert (w, r) == (world, rank)
    sizes = _sizes()
    idx = R.shard_indices(sizes, w, r)
    lp = np.empty(len(idx))
    sg = np.empty(len(idx))
    for j, b in enumerate(idx):
        lp[j], sg[j] = O.logabspfaffian(_mat(sizes[b], int(b)))
    all_lp = R.gather_scalars(idx, lp, len(sizes), dist)
    all_sg = R.gather_scalars(idx, sg, len(sizes), dist)
    all_owner = R.gather_scalars(idx, np.full(len(idx), float(r)), len(sizes), dist)
    t = R.max_over_ranks(0.5 + r, dist)
    np.savez(os.path.join(outdir, f"rank{r}.npz"), idx=idx, lp=all_lp, sg=all_sg, owner=all_owner, t=t)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_gloo_shards_and_gathers(tmp_path, oracle):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    sizes = _sizes()
    # shards partition the batch
    allidx = np.concatenate([r["idx"] for r in res])
    assert sorted(allidx.tolist()) == list(range(len(sizes)))
    # every rank holds the same gathered arrays, equal to a one-process pass
    ref = [oracle.logabspfaffian(_mat(n, k)) for k, n in enumerate(sizes)]
    for r in res:
        np.testing.assert_array_equal(r["lp"], np.array([x[0] for x in ref]))
        np.testing.assert_array_equal(r["sg"], np.array([x[1] for x in ref]))
        np.testing.assert_array_equal(r["owner"], res[0]["owner"])
        assert float(r["t"]) == 1.5  # max over ranks of 0.5 + rank


def test_shard_balance_and_determinism():
    sizes = np.random.default_rng(3).integers(8, 257, 4096)
    for world in (1, 2, 3, 8):
        shards = [replicas.shard_indices(sizes, world, r) for r in range(world)]
        assert sorted(np.concatenate(shards).tolist()) == list(range(len(sizes)))
        load = np.array([replicas.matrix_cost(sizes[s]).sum() for s in shards])
        # LPT bound: no shard exceeds the mean by more than the largest single matrix
        assert load.max() - load.mean() <= replicas.matrix_cost([sizes.max()])[0]
        again = [replicas.shard_indices(sizes, world, r) for r in range(world)]
        assert all((a == b).all() for a, b in zip(shards, again))
    with pytest.raises(ValueError):
        replicas.shard_indices(sizes, 2, 2)


def test_single_process_helpers():
    idx = np.array([2, 0])
    out = replicas.gather_scalars(idx, np.array([5.0, 7.0]), 3)
    assert out[0] == 7.0 and out[2] == 5.0 and np.isnan(out[1])
    assert replicas.max_over_ranks(3.25) == 3.25
    assert replicas.weak_scaling_throughput(4096, 4, 10, 2.0) == 4 * 4096 * 10 / 2.0
    with pytest.raises(ValueError):
        replicas.weak_scaling_throughput(1, 1, 1, 0.0)
