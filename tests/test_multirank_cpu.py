"""The multi-GPU path on CPU: one accumulator per process, merged across ranks with
torch.distributed (gloo, world size 2), against the single-process merge of the same
accumulators (merge_correlations' arithmetic, SampledCorrelations.jl:128-142)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_data(rank):
    rng = np.random.default_rng(100 + rank)
    shape = (6, 2, 2, 3, 3, 2, 10)
    data = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    M = rng.random(shape)
    count = 3 + 2 * rank
    return data, count, M


def _worker(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    import torch.distributed as dist
    import __graft_entry__ as ge
    sg = ge.package()
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    data, count, M = _rank_data(rank)
    mu, n, Mt = sg.correlations.allreduce_correlations(data, count, M)
    np.save(out / f"mu{rank}.npy", mu)
    np.save(out / f"M{rank}.npy", Mt)
    (out / f"n{rank}.txt").write_text(str(n))
    dist.barrier()
    dist.destroy_process_group()


def test_allreduce_merge_matches_single_process(sg, tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), tmp_path), nprocs=world, start_method="spawn")
    datas, counts, Ms = zip(*[_rank_data(r) for r in range(world)])
    d_ref, n_ref, M_ref = sg.correlations.merge_host(datas, counts, Ms)
    for r in range(world):
        assert int((tmp_path / f"n{r}.txt").read_text()) == n_ref
        assert np.allclose(np.load(tmp_path / f"mu{r}.npy"), d_ref, rtol=1e-12, atol=1e-12)
        assert np.allclose(np.load(tmp_path / f"M{r}.npy"), M_ref, rtol=1e-12, atol=1e-12)


def test_merge_host_equals_sequential_running_mean(sg):
    # merging 1 + 2 + 3 sample accumulators equals the mean over all samples
    rng = np.random.default_rng(7)
    samples = rng.standard_normal((6, 4, 5)) + 1j * rng.standard_normal((6, 4, 5))
    groups = [samples[:1], samples[1:3], samples[3:]]
    datas = [g.mean(axis=0) for g in groups]
    Ms = [np.sum(np.abs(g - g.mean(axis=0)) ** 2, axis=0) for g in groups]
    d, n, M = sg.correlations.merge_host(datas, [len(g) for g in groups], Ms)
    assert n == 6
    assert np.allclose(d, samples.mean(axis=0), rtol=1e-13, atol=1e-13)
    assert np.allclose(M, np.sum(np.abs(samples - samples.mean(axis=0)) ** 2, axis=0), rtol=1e-12)
