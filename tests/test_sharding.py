"""Orientation sharding and the reduction of per-rank search maps.

The reduction restates ``aggregate_distributed_results``
(backend/process_results.py:7-64); the multi-rank path runs as two ``gloo``
ranks on the CPU, each folding its orientation shard of a golden search into
its own maps with the oracle, then ``gather_search_maps`` to rank 0.  The
reduced maps must equal one oracle run over all orientations.
"""

import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from leopard_em_gb300 import sharding
from oracle import ref_match_template as orc

GOLD_PATH = os.path.join(os.path.dirname(__file__), "golden", "match_small.npz")


def _inputs(case):
    gold = np.load(GOLD_PATH)
    keys = ["image_dft", "template_dft", "ctf_filters", "whitening_filter_template",
            "defocus_values", "pixel_values", "euler_angles"]
    return {k: torch.from_numpy(gold[f"{case}/in/{k}"]) for k in keys}


def _oracle_maps(inp, begin, end, batch):
    """The oracle's search loop (core_match_template.py:492-550) over the
    global orientation range [begin, end) of the full set."""
    euler = inp["euler_angles"]
    n_o, n_df, n_cs = euler.shape[0], inp["defocus_values"].shape[0], inp["pixel_values"].shape[0]
    H, W = inp["image_dft"].shape[0], 2 * (inp["image_dft"].shape[1] - 1)
    pf = inp["ctf_filters"] * inp["whitening_filter_template"][None, None]
    incr = torch.tensor([df * n_o + cs * n_df * n_o for cs in range(n_cs) for df in range(n_df)])
    mip = torch.full((H, W), -float("inf"))
    best = torch.full((H, W), -1, dtype=torch.int64)
    s1 = torch.zeros((H, W), dtype=torch.float64)
    s2 = torch.zeros((H, W), dtype=torch.float64)
    for i in range(begin, end, batch):
        j = min(end, i + batch)
        rot = orc.euler_to_rotmat_zyz(euler[i:j])
        bsi = (torch.arange(i, j) + incr[:, None]).flatten()
        cc = orc.cross_correlate_batched_cpu(inp["image_dft"], inp["template_dft"], rot, pf)
        orc.iteration_statistics_update(cc, bsi, mip, best, s1, s2, H, W)
    return {"mip": mip, "best_global_index": best, "correlation_sum": s1, "correlation_squared_sum": s2}


def test_orientation_shards_cover_range_in_whole_batches():
    for n, world, b in [(0, 2, 4), (7, 1, 3), (100, 3, 8), (1_580_000, 8, 8), (5, 8, 2)]:
        shards = sharding.orientation_shards(n, world, b)
        assert len(shards) == world
        assert shards[0][0] == 0 and shards[-1][1] == n
        for (a0, a1), (b0, _) in zip(shards, shards[1:]):
            assert a1 == b0 and a0 <= a1
        for a0, a1 in shards[:-1]:
            assert a0 % b == 0 and (a1 % b == 0 or a1 == n)
        sizes = [a1 - a0 for a0, a1 in shards]
        assert max(sizes) - min(sizes) <= b
    with pytest.raises(ValueError):
        sharding.orientation_shards(10, 0)


def test_reduce_matches_first_occurrence_argmax():
    g = torch.Generator().manual_seed(3)
    shards = []
    for r in range(4):
        m = torch.randint(0, 5, (16, 24), generator=g).float()  # many exact ties
        shards.append({
            "mip": m,
            "best_global_index": torch.full((16, 24), 100 * r + 1, dtype=torch.int32),
            "correlation_sum": torch.rand(16, 24, generator=g, dtype=torch.float64),
            "correlation_squared_sum": torch.rand(16, 24, generator=g, dtype=torch.float64),
        })
    out = sharding.reduce_search_maps(shards)
    mips = np.stack([s["mip"].numpy() for s in shards])
    arg = mips.argmax(axis=0)  # numpy: first occurrence, as process_results.py:40-42
    idx = np.stack([s["best_global_index"].numpy() for s in shards])
    np.testing.assert_array_equal(out["mip"].numpy(), mips.max(axis=0))
    np.testing.assert_array_equal(out["best_global_index"].numpy(), np.take_along_axis(idx, arg[None], 0)[0])
    np.testing.assert_allclose(out["correlation_sum"].numpy(),
                               np.stack([s["correlation_sum"].numpy() for s in shards]).sum(0), rtol=1e-15)
    np.testing.assert_allclose(out["correlation_squared_sum"].numpy(),
                               np.stack([s["correlation_squared_sum"].numpy() for s in shards]).sum(0), rtol=1e-15)
    assert out["best_global_index"].dtype == torch.int32


def test_reduce_rejects_bad_input():
    with pytest.raises(ValueError):
        sharding.reduce_search_maps([])
    with pytest.raises(ValueError):
        sharding.reduce_search_maps([{"mip": torch.zeros(2, 2)}])


def test_sharded_oracle_equals_single_run_in_process():
    inp = _inputs("b")
    n = inp["euler_angles"].shape[0]
    full = _oracle_maps(inp, 0, n, 3)
    parts = [_oracle_maps(inp, a, b, 3) for a, b in sharding.orientation_shards(n, 2, 3)]
    red = sharding.reduce_search_maps(parts)
    torch.testing.assert_close(red["mip"], full["mip"], rtol=0, atol=0)
    assert (red["best_global_index"] == full["best_global_index"]).all()
    torch.testing.assert_close(red["correlation_sum"], full["correlation_sum"], rtol=1e-12, atol=1e-12)
    torch.testing.assert_close(red["correlation_squared_sum"], full["correlation_squared_sum"], rtol=1e-12,
                               atol=1e-12)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case, batch, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        inp = _inputs(case)
        n = inp["euler_angles"].shape[0]
        begin, end = sharding.orientation_shards(n, world, batch)[rank]
        maps = _oracle_maps(inp, begin, end, batch)
        red = sharding.gather_search_maps(maps, dst=0)
        if rank == 0:
            torch.save(red, out_path)
        else:
            assert red is None
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case,batch", [("a", 4), ("b", 2)])
def test_gloo_two_ranks_gather_reduce(case, batch):
    inp = _inputs(case)
    n = inp["euler_angles"].shape[0]
    full = _oracle_maps(inp, 0, n, batch)
    with tempfile.TemporaryDirectory() as d:
        out_path = os.path.join(d, "reduced.pt")
        mp.start_processes(_rank_main, args=(2, _free_port(), case, batch, out_path), nprocs=2, join=True,
                           start_method="spawn")
        red = torch.load(out_path)
    torch.testing.assert_close(red["mip"], full["mip"], rtol=0, atol=0)
    assert (red["best_global_index"] == full["best_global_index"]).all()
    torch.testing.assert_close(red["correlation_sum"], full["correlation_sum"], rtol=1e-12, atol=1e-12)
    torch.testing.assert_close(red["correlation_squared_sum"], full["correlation_squared_sum"], rtol=1e-12,
                               atol=1e-12)
