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


def _subgroup_rank_main(rank, world, port, case, batch, out_path):
    """Ranks 1 and 2 of a world of 3 form a subgroup and gather to its rank 0
    (global rank 1); global rank 0 takes no part."""
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        group = dist.new_group([1, 2])
        if rank in (1, 2):
            inp = _inputs(case)
            n = inp["euler_angles"].shape[0]
            g = dist.get_rank(group)
            begin, end = sharding.orientation_shards(n, 2, batch)[g]
            maps = _oracle_maps(inp, begin, end, batch)
            red = sharding.gather_search_maps(maps, dst=0, group=group)
            if g == 0:
                assert rank == 1
                torch.save(red, out_path)
            else:
                assert red is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_gloo_subgroup_gather_uses_group_rank():
    """``dst`` is a rank within the group: with the group {1, 2} the maps are
    reduced on global rank 1, and equal one search over all orientations."""
    case, batch = "a", 4
    inp = _inputs(case)
    n = inp["euler_angles"].shape[0]
    full = _oracle_maps(inp, 0, n, batch)
    with tempfile.TemporaryDirectory() as d:
        out_path = os.path.join(d, "reduced.pt")
        mp.start_processes(_subgroup_rank_main, args=(3, _free_port(), case, batch, out_path), nprocs=3,
                           join=True, start_method="spawn")
        red = torch.load(out_path)
    torch.testing.assert_close(red["mip"], full["mip"], rtol=0, atol=0)
    assert (red["best_global_index"] == full["best_global_index"]).all()
    torch.testing.assert_close(red["correlation_sum"], full["correlation_sum"], rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_device_shards_reduce_to_the_full_search():
    """Two orientation shards searched on the device, reduced in rank order and
    finalised, equal one search over all orientations."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend import MatchTemplateSearch

    cfg = sy.MatchConfig(image_shape=(256, 256), template_size=32, n_blobs=60, blob_radius=11.0, n_particles=2,
                         snr=0.5, seed=8, defocus_offsets=(-200.0, 0.0, 200.0))
    eul = sy.uniform_euler_grid(30.0, 30.0)[:23]
    kw = sy.make_match_workload(cfg, euler_angles=eul).kwargs
    dev = torch.device("cuda:0")
    full = MatchTemplateSearch(**kw, device=dev, orientation_batch_size=4)
    full.run()
    ref = full.result(to_cpu=True)
    shards = []
    for a, b in sharding.orientation_shards(23, 2, 4):
        s = MatchTemplateSearch(**kw, device=dev, orientation_batch_size=4)
        s.run(a, b)
        shards.append({k: v.clone() for k, v in s.maps().items()})
    red = sharding.reduce_search_maps(shards)
    host = MatchTemplateSearch(**kw, device=dev, orientation_batch_size=4)
    host.load_maps(red)
    host.orientations_done = 23
    got = host.result(to_cpu=True)
    assert torch.equal(got["mip"], ref["mip"])
    for k in ("best_phi", "best_theta", "best_psi", "best_defocus"):
        assert torch.equal(got[k], ref[k]), k
    torch.testing.assert_close(got["scaled_mip"], ref["scaled_mip"], rtol=1e-5, atol=1e-5)
