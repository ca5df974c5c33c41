"""Host-side parts of the batched form (no GPU): grid selection through the C
ABI, the autotuner's cache and the batched workload's configuration."""

import json

import pytest

from leopard_em_gb300 import autotune
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300._native import lib
from leopard_em_gb300.backend.core_match_template import padded_grid


@pytest.mark.parametrize(
    "n,axis,want",
    [
        (4096, 0, 4096), (4092, 1, 4096), (3838, 0, 3840), (3710, 1, 3840), (2880, 1, 2880), (2880, 0, 2880),
        (3072, 0, 3072), (5760, 0, 5760), (5760, 1, 5760), (4097, 0, 5760), (250, 0, 256), (270, 1, 288),
        (130, 1, 256), (47, 0, 48), (1, 0, 48),
    ],
)
def test_fft_grid_lengths(n, axis, want):
    assert lib().lgb_match_fft_size(n, axis) == want


def test_fft_grid_rejects_bad_queries():
    assert lib().lgb_match_fft_size(0, 0) == 0
    assert lib().lgb_match_fft_size(100, 2) == 0
    assert lib().lgb_match_fft_size(6000, 0) == 0  # beyond the largest compiled length


def test_every_batched_micrograph_has_a_grid():
    for cfg in sy.batched_micrograph_configs(12):
        H, W = cfg.image_shape
        Hp, Wp = padded_grid(H, W)
        assert H <= Hp <= H + 64 and W <= Wp <= W + 256
        assert 50 <= cfg.n_particles <= 300 and 0.05 <= cfg.snr <= 0.2
    with pytest.raises(ValueError):
        padded_grid(7000, 100)


def test_tuning_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv(autotune.CACHE_ENV, str(path))
    assert autotune.cache_path() == str(path)
    assert autotune._load_cache(str(path)) == {}
    autotune._store_cache(str(path), "k1", {"orientation_batch": 8, "col_waves": 4, "graph_batches": 16,
                                            "ms_per_orientation": 1.5})
    autotune._store_cache(str(path), "k2", {"orientation_batch": 4, "col_waves": 2, "graph_batches": 32,
                                            "ms_per_orientation": 0.5})
    data = json.loads(path.read_text())
    assert set(data) == {"k1", "k2"}
    assert autotune.SearchTuning(**data["k1"]).orientation_batch == 8
    path.write_text("not json")
    assert autotune._load_cache(str(path)) == {}


def test_graph_batches_heuristic():
    assert autotune.SearchTuning.graph_batches_for(8) == 16
    assert autotune.SearchTuning.graph_batches_for(200) == 1
