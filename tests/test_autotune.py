"""Tile-plan tuning: candidates, block planning and the JSON cache (CPU)."""
import json

import numpy as np
import pytest

from ustb_gb300 import autotune, fast
from ustb_gb300.uff import LinearScan, LinearScan3D


def test_plan_tiles_with_a_given_block_covers_every_pixel_once():
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 40), np.linspace(10e-3, 20e-3, 100))
    tiles = fast.plan_tiles(scan, 20e6, 1540.0, block=(64, 8, 1))
    got = np.sort(tiles[tiles >= 0])
    assert np.array_equal(got, np.arange(scan.N_pixels))
    # blocks are at most 64 deep and 8 wide: every tile's pixels span <= 64 z rows
    for row in tiles:
        p = row[row >= 0]
        iz, ix = p % 100, p // 100
        assert iz.max() - iz.min() < 64 and ix.max() - ix.min() < 8


def test_plan_tiles_rejects_oversized_blocks():
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 40), np.linspace(10e-3, 20e-3, 100))
    with pytest.raises(ValueError):
        fast.plan_tiles(scan, 20e6, 1540.0, block=(32, 32, 1))


def test_candidates_2d_and_3d():
    s2 = LinearScan(np.linspace(-1e-2, 1e-2, 256), np.linspace(5e-3, 5e-2, 512))
    c2 = autotune.candidates(s2)
    assert c2[0].block is None and {c.order for c in c2} == {"cost", "scan"}
    assert all(np.prod(c.block) == fast.TILE for c in c2 if c.block is not None)
    s3 = LinearScan3D(np.linspace(-1e-2, 1e-2, 64), np.linspace(5e-3, 4e-2, 128), np.linspace(-1e-2, 1e-2, 64))
    c3 = autotune.candidates(s3)
    assert any(c.block is not None and c.block[2] > 1 for c in c3)


def test_cache_roundtrip_skips_the_search(tmp_path, monkeypatch):
    monkeypatch.setenv("USTB_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    autotune._store("k", autotune.Choice((16, 32, 1), "scan", 1.5))
    calls = []
    got = autotune.tune(lambda *a: calls.append(a), lambda g: None, "k")
    assert got.block == (16, 32, 1) and got.order == "scan" and got.ms == 1.5 and not calls
    data = json.load(open(tmp_path / "t.json"))
    assert data["k"]["order"] == "scan"


def test_candidates_cover_the_stage_shapes_of_each_mode():
    s2 = LinearScan(np.linspace(-1e-2, 1e-2, 256), np.linspace(5e-3, 5e-2, 512))
    for dim, shapes in ((3, {1, 2, 3}), (1, {1}), (2, {2, 3}), (0, {2, 3})):
        got = {c.stage_shape for c in autotune.candidates(s2, both=dim == 3, dimension=dim) if c.stage_shape}
        assert got == shapes


def test_tune_times_every_candidate_and_caches_the_stage_shape(tmp_path, monkeypatch):
    monkeypatch.setenv("USTB_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    s2 = LinearScan(np.linspace(-1e-2, 1e-2, 64), np.linspace(5e-3, 5e-2, 64))
    made = []

    class Ev:
        t = 0.0

        def __init__(self, enable_timing=True):
            pass

        def record(self):
            self.at = Ev.t

        def elapsed_time(self, other):
            return other.at - self.at

    def make(block, order, cpt, shape):
        made.append((block, order, cpt, shape))
        return (block, order, cpt, shape)

    def run(g):  # stage shape 3 is the fastest candidate
        Ev.t += 1.0 if g[3] == 3 else 2.0

    monkeypatch.setattr(autotune.torch.cuda, "Event", Ev)
    monkeypatch.setattr(autotune.torch.cuda, "synchronize", lambda *a: None)
    best = autotune.tune(make, run, "k3", scan=s2, both=True, dimension=3)
    assert best.stage_shape == 3 and {m[3] for m in made} >= {1, 2, 3}
    # the best plan is then tried with 1 to 4 CTAs per tile
    assert {m[2] for m in made if m[3] == 3} >= {1, 2, 3, 4}
    assert json.load(open(tmp_path / "t.json"))["k3"]["stage_shape"] == 3
    again = autotune.tune(lambda *a: 1 / 0, run, "k3")  # from the cache, no search
    assert again.stage_shape == 3


def test_tune_picks_the_ctas_per_tile_after_the_other_knobs(tmp_path, monkeypatch):
    monkeypatch.setenv("USTB_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    s2 = LinearScan(np.linspace(-1e-2, 1e-2, 64), np.linspace(5e-3, 5e-2, 64))

    class Ev:
        t = 0.0

        def __init__(self, enable_timing=True):
            pass

        def record(self):
            self.at = Ev.t

        def elapsed_time(self, other):
            return other.at - self.at

    def run(g):  # waves outer is the best shape; 4 CTAs per tile shorten it further
        block, order, cpt, shape = g
        Ev.t += (1.0 if shape == 1 else 2.0) - (0.25 if cpt == 4 else 0.0)

    monkeypatch.setattr(autotune.torch.cuda, "Event", Ev)
    monkeypatch.setattr(autotune.torch.cuda, "synchronize", lambda *a: None)
    best = autotune.tune(lambda *a: a, run, "k4", scan=s2, both=True, dimension=3)
    assert (best.stage_shape, best.ctas_per_tile) == (1, 4)
    assert json.load(open(tmp_path / "t.json"))["k4"]["ctas_per_tile"] == 4
