"""Autotuner host logic on the CPU: the crossover from per-body-step timing
tables, and the stored tuning file (shape, version, device name)."""
import json
import math
import os

import pytest


def test_crossover_interpolates_between_grid_points():
    from nbody_gb300.autotune import crossover_from

    grid = [1024, 2048, 4096, 8192]
    pp = {n: n * 1e-3 for n in grid}            # the direct sum grows ~ N per body
    bh = {n: 5.0 for n in grid}                 # Barnes-Hut flat
    x = crossover_from(grid, pp, bh)
    assert 4096 < x < 8192
    # pp == bh at N = 5000 on this model; log interpolation of the ratio lands near it
    assert x == pytest.approx(5000, rel=0.1)


def test_crossover_edges():
    from nbody_gb300.autotune import crossover_from

    grid = [256, 512, 1024]
    assert crossover_from(grid, {n: 10.0 for n in grid}, {n: 1.0 for n in grid}) == 256   # BH always cheaper
    assert crossover_from(grid, {n: 1.0 for n in grid}, {n: 10.0 for n in grid}) == 2048  # never cheaper


def test_crossover_exact_at_equal_cost():
    from nbody_gb300.autotune import crossover_from

    grid = [1000, 4000]
    # cost ratio pp/bh = 1/2 at 1000 and 2 at 4000: equal at the geometric mean
    x = crossover_from(grid, {1000: 1.0, 4000: 2.0}, {1000: 2.0, 4000: 1.0})
    assert x == pytest.approx(math.sqrt(1000 * 4000), abs=1)


def test_stored_tuning_file_is_complete():
    from nbody_gb300 import autotune
    from nbody_gb300.ensemble import PP_SHAPES

    path = autotune.default_path("NVIDIA GB300")
    assert os.path.exists(path)
    d = json.load(open(path))
    assert d["version"] == autotune.VERSION and d["device_name"] == "NVIDIA GB300"
    assert d["pp_shape"] in PP_SHAPES and set(d["pp_shape_ms_per_step"]) == set(PP_SHAPES)
    assert 256 <= d["crossover"] <= 65536
    grid = [int(k) for k in d["ns_per_body_step"]["pp"]]
    assert d["crossover"] == autotune.crossover_from(grid, {int(k): v for k, v in d["ns_per_body_step"]["pp"].items()},
                                                     {int(k): v for k, v in d["ns_per_body_step"]["bh"].items()})


def test_env_overrides_the_tuning_path(monkeypatch, tmp_path):
    from nbody_gb300 import autotune

    monkeypatch.setenv("NBODY_TUNE_FILE", str(tmp_path / "t.json"))
    assert autotune.default_path("anything") == str(tmp_path / "t.json")
