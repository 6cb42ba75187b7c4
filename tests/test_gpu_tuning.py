"""Autotuning (eikx_autotune3d): the chosen configuration is used by default solves of the
same grid class, survives a save/load round trip, and never changes the travel times."""
import json

import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def test_autotune_choice_is_used_and_exact(ctx, oracle, tmp_path):
    rng = np.random.default_rng(5)
    shape = (45, 38, 27, 50., 50., 50.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    srcs = [(rng.uniform(0, (nx - 1) * 50.), rng.uniform(0, (ny - 1) * 50.), rng.uniform(0, (nz - 1) * 50.))
            for _ in range(3)]
    t = ctx.autotune3d(srcs, ex.F32)
    assert t["sweep_kernel"] in (1, 2) and 1 <= t["block_shape"] <= 3 and t["blocks_per_sm"] >= 1
    assert t["candidates"] >= 7 and 0 < t["ms_per_sweep"] <= t["default_ms_per_sweep"]
    opt = ex.Options(n_sweeps=3, tolerance=-1, factored_radius=3)     # all "auto": takes the tuned choice
    out = ctx.solve3d(srcs, opt, ex.F32)
    for i, p in enumerate(srcs):
        cell = [min(n - 2, int(q / 50.)) for q, n in zip(p, (nx, ny, nz))]
        ref = oracle.solve3d(s, shape, cell, p, n_sweeps=3, radius=3)
        assert np.array_equal(_bits(out[i]), _bits(ref)), i

    path = tmp_path / "tuning.jsonl"
    ctx.save_tuning(str(path))
    rows = [json.loads(line) for line in path.read_text().splitlines()]
    assert any(r["nx"] == 64 and r["ny"] == 64 and r["nz"] == 32 and r["nsrc"] == 4 and
               r["block_shape"] == t["block_shape"] for r in rows)
    other = ex.Context(0)
    other.load_tuning(str(path))
    other.save_tuning(str(tmp_path / "again.jsonl"))
    assert (tmp_path / "again.jsonl").read_text() == path.read_text()

    bad = tmp_path / "bad.jsonl"
    bad.write_text("not a tuning line\n")
    with pytest.raises(ex.InvalidArgument):
        other.load_tuning(str(bad))


def test_invalid_tuning_options_are_rejected(ctx):
    ctx.set_grid3d(5, 5, 5, 10., 10., 10.)
    ctx.set_slowness3d(np.full(64, 1 / 3000., np.float32))
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d([(10., 10., 10.)], ex.Options(block_shape=7))
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d([(10., 10., 10.)], ex.Options(sweep_kernel=5))
