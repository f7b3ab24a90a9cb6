"""The autotuner's host-side rules, without a GPU: the scratch engine it times candidates
on aliases the run's inverse-epsilon volumes as the run does, and the x-range split it
keeps takes more ranges only when they step at least 1 % faster than fewer, and the
wavefront path is offered to 3-D runs only."""

from types import SimpleNamespace

import numpy as np
import torch

from meep_gpu_gb300.engine import SPLIT_CANDIDATES, Engine, host_volumes


def test_host_volumes_keep_the_run_aliasing():
    iso = torch.arange(24, dtype=torch.float32).reshape(2, 3, 4)
    out = host_volumes([iso, iso, iso])
    assert out[0] is out[1] is out[2]
    assert np.array_equal(out[0], iso.numpy())
    a, b = torch.zeros(2, 3, 4), torch.ones(2, 3, 4)
    out = host_volumes([a, b, a])
    assert out[0] is out[2] and out[0] is not out[1]
    assert np.array_equal(out[1], b.numpy())


class _Scratch:
    """Stands in for the scratch engine: records the split being timed."""

    split_eligible = True

    def __init__(self):
        self.ranges = 0

    def select(self, halves):
        self.halves = halves

    def set_split(self, ranges):
        self.ranges = ranges


def _tuned(times, monkeypatch, nx=192):
    """The split _tune_split keeps when a run of steps with R ranges takes times[R] ms."""
    tuner = Engine.__new__(Engine)
    tuner.grid = SimpleNamespace(shape=(nx, nx, nx))
    scratch = _Scratch()
    monkeypatch.setattr(Engine, "_run_ms", lambda self, s, stream, steps=48: times[s.ranges])
    return tuner._tune_split(scratch, ((4, 32, 4, 4), (4, 16, 16, 4)), None, with_time=True)


def test_split_takes_more_ranges_only_when_one_percent_faster(monkeypatch):
    # the 192^3 sphere on the scratch engine: 3 and 4 ranges within 0.3 % of each other
    times = {0: 7.60, 2: 7.31, 3: 7.03, 4: 7.05, 6: 7.23}
    assert _tuned(times, monkeypatch) == (3, 7.03)
    times = {0: 7.60, 2: 7.31, 3: 7.03, 4: 7.01, 6: 7.23}  # 4 ranges 0.3 % faster: kept at 3
    assert _tuned(times, monkeypatch) == (3, 7.03)
    times = {0: 7.60, 2: 7.31, 3: 7.03, 4: 6.90, 6: 7.23}  # 4 ranges 1.8 % faster: taken
    assert _tuned(times, monkeypatch) == (4, 6.90)
    times = {0: 7.00, 2: 6.97, 3: 6.99, 4: 7.10, 6: 7.20}  # nothing 1 % faster: unsplit
    assert _tuned(times, monkeypatch) == (0, 7.00)


def test_split_skips_ranges_thinner_than_two_planes(monkeypatch):
    times = {r: 10.0 - r for r in (0,) + SPLIT_CANDIDATES}  # every split faster
    ranges, _ = _tuned(times, monkeypatch, nx=8)
    assert ranges == 4  # 6 ranges of an 8-plane grid are refused before they are timed


def _engine_on(grid, conductivity=None):
    engine = Engine.__new__(Engine)
    engine.grid = grid
    engine.conductivity = conductivity or {}
    return engine


def test_wavefront_path_takes_3d_runs_only():
    """The wavefront marches compile the 3-D curl alone: a 2-D or 1-D run never takes
    them (the library refuses it too), while a plain 3-D metallic-x run may."""
    from meep_gpu_gb300.grid import Grid

    assert _engine_on(Grid((4.0, 4.0, 4.0), 10, 0.5, "metallic")).wave_eligible
    two_d = Grid((4.0, 4.0, 0.0), 10, 0.5, {"x": "metallic", "y": "metallic"}, dimensions=2)
    assert two_d.dimensions == 2 and two_d.is_metallic(0)
    assert not _engine_on(two_d).wave_eligible
    lossy = _engine_on(Grid((4.0, 4.0, 4.0), 10, 0.5, "metallic"), conductivity={"Dz": object()})
    assert not lossy.wave_eligible
