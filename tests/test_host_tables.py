"""Host-side setup tables against the reference's, recorded in tests/golden/tables.npz."""

import numpy as np
import pytest

from meep_gpu_gb300.dft import FluxMonitor
from meep_gpu_gb300.grid import Grid
from meep_gpu_gb300.pml import PML, one_rank_line, runs_of, slab_index
from meep_gpu_gb300.sources import deposition_table
from tests import golden_io

GOLD, META = golden_io.tables()
GRID = Grid(tuple(META["grid"]["cell_size"]), META["grid"]["resolution"],
            boundaries=META["grid"]["boundaries"])


@pytest.mark.parametrize("thickness", META["pml_thicknesses"])
def test_pml_coefficients_are_the_reference_words(thickness):
    pml = PML(GRID, thickness)
    for axis, name_axis in enumerate("xyz"):
        for lattice, suffix in ((0, ""), (1, "_h")):
            table = pml.tables[(lattice, axis)]
            for name in ("kms", "sinv", "kps"):
                expected = GOLD[f"pml_{thickness}_{name}_{name_axis}{suffix}"]
                assert np.array_equal(getattr(table, name), expected), (thickness, name, name_axis, suffix)


@pytest.mark.parametrize("index", range(len(META["sources"])))
def test_source_tables_are_the_reference_tables(index):
    request = META["sources"][index]
    cells, amps = deposition_table(GRID, request["component"], tuple(request["center"]),
                                   tuple(request["size"]))
    expected_cells = [tuple(int(v) for v in row) for row in GOLD[f"src{index}_cells"]]
    assert cells == expected_cells
    assert np.array_equal(np.asarray(amps, dtype=np.complex128), GOLD[f"src{index}_amps"])


@pytest.mark.parametrize("index", range(len(META["planes"])))
def test_flux_plane_registration_is_the_reference(index):
    plane = META["planes"][index]
    monitor = FluxMonitor(GRID, (0.1, 0.2), tuple(plane["center"]), tuple(plane["size"]),
                          None, 1.0, 1)
    assert tuple(monitor.region) == tuple(int(v) for v in GOLD[f"plane{index}_region"])
    assert np.array_equal(monitor.weights, GOLD[f"plane{index}_weights"])
    assert monitor.measure == float(GOLD[f"plane{index}_measure"])


def test_one_rank_membership_runs():
    # 4-cell faces: span int(4 + 1.5) = 5; integer cells 1..5 low, n-4..n-1 high.
    line = one_rank_line(24, (4, 4), 0, wraps=False)
    assert runs_of(line) == (1, 6, 20, 24)
    line = one_rank_line(24, (4, 4), 1, wraps=False)
    assert runs_of(line) == (0, 5, 19, 24)
    wrapped = one_rank_line(24, (0, 4), 0, wraps=True)
    assert runs_of(wrapped) == (0, 1, 20, 24)
    record = (1, 6, 20, 24)
    rows = slab_index(record, np.arange(24))
    assert list(rows[:7]) == [-1, 0, 1, 2, 3, 4, -1]
    assert list(rows[19:]) == [-1, 5, 6, 7, 8]


def test_array_deposit_words_equal_the_per_step_form():
    from meep_gpu_gb300 import sources as S

    grid = Grid((3.2, 3.2, 3.2), 10)
    srcs = [
        S.Source(grid, "Ez", (-0.8, 0.0, 0.0), (0, 0, 0), S.GaussianWaveform(0.15, 0.1)),
        S.Source(grid, "Ex", (0.05, 0.1, 0.0), (0.3, 0, 0), S.ContinuousWaveform(0.4, width=2.0),
                 amplitude=0.7 - 0.3j),
        S.Source(grid, "Ey", (0.0, 0.0, 0.3), (0, 0, 0),
                 S.CustomWaveform(lambda t: np.exp(-((t - 3.0) ** 2)) * (1 + 0.5j))),
        # magnetic: its current is taken at n*dt, not n*dt + dt/2
        S.Source(grid, "Hx", (0.1, 0.0, 0.0), (0, 0, 0), S.GaussianWaveform(0.15, 0.1)),
        S.Source(grid, "Hz", (0.0, 0.1, 0.0), (0.2, 0, 0), S.ContinuousWaveform(0.4)),
    ]
    S._CURRENT_CACHE.clear()
    for first, steps in ((0, 300), (250, 400), (0, 900), (1000, 17)):
        fast = S.deposit_words(srcs, first, steps, grid.dt)
        slow = S.deposit_words_scalar(srcs, first, steps, grid.dt)
        assert fast.shape == slow.shape
        assert np.array_equal(fast.view(np.uint64), slow.view(np.uint64)), (first, steps)


def test_device_status_word_is_decoded():
    """Bit 1 is a divergence (reported to the caller as such); the wait time-out bits raise."""
    import types

    import torch

    from meep_gpu_gb300.engine import Engine

    def fake(word):
        return types.SimpleNamespace(status=torch.tensor([word], dtype=torch.int32),
                                     STATUS_NONFINITE=1, STATUS_TILE_TIMEOUT=2, STATUS_MMA_TIMEOUT=4,
                                     STATUS_WAVE_TIMEOUT=8,
                                     device_status=lambda: Engine.device_status(fake_obj[0]))

    fake_obj = [None]
    for word, diverged in ((0, False), (1, True)):
        fake_obj[0] = fake(word)
        assert Engine.device_status(fake_obj[0]) == word
        assert Engine.nonfinite(fake_obj[0]) is diverged
    for word in (2, 4, 6, 3, 8, 9):
        fake_obj[0] = fake(word)
        with pytest.raises(RuntimeError, match="timed out"):
            Engine.device_status(fake_obj[0])
    fake_obj[0] = fake(8)
    with pytest.raises(RuntimeError, match="wavefront"):
        Engine.device_status(fake_obj[0])


def test_magnetic_sources_take_their_current_at_the_whole_step():
    from meep_gpu_gb300 import sources as S

    grid = Grid((3.2, 3.2, 3.2), 10)
    wave = S.GaussianWaveform(0.15, 0.1)
    electric = S.Source(grid, "Ez", (0.0, 0.0, 0.0), (0, 0, 0), wave)
    magnetic = S.Source(grid, "Bz", (0.0, 0.0, 0.0), (0, 0, 0), wave)
    assert magnetic.component == "Hz" and magnetic.magnetic and magnetic.comp_index == 5
    assert electric.comp_index == 2 and not electric.magnetic
    n = 123
    e = S.deposit_words([electric], n, 1, grid.dt)[0, 0] / (electric.amps[0].real * grid.dt)
    m = S.deposit_words([magnetic], n, 1, grid.dt)
    assert e == S.current(wave, n * grid.dt + 0.5 * grid.dt, grid.dt)[0]
    assert m[0, 0] == (magnetic.amps[0].real * S.current(wave, n * grid.dt, grid.dt)[0]
                       - magnetic.amps[0].imag * S.current(wave, n * grid.dt, grid.dt)[1]) * grid.dt
