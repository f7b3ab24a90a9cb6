"""Bloch-periodic complex runs (k_point != 0) and MEEP's src_vol deposit entries.

CPU: each axis's wrap factor ``eikna`` and each source's deposit entries (per lattice
shift and chunk, merged where MEEP merges them, a seam cell listed twice) against the
reference's own (``tests/golden/src_vol_tables.npz``); the driver's refusals. GPU: the
golden Bloch cases are stepped bit for bit in ``test_gpu_parity.py``; here, the kernel
families a phased run refuses and the batch's refusal.
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver
from meep_gpu_gb300 import sources as S
from meep_gpu_gb300.grid import Grid, cpow_int
from meep_gpu_gb300.pml import normalize_thickness
from tests.golden.make_golden_configs import SRC_VOL_CONFIGS, src_vol_config
from tests.golden_io import GOLDEN


@pytest.fixture(scope="module")
def tables():
    with np.load(GOLDEN / "src_vol_tables.npz") as data:
        return {k: data[k] for k in data.files}


@pytest.mark.parametrize("t", range(SRC_VOL_CONFIGS))
def test_src_vol_entries_are_the_reference_entries(tables, t):
    dims, k, pml, specs = src_vol_config(t)
    grid = Grid(dims, 10, 0.5, "periodic", k)
    eikna = tables[f"c{t}_eikna"]
    for axis in range(3):
        phase = grid.bloch_phase(axis)
        assert (0j if phase is None else phase) == eikna[axis]
    sources = [S.Source(grid, spec["component"], spec["center"], spec["size"], S.make_waveform(spec),
                        spec["amplitude"]) for spec in specs]
    S.bind_src_vols(sources, grid, normalize_thickness(pml) if pml is not None else None)
    for m, source in enumerate(sources):
        cells = [tuple(int(v) for v in c) for c in tables[f"c{t}_s{m}_cells"]]
        assert source.cells == cells, (t, m)
        assert np.array_equal(np.asarray(source.amps, dtype=np.complex128), tables[f"c{t}_s{m}_amps"]), (t, m)


def test_complex_powers_of_a_phase():
    x = (np.cos(0.7), np.sin(0.7))
    assert cpow_int(x, 0) == (1.0, 0.0)
    assert cpow_int(x, 1) == x
    inv = cpow_int(x, -1)
    assert abs(complex(*inv) * complex(*x) - 1) < 1e-15
    two = cpow_int(x, 2)
    assert two == (x[0] * x[0] - x[1] * x[1], x[0] * x[1] + x[1] * x[0])


def test_bloch_refusals():
    with pytest.raises(ValueError, match="complex fields"):
        FdtdDriver((1.2, 1.2, 1.2), 10, force_complex_fields=False, k_point=(0.3, 0, 0))
    with pytest.raises(ValueError, match="lattice vector"):
        FdtdDriver((1.2, 1.2, 1.2), 10, boundaries="metallic", k_point=(0.3, 0, 0))
    d = FdtdDriver((1.2, 1.3, 1.2), 10, boundaries=("periodic", "metallic", "metallic"), k_point=(0.3, 0, 0))
    assert d.grid.has_bloch and d.grid.bloch_phase(1) is None
    # the zone edge is exactly -1
    edge = Grid((1.2, 1.2, 1.2), 10, 0.5, "periodic", (10 * 0.5 / 12, 0, 0))
    assert edge.bloch_phase(0) == complex(-1.0, 0.0)


@pytest.mark.gpu
def test_phased_run_refuses_other_families_and_the_batch(gpu):
    import ctypes

    import torch

    from meep_gpu_gb300 import _lib
    from meep_gpu_gb300.engine import ComplexEngine
    from tests.golden.cases import CASES, build_case
    from meep_gpu_gb300 import Susceptibility

    driver, _, _ = build_case(FdtdDriver, Susceptibility, CASES["bloch"])
    engine = driver.freeze(autotune=False)
    assert isinstance(engine, ComplexEngine) and engine.bloch
    lib = engine.lib
    for family, bz, by in ((1, 32, 8), (2, 32, 4), (5, 32, 4)):
        assert lib.mgb_select_half(engine.re.handle, 0, family, bz, by, 4) == -3
    assert lib.mgb_select_half(engine.re.handle, 0, 4, 32, 4, 4) == 0
    # the pair is the real part then the imaginary part
    assert lib.mgb_step_pair(engine.im.handle, engine.re.handle, 0, 1, None) == -1
    nbytes = lib.mgb_batch_bytes(2, 64, 64)
    buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    handle = ctypes.c_void_p()
    _lib.check(lib, lib.mgb_batch_create(2, 64, 64, buf.data_ptr(), nbytes, ctypes.byref(handle)))
    engine.re.ensure_source_words(0, 10)
    assert lib.mgb_batch_set_slot(handle, 0, engine.re.handle, 10, engine.re._words.data_ptr()) == -3
    lib.mgb_batch_destroy(handle)
    driver.close()
