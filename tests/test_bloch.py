"""Bloch-periodic complex runs (k_point != 0) and MEEP's src_vol deposit entries.

CPU: each axis's wrap factor ``eikna`` and each source's deposit entries (per lattice
shift and chunk, merged where MEEP merges them, a seam cell listed twice) against the
reference's own (``tests/golden/src_vol_tables.npz``); the driver's refusals; the
oracle's Bloch pair (both parts stepped half by half, the phased operands and lattice
images) against the reference's words. GPU: the golden Bloch cases are stepped bit for
bit in ``test_gpu_parity.py``; here, a larger Bloch run against the float64 oracle, the
kernel families a phased run refuses and the batch's refusal.
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from meep_gpu_gb300 import sources as S
from meep_gpu_gb300.grid import Grid, cpow_int
from meep_gpu_gb300.pml import normalize_thickness
from oracle.oracle import BlochPair, complex_accumulator, complex_flux_spectrum, problem_from_driver
from tests import golden_io
from tests.golden.cases import CASES, build_case
from tests.golden.make_golden_configs import SRC_VOL_CONFIGS, src_vol_config
from tests.golden_io import GOLDEN

FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


def _close(got, expected, tol):
    return np.max(np.abs(got - expected)) <= tol * np.max(np.abs(expected))


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


@pytest.mark.parametrize("name", ["bloch", "bloch_pml", "bloch_sphere", "bloch_magnetic"])
def test_oracle_bloch_pair_matches_reference_words(name):
    """The float32 oracle's two parts, stepped together, are the reference's complex words
    bit for bit; its transforms and spectra match to float32 rounding."""
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, flux, dft = build_case(FdtdDriver, Susceptibility, case)
    pair = BlochPair(problem_from_driver(driver), "f32")
    pair.run(case["steps"])
    for c in FIELDS:
        assert np.array_equal(pair.field(c).astype(np.complex64), gold[c]), (name, c)
    for index in range(len(flux)):
        assert _close(complex_flux_spectrum(pair.re, pair.im, index), gold[f"flux{index}"], 1e-5), (name, index)
    for index, monitor in enumerate(dft):
        total = complex_accumulator(pair.re, pair.im, len(flux) + index)
        for q, c in enumerate(monitor.components):
            expected = gold[f"dft{index}_{c}"].reshape(len(monitor.frequencies), -1)
            assert _close(total[q], expected, 1e-5), (name, c)


def test_float64_bloch_pair_agrees_with_float32():
    case = CASES["bloch_pml"]
    driver, flux, _ = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    runs = {}
    for precision in ("f32", "f64"):
        pair = BlochPair(problem, precision)
        pair.run(case["steps"])
        runs[precision] = pair
    num = sum(float(np.sum(np.abs(runs["f32"].field(c) - runs["f64"].field(c)) ** 2)) for c in FIELDS)
    den = sum(float(np.sum(np.abs(runs["f64"].field(c)) ** 2)) for c in FIELDS)
    assert np.sqrt(num / den) <= 1e-5


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


@pytest.mark.gpu
def test_bloch_run_against_the_float64_oracle(gpu):
    """A Bloch run with poles, a PML and monitors, on the GPU against the float64 oracle
    pair: fields to 1e-5 relative L2, flux to 1e-4."""
    case = dict(CASES["bloch_pml"], steps=120, n=(20, 16, 24))
    driver, flux, _ = build_case(FdtdDriver, Susceptibility, case)
    driver.run(num_steps=case["steps"])
    ref, _, _ = build_case(FdtdDriver, Susceptibility, case)
    pair = BlochPair(problem_from_driver(ref), "f64")
    pair.run(case["steps"])
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        got = driver.get_field(c, cell_centered=False).astype(np.complex128)
        num += float(np.sum(np.abs(got - pair.field(c)) ** 2))
        den += float(np.sum(np.abs(pair.field(c)) ** 2))
    assert np.sqrt(num / den) <= 1e-5
    for index, monitor in enumerate(flux):
        expected = complex_flux_spectrum(pair.re, pair.im, index)
        if np.max(np.abs(expected)) > 0:
            assert _close(monitor.get_flux_spectrum(), expected, 1e-4), index
    driver.close()
