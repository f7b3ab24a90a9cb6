"""D and B conductivity (material sigma and ``mp.Absorber``).

CPU: the host tables against fixtures recorded from the reference (absorber ramps,
condfac / condinv words, the chunks that keep a conductivity under a one-rank PML), the
oracle's own restatement of those chunks against the product's, the driver's
validation and refusals, and the float64 oracle against the reference's float32 words.
GPU: the lossy kernels bit-exact against the reference's words and the float32 oracle,
on every launch shape, and refused by name where a lossy run is not carried.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from meep_gpu_gb300 import AbsorberLayer, FdtdDriver, Susceptibility, Unsupported
from meep_gpu_gb300 import conductivity as cond
from meep_gpu_gb300.grid import IYEE, Grid
from meep_gpu_gb300.pml import normalize_thickness
from oracle.oracle import Oracle, keeps_volume, problem_from_driver
from tests import golden_io
from tests.golden.cases import CASES, build_case

GOLDEN = Path(__file__).resolve().parent / "golden"
UNSUPPORTED = -3  # MGB_ERR_UNSUPPORTED
FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")
LOSSY = sorted(name for name, case in CASES.items() if case.get("conductivity"))


@pytest.fixture(scope="module")
def tables():
    meta = json.loads((GOLDEN / "conductivity_tables.json").read_text())
    with np.load(GOLDEN / "conductivity_tables.npz") as data:
        arrays = {k: data[k] for k in data.files}
    return meta, arrays


# --- host tables against the reference -----------------------------------------------
def test_absorber_ramps_are_the_reference_words(tables):
    meta, arrays = tables
    for g, spec in enumerate(meta["absorber_grids"]):
        grid = Grid(spec["cell"], spec["resolution"], 0.5, spec["boundaries"])
        layers = [AbsorberLayer(t, a, side) for t, a, side in spec["layers"]]
        volumes = cond.absorber_conductivity(grid, layers)
        for name in cond.CONDUCTIVITY_COMPONENTS:
            assert np.array_equal(volumes[name], arrays[f"absorber{g}_{name}"]), (g, name)


def test_coefficients_are_the_reference_words(tables):
    meta, arrays = tables
    fac, inv = cond.coefficients(arrays["coef_sigma"], meta["coef_dt"])
    assert np.array_equal(fac, arrays["coef_condfac"])
    assert np.array_equal(inv, arrays["coef_condinv"])


def test_keeping_chunks_are_the_reference_cells(tables):
    """The product's per-axis pieces and 27-bit masks, and the oracle's owner-volume
    restatement, both give the reference's cells for every component."""
    meta, arrays = tables
    for g, spec in enumerate(meta["chunk_grids"]):
        grid = Grid(spec["cell"], 10, 0.5, spec["boundaries"])
        faces = normalize_thickness(spec["pml"])
        metallic = tuple(int(grid.is_metallic(a)) for a in range(3))
        for t in range(meta["chunk_trials"]):
            sigma = arrays[f"chunks{g}_{t}_sigma"]
            for name, iyee in IYEE.items():
                if name[0] not in "DB":
                    continue
                expected = np.unpackbits(arrays[f"chunks{g}_{t}_{name}"])[:sigma.size].reshape(sigma.shape)
                mask = cond.keeps_mask(grid, faces, sigma)
                lines = [cond.piece_line(grid.shape[a], faces[a], iyee[a], grid.axis_wraps(a)).astype(int)
                         for a in range(3)]
                px, py, pz = np.meshgrid(*lines, indexing="ij")
                product = ((mask >> (px * 9 + py * 3 + pz)) & 1).astype(bool)
                assert np.array_equal(product, expected.astype(bool)), (g, t, name)
                oracle = keeps_volume(grid.shape, metallic, faces, iyee, sigma)
                assert np.array_equal(oracle, expected.astype(bool)), (g, t, name)


# --- driver API -------------------------------------------------------------------------
def small_driver(**kwargs):
    return FdtdDriver((1.4, 1.2, 1.6), 10, force_complex_fields=False, boundaries="metallic", **kwargs)


def test_conductivity_spellings_and_removal():
    d = small_driver()
    d.set_conductivity(0.2)
    vols = d.conductivity_volumes()
    assert all(vols[c] is not None and np.all(vols[c] == np.float32(0.2)) for c in cond.D_COMPONENTS)
    assert all(vols[c] is None for c in cond.B_COMPONENTS)
    padded = np.full(tuple(n + 1 for n in d.grid.shape), 0.1)
    d.set_conductivity(padded)
    assert d.conductivity_volumes()["Dy"].shape == d.grid.shape
    d.set_conductivity({"Dz": 0.3})
    vols = d.conductivity_volumes()
    assert vols["Dx"] is None and vols["Dy"] is None and np.all(vols["Dz"] == np.float32(0.3))
    d.set_conductivity(0.0)
    assert not d.has_conductivity
    d.set_b_conductivity({"By": 0.4})
    assert d.has_conductivity and d.conductivity_volumes()["By"] is not None
    d.set_b_conductivity(None)
    assert not d.has_conductivity


@pytest.mark.parametrize("bad,error", [(-0.1, ValueError), (float("nan"), ValueError),
                                       (0.1 + 0.2j, ValueError), (np.ones((3, 3)), ValueError),
                                       (np.ones((5, 5, 5)), ValueError), ({"Ex": 0.1}, ValueError)])
def test_conductivity_refusals(bad, error):
    with pytest.raises(error):
        small_driver().set_conductivity(bad)


def test_absorber_adds_to_the_material_sigma():
    d = small_driver()
    layers = [AbsorberLayer(0.3, axis, side) for axis in range(3) for side in ("low", "high")]
    d.set_absorber(layers)
    d.set_conductivity(0.05)
    d.set_b_conductivity(0.02)
    both = d.conductivity_volumes()
    raw = cond.absorber_conductivity(d.grid, layers)
    for c in cond.D_COMPONENTS:
        assert np.array_equal(both[c], (raw[c] + np.float32(0.05).astype(np.float64)).astype(np.float32))
    for c in cond.B_COMPONENTS:
        assert np.array_equal(both[c], (raw[c] + np.float32(0.02).astype(np.float64)).astype(np.float32))
    # the D read-back that already carries the ramp is not ramped twice
    d.set_conductivity(0.05, absorber_included=True)
    assert np.all(d.conductivity_volumes()["Dx"] == np.float32(0.05))
    d.set_absorber([])
    assert np.all(d.conductivity_volumes()["Bx"] == np.float32(0.02))
    with pytest.raises(TypeError):
        d.set_absorber([(0.3, 0, "low")])
    with pytest.raises(ValueError):
        AbsorberLayer(0.0, 0, "low")
    with pytest.raises(ValueError):
        AbsorberLayer(0.3, 3, "low")


def test_source_near_a_lossy_pml_is_refused():
    d = small_driver()
    d.setup_pml(3)
    d.set_conductivity(0.3)  # reaches every layer
    with pytest.raises(ValueError, match="inside every absorbing face"):
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.35, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.15, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
    # a conductivity that stays out of the layers takes no refusal
    e = small_driver()
    e.setup_pml(3)
    x, y, z = e.grid.meshgrid()
    e.set_conductivity(np.where(x * x + y * y + z * z < 0.1 ** 2, 0.3, 0.0))
    e.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.35, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
    # a PML set up after a lossy run's sources is checked against them
    f = small_driver()
    f.set_conductivity(0.3)
    f.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.35, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
    with pytest.raises(ValueError, match="inside every absorbing face"):
        f.setup_pml(3)


def test_overlapping_pml_chunks_are_refused():
    grid = Grid((0.5, 1.0, 1.0), 10, 0.5, "metallic")
    with pytest.raises(Unsupported):
        cond.piece_line(grid.nx, (3, 3), 0, False)


# --- oracle ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", [n for n in LOSSY if not CASES[n].get("complex")])
def test_float64_oracle_agrees_to_single_precision(name):
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    oracle = Oracle(problem_from_driver(driver), "f64")
    oracle.run(case["steps"])
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        expected = gold[c].astype(np.float64)
        got = oracle.field(c)
        rel = np.linalg.norm(got - expected) / max(np.linalg.norm(got), 1e-300)
        assert rel < 2e-5, f"{name} {c}: rel-L2 {rel:.2e}"


def test_a_conductivity_changes_the_fields():
    """The oracle's lossy run is not the lossless one (the loss is live)."""
    case = CASES["cond_pml"]
    lossy, _, _ = build_case(FdtdDriver, Susceptibility, case)
    plain = dict(case)
    plain.pop("conductivity")
    lossless, _, _ = build_case(FdtdDriver, Susceptibility, plain)
    a = Oracle(problem_from_driver(lossy), "f32")
    b = Oracle(problem_from_driver(lossless), "f32")
    a.run(40)
    b.run(40)
    assert not np.array_equal(a.field("Ez"), b.field("Ez"))


# --- GPU --------------------------------------------------------------------------------
def lossy_big(kernels=None):
    """The 40^3 lossy workload (PML on x and y, absorber on z, D and B sigma, a pole, a
    lossy extended source, a flux plane)."""
    from meep_gpu_gb300 import workloads

    d, flux, _ = workloads.build("lossy40", FdtdDriver, kernels=kernels)
    return d, flux[0]


@pytest.mark.gpu
@pytest.mark.parametrize("kernels", [(0, 32, 4, 4), (0, 16, 8, 3), (0, 64, 2, 40), (4, 32, 4, 4)])
def test_lossy_run_is_the_float32_oracle(gpu, kernels):
    steps = 150
    d, flux = lossy_big(kernels)
    d.run(num_steps=steps)
    assert d.engine.uses_tiles is False
    ref, _ = lossy_big()
    oracle = Oracle(problem_from_driver(ref), "f32")
    oracle.run(steps)
    for c in FIELDS:
        got = d.get_field(c, cell_centered=False)
        assert int(np.sum(got != oracle.field(c))) == 0, c
    expected = oracle.flux_spectrum(0)
    assert np.max(np.abs(flux.get_flux_spectrum() - expected)) <= 1e-5 * np.max(np.abs(expected))
    d.close()


@pytest.mark.gpu
def test_lossy_run_error_against_float64(gpu):
    """The stated bars against the float64 oracle: fields rel-L2 1e-5, flux 1e-4."""
    steps = 300
    d, flux = lossy_big()
    d.run(num_steps=steps)
    ref, _ = lossy_big()
    oracle = Oracle(problem_from_driver(ref), "f64")
    oracle.run(steps)
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        got = d.get_field(c, cell_centered=False).astype(np.float64)
        want = oracle.field(c)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5, c
    expected = oracle.flux_spectrum(0)
    assert np.max(np.abs(flux.get_flux_spectrum() - expected)) <= 1e-4 * np.max(np.abs(expected))
    d.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", LOSSY)
@pytest.mark.parametrize("kernels", [(0, 32, 8, 16), (0, 64, 4, 7), (0, 128, 2, 1)])
def test_lossy_launch_shape_does_not_change_a_word(gpu, name, kernels):
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    driver.kernels = kernels
    driver.run(num_steps=case["steps"])
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), (kernels, c)
    driver.close()


@pytest.mark.gpu
def test_lossy_run_refuses_the_other_kernel_families(gpu):
    from meep_gpu_gb300 import _lib

    d, _ = lossy_big()
    engine = d.freeze(autotune=False)
    lib = engine.lib
    for family, bz, by in ((1, 32, 8), (2, 32, 4), (3, 32, 8), (5, 32, 4)):
        for part in (0, 1):
            assert lib.mgb_select_half(engine.handle, part, family, bz, by, 4) == UNSUPPORTED
            assert "generic kernels" in _lib.last_error(lib)
    assert lib.mgb_select_half(engine.handle, 0, 0, 32, 4, 4) == 0
    assert lib.mgb_select_half(engine.handle, 1, 4, 32, 4, 4) == 0
    d.close()


@pytest.mark.gpu
def test_lossy_autotune_picks_a_generic_shape(gpu):
    d, _ = lossy_big()
    engine = d.freeze()
    (h, e) = engine.choice
    assert h[0] in (0, 4) and e[0] in (0, 4)
    d.close()


@pytest.mark.gpu
def test_adjoint_and_batch_refuse_a_lossy_run(gpu):
    import ctypes

    import torch

    from meep_gpu_gb300 import _lib
    from meep_gpu_gb300.adjoint import FluxAdjoint

    d, flux = lossy_big()
    with pytest.raises(Unsupported):
        FluxAdjoint(d, flux, ((10, 20), (10, 20), (10, 20)), 10)
    engine = d.freeze(autotune=False)
    lib = engine.lib
    nbytes = lib.mgb_batch_bytes(2, 64, 64)
    buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    handle = ctypes.c_void_p()
    _lib.check(lib, lib.mgb_batch_create(2, 64, 64, buf.data_ptr(), nbytes, ctypes.byref(handle)))
    engine.ensure_source_words(0, 10)
    assert lib.mgb_batch_set_slot(handle, 0, engine.handle, 10, engine._words.data_ptr()) == UNSUPPORTED
    assert "conductivity" in _lib.last_error(lib)
    lib.mgb_batch_destroy(handle)
    d.close()
