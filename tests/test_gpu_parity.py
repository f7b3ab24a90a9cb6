"""CUDA engine parity: libmeepgb.so against the reference's recorded words and the oracle.

Every stepping kernel is compiled with -fmad=false and follows the reference's
operation order, so the bar for fields is bit-exactness (zero differing float32 words)
against the reference's own words (golden fixtures) and against the float32 oracle.
Monitors form their phases on the device in float64 (CUDA sincos), which may round a
phase word differently from the host's libm once in a while, so DFT accumulators and
flux spectra are held to tolerances: relative 1e-5 of the spectrum's peak against the
reference (a float32-rounding bound), and 1e-4 against the float64 oracle (the stated
flux tolerance).
"""

import hashlib

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from oracle.oracle import Oracle, problem_from_driver
from tests import golden_io
from tests.golden.cases import CASES, SPHERE80, build_case

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


TILES = (1, 64, 8, 8)
GENERIC = (0, 32, 8, 4)
PREFETCH = (2, 32, 4, 4)
WARP_SPECIALIZED = ((2, 16, 8, 4), (3, 64, 8, 8))  # H prefetching, E warp-specialized tiles
L2_PREFETCH = ((4, 32, 4, 4), (5, 16, 8, 4))  # families 0 / 2 with the x chunk prefetched into L2
WAVE = (6, 2, 32, 4, 4, 3)  # the wavefront path: prefetching marches, 32 x 4 tiles, 4-plane chunks,
# 3-step blocks
SPLIT = ((4, 32, 4, 4), (2, 32, 4, 2), None, 3)  # each half as three x-range launches on three streams
YLANES = ((0, 1, 128, 4), (4, 1, 64, 2))  # y on the lanes: CTAs one cell wide in z
MODES = {"tiles": TILES, "generic": GENERIC, "prefetch": PREFETCH, "ws": WARP_SPECIALIZED,
         "l2": L2_PREFETCH, "wave": WAVE, "split": SPLIT, "ylanes": YLANES}


def x_metallic(case) -> bool:
    """Whether a case's x axis is metallic (a 1-D case's x is its one invariant cell)."""
    if case.get("dims"):
        return case["dims"] == 2
    boundaries = case.get("boundaries", "metallic")
    x = boundaries if isinstance(boundaries, str) else boundaries[0]
    return x == "metallic"


def wave_steps(case) -> bool:
    """Whether the wavefront path takes a case (a 3-D run, metallic x, no folds, Bloch or
    conductivity)."""
    return (x_metallic(case) and not case.get("symmetry") and not case.get("k_point")
            and not case.get("conductivity") and not case.get("dims"))


def split_steps(case) -> bool:
    """Whether the x-range split takes a case (metallic x, no Bloch phase; folded runs
    fold each range's ghosts with it)."""
    return x_metallic(case) and not case.get("k_point")


def gpu_case(case, steps=None, kernels=None, chunks=None):
    driver, flux, dft = build_case(FdtdDriver, Susceptibility, case)
    driver.kernels = kernels
    total = steps if steps is not None else case["steps"]
    if chunks:
        done = 0
        for chunk in chunks:
            driver.run(num_steps=chunk)
            done += chunk
        assert done == total
    else:
        driver.run(num_steps=total)
    return driver, flux, dft


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("name", sorted(CASES))
def test_fields_are_the_reference_words(gpu, name, mode):
    """Every kernel family: the TMA tile kernels (z extent a multiple of 4), the generic
    plain-load kernels, their prefetching form, and both with the x chunk prefetched
    into L2."""
    case = CASES[name]
    gold = golden_io.fields(name)
    # the tile kernels step 3-D runs whose z extent is a multiple of 4
    tileable = case["n"][2] % 4 == 0 and not case.get("dims")
    if mode == "wave" and not wave_steps(case):
        pytest.skip("the wavefront path steps 3-D metallic-x runs without folds, Bloch phases or conductivity")
    if mode == "split" and not split_steps(case):
        pytest.skip("the x-range split steps metallic-x runs without Bloch phases")
    if (case.get("conductivity") or case.get("k_point")) and mode not in ("generic", "l2", "wave", "split", "ylanes"):
        pytest.skip("lossy and Bloch-phased runs step with the generic kernels only (the others are refused)")
    if mode in ("tiles", "ws") and not tileable:
        mode = "generic"
    kernels = MODES[mode]
    if (case.get("conductivity") or case.get("k_point")) and mode == "l2":
        kernels = (4, 32, 4, 4)  # lossy and Bloch-phased runs take families 0 and 4
    if case.get("conductivity") and mode == "split":
        kernels = ((4, 32, 4, 4), (0, 32, 4, 2), None, 3)
    driver, flux, dft = gpu_case(case, kernels=kernels)
    if mode == "split":
        engines = [driver.engine.re, driver.engine.im] if case.get("complex") else [driver.engine]
        assert all(e.split == 3 for e in engines)
    elif mode != "wave":  # the wavefront path leaves the per-half choice at its default
        assert driver.engine.uses_tiles == (mode in ("tiles", "ws"))
    else:
        engines = [driver.engine.re, driver.engine.im] if case.get("complex") else [driver.engine]
        assert all(e.wave == WAVE[1:] for e in engines)
    for c in FIELDS:
        got = driver.get_field(c, cell_centered=False)
        mismatched = int(np.sum(got != gold[c]))
        assert mismatched == 0, f"{name} {c}: {mismatched} words differ from the reference"
    for index, monitor in enumerate(flux):
        expected = gold[f"flux{index}"]
        got = monitor.get_flux_spectrum()
        assert np.max(np.abs(got - expected)) <= 1e-5 * np.max(np.abs(expected)), f"{name} flux {index}"
    for index, monitor in enumerate(dft):
        for c in monitor.components:
            expected = gold[f"dft{index}_{c}"]
            got = monitor.raw(c)
            scale = np.max(np.abs(expected))
            assert np.max(np.abs(got - expected)) <= 1e-5 * scale, f"{name} dft {c}"
    # a complex run is two real engines (real and imaginary parts)
    engines = [driver.engine.re, driver.engine.im] if case.get("complex") else [driver.engine]
    for m in range(len(engines[0].pole_tensors)):
        box = engines[0].pbox
        for q in engines[0].pole_tensors[m]:
            parts = []
            for engine in engines:
                _, p0, p1 = engine.pole_tensors[m][q]
                parts.append((p0 if driver.step_count % 2 == 0 else p1).cpu().numpy())
            current = parts[0] if len(parts) == 1 else parts[0] + 1j * parts[1]
            expected = gold[f"P{m}_{'Ex Ey Ez'.split()[q]}"][box[0]:box[1], box[2]:box[3], box[4]:box[5]]
            assert np.array_equal(current, expected), f"{name} P{m}"
    driver.close()


@pytest.mark.parametrize("name", ["mixed", "tile_mixed", "tile_periodic_pml"])
@pytest.mark.parametrize("choice", [(0, 32, 8, 16), (0, 64, 4, 7), (0, 16, 16, 200), (0, 128, 2, 1),
                                    (0, 32, 4, 3), (1, 64, 8, 1), (1, 64, 8, 5), (1, 64, 8, 200),
                                    (2, 32, 8, 16), (2, 64, 4, 7), (2, 32, 4, 1), (2, 128, 2, 3),
                                    (3, 64, 8, 1), (3, 64, 8, 5), (3, 64, 8, 200),
                                    (4, 32, 8, 16), (4, 64, 4, 7), (5, 32, 4, 1), (5, 128, 2, 3)])
def test_launch_shape_does_not_change_a_word(gpu, choice, name):
    """The x chunk (every family) and block shape (generic families) change no word."""
    case = CASES[name]
    if choice[0] == 3:
        choice = ((0, 32, 4, 4), choice)  # the warp-specialized kernel steps the E half
    if (choice[0] == 1 or (isinstance(choice[0], tuple) and choice[1][0] == 3)) and case["n"][2] % 4:
        pytest.skip("the tile kernels need a z extent that is a multiple of 4")
    gold = golden_io.fields(name)
    driver, _, _ = gpu_case(case, kernels=choice)
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), (choice, c)
    driver.close()


@pytest.mark.parametrize("kernels", [TILES, WARP_SPECIALIZED])
@pytest.mark.parametrize("stages", ["2", "3", "6"])
def test_ring_depth_does_not_change_a_word(gpu, stages, kernels, monkeypatch):
    monkeypatch.setenv("MEEPGB_STAGES", stages)
    case = CASES["tile_lorentz"]
    gold = golden_io.fields("tile_lorentz")
    driver, _, _ = gpu_case(case, kernels=kernels)
    assert driver.engine.uses_tiles
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), (stages, c)
    assert driver.engine.status.item() == 0
    driver.close()


@pytest.mark.parametrize("pdl", ["0", "1"])
@pytest.mark.parametrize("kernels", [GENERIC, PREFETCH, L2_PREFETCH, TILES, WARP_SPECIALIZED])
def test_programmatic_launches_change_no_word(gpu, kernels, pdl, monkeypatch):
    """An unsplit plan launches each half as its predecessor's programmatic dependent
    (every step kernel waits for it before touching memory); with MEEPGB_PDL=0 the
    launches are plain. Both step the reference's words, with every kernel family."""
    monkeypatch.setenv("MEEPGB_PDL", pdl)
    case = CASES["tile_lorentz"]
    gold = golden_io.fields("tile_lorentz")
    driver, _, _ = gpu_case(case, kernels=kernels)
    assert driver.engine.split == 0
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), (kernels, pdl, c)
    assert driver.engine.status.item() == 0
    driver.close()


def test_chunked_runs_equal_one_run(gpu):
    case = CASES["lorentz_slab"]
    gold = golden_io.fields("lorentz_slab")
    driver, _, _ = gpu_case(case, chunks=[1, 2, 17, 40])
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), c
    driver.close()


@pytest.mark.parametrize("mode", sorted(MODES))
def test_sphere80_words_after_200_steps(gpu, mode):
    gold = golden_io.digest()
    driver, flux, _ = gpu_case(SPHERE80, steps=gold["steps"], kernels=MODES[mode])
    if mode not in ("wave", "split"):
        assert driver.engine.uses_tiles == (mode in ("tiles", "ws"))
    assert (driver.engine.wave is not None) == (mode == "wave")
    assert (driver.engine.split == 3) == (mode == "split")
    assert (driver.engine.wave is not None) == (mode == "wave")
    for c, expected in gold["sha256"].items():
        words = np.ascontiguousarray(driver.get_field(c, cell_centered=False), dtype=np.float32)
        assert hashlib.sha256(words.tobytes()).hexdigest() == expected, c
    got = flux[0].get_flux_spectrum()
    expected = np.asarray(gold["flux"])
    assert np.max(np.abs(got - expected)) <= 1e-5 * np.max(np.abs(expected))
    driver.close()


def test_flux_against_float64_oracle(gpu):
    """Flux after the pulse has crossed the plane: float32 engine vs float64 oracle."""
    case = dict(CASES["sphere_pml"], steps=400)
    driver, flux, _ = gpu_case(case)
    mine, _, _ = build_case(FdtdDriver, Susceptibility, case)
    oracle = Oracle(problem_from_driver(mine), "f64")
    oracle.run(case["steps"])
    expected = oracle.flux_spectrum(0)
    got = flux[0].get_flux_spectrum()
    rel = np.max(np.abs(got - expected)) / np.max(np.abs(expected))
    assert rel <= 1e-4, f"flux vs float64 oracle {rel:.2e}"
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = driver.get_field(c, cell_centered=False).astype(np.float64)
        b = oracle.field(c)
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), c
    driver.close()


def test_autotuned_choice_steps_the_same_words(gpu):
    """Whatever the autotuner picks, the words are the reference's."""
    case = CASES["tile_lorentz"]
    gold = golden_io.fields("tile_lorentz")
    driver, _, _ = gpu_case(case)
    assert driver.engine.choice is not None
    for c in FIELDS:
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), c
    driver.close()


def test_autotuner_times_the_same_volumes(gpu, monkeypatch):
    """The autotuner's scratch engine aliases the inverse-epsilon volumes as the run does
    (an isotropic run's E half reads one volume; a scratch with three would time another
    workload and rank the launch shapes differently)."""
    from meep_gpu_gb300 import engine as engine_mod

    engine_mod._AUTOTUNE_CACHE.clear()
    distinct = []
    original = engine_mod.Engine.finish

    def recording(self):
        distinct.append(len({t.data_ptr() for t in self.inv_eps}))
        return original(self)

    monkeypatch.setattr(engine_mod.Engine, "finish", recording)
    driver, _, _ = gpu_case(CASES["tile_lorentz"])
    assert len(distinct) >= 2, "the autotuner built no scratch engine"
    assert set(distinct) == {1}, distinct
    driver.close()


def test_nonfinite_detector_raises(gpu):
    """A current large enough to overflow float32 is reported by the run, not returned."""
    from meep_gpu_gb300 import FdtdDivergence
    driver = FdtdDriver((1.2, 1.2, 1.2), 10, force_complex_fields=False, boundaries="metallic")
    driver.add_source({"source_type": "continuous", "component": "Ez", "center": (0, 0, 0),
                       "size": (0, 0, 0), "frequency": 0.5, "amplitude": 1e40})
    with pytest.raises(FdtdDivergence):
        driver.run(num_steps=40, progress_interval=10)
    driver.close()
