"""The benchmarked configurations at their stated sizes, on the GPU.

* The 80^3 sphere-under-PML workload over its full 2000 steps: every float32 word of
  every component equal to the reference's own words (SHA-256 of each component,
  recorded from the reference by ``tests/golden/make_golden.py digest2000``), the flux
  spectrum within 1e-5 of its peak of the reference's, and the error against the
  float64 oracle stated and bounded.
* The 192^3 Lorentz slab (1000 of its 10,000 steps: the pulse emitted and through the
  slab) and the 192^3 sphere with eight DFT objects (600 of its 5000 steps, five DFT
  samples each): every word equal to the float32 oracle's (the C restatement that
  reproduces the reference's words bit for bit on every golden case), P included, and
  every monitor's transforms within 1e-5 of their peak.
"""

import hashlib
import json
import os

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility, workloads
from oracle.oracle import Oracle, problem_from_driver
from tests import golden_io
from tests.golden.cases import SPHERE80_FULL, build_case

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")
EH = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _oracle_threads():
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))


def test_sphere80_full_run_is_the_reference_words(gpu):
    gold = json.loads((golden_io.GOLDEN / "digest_sphere80_2000.json").read_text())
    steps = gold["steps"]
    assert steps == 2000
    driver, flux, _ = build_case(FdtdDriver, Susceptibility, SPHERE80_FULL)
    driver.run(num_steps=steps)
    assert flux[0].decimation_factor == gold["decimation"]
    for c, expected in gold["sha256"].items():
        words = np.ascontiguousarray(driver.get_field(c, cell_centered=False), dtype=np.float32)
        assert hashlib.sha256(words.tobytes()).hexdigest() == expected, c
    got = flux[0].get_flux_spectrum()
    reference = np.asarray(gold["flux"])
    assert np.max(np.abs(got - reference)) <= 1e-5 * np.max(np.abs(reference))
    # Against the float64 oracle. Flux: 1e-4 of the peak (measured ~1e-7). Fields: by
    # step 2000 the pulse has left through the PML and the remaining field is a small
    # residue, on which float32 rounding weighs more: the reference's own words are
    # 2.7e-5 (relative L2) from float64 there (5.4e-7 at step 600), and these words are
    # the reference's. The bound is 1e-4.
    _oracle_threads()
    mine, _, _ = build_case(FdtdDriver, Susceptibility, SPHERE80_FULL)
    oracle = Oracle(problem_from_driver(mine), "f64")
    oracle.run(steps)
    expected = oracle.flux_spectrum(0)
    assert np.max(np.abs(got - expected)) <= 1e-4 * np.max(np.abs(expected))
    num = sum(float(np.sum((driver.get_field(c, cell_centered=False).astype(np.float64) - oracle.field(c)) ** 2))
              for c in EH)
    den = sum(float(np.sum(oracle.field(c) ** 2)) for c in EH)
    assert np.sqrt(num / den) <= 1e-4
    driver.close()


@pytest.mark.parametrize("name,steps", [("lorentz192", 1000), ("sphere192_8dft", 600)])
def test_192_cube_workloads_are_the_oracle_words(gpu, name, steps):
    driver, flux, dft = workloads.build(name, FdtdDriver)
    driver.run(num_steps=steps, progress_interval=steps)
    _oracle_threads()
    mine, _, _ = workloads.build(name, FdtdDriver)
    oracle = Oracle(problem_from_driver(mine), "f32")
    oracle.run(steps)
    for c in FIELDS:
        got = driver.get_field(c, cell_centered=False)
        bad = int(np.sum(got != oracle.field(c)))
        assert bad == 0, f"{name} {c}: {bad} words differ from the float32 oracle"
    engine = driver.engine
    for m in range(len(engine.pole_tensors)):
        box = engine.pbox
        for q in engine.pole_tensors[m]:
            _, p0, p1 = engine.pole_tensors[m][q]
            got = (p0 if driver.step_count % 2 == 0 else p1).cpu().numpy()
            expected = oracle.polarization_array(m, q)[box[0]:box[1], box[2]:box[3], box[4]:box[5]]
            assert np.array_equal(got, expected), f"{name} P{m} {q}"
    if name == "lorentz192":
        assert engine.pole_tensors, "the Lorentz workload steps a pole"
    for index, monitor in enumerate(flux):
        expected = oracle.flux_spectrum(index)
        got = monitor.get_flux_spectrum()
        assert np.max(np.abs(got - expected)) <= 1e-5 * max(np.max(np.abs(expected)), 1e-300), f"flux {index}"
    for index, monitor in enumerate(dft):
        for c in monitor.components:
            expected = oracle.dft(len(flux) + index, c)
            got = monitor.raw(c).reshape(expected.shape)
            scale = max(float(np.max(np.abs(expected))), 1e-300)
            assert np.max(np.abs(got - expected)) <= 1e-5 * scale, f"dft {index} {c}"
    driver.close()


def test_folded_192_split_is_the_oracle_words(gpu):
    """The folded 192^3 case (the eight-DFT sphere under an even Y and an odd Z plane,
    192 x 97 x 97 stored cells) with each half split into three x ranges, each range's
    ghosts folded on the range's stream: every word equal to the float32 oracle's after
    120 steps run as 1 + 39 + 80 (each call starts without the step before's E fold, so
    every range keeps its B ghosts' state first), every monitor's transforms within 1e-5
    of their peak."""
    chunks = (1, 39, 80)
    driver, flux, dft = workloads.build("mirror192", FdtdDriver)
    driver.kernels = ((4, 32, 4, 4), (4, 16, 16, 4), None, 3)
    for chunk in chunks:
        driver.run(num_steps=chunk, progress_interval=chunk)
    assert driver.engine.split == 3
    _oracle_threads()
    mine, _, _ = workloads.build("mirror192", FdtdDriver)
    oracle = Oracle(problem_from_driver(mine), "f32")
    oracle.run(sum(chunks))
    for c in FIELDS:
        bad = int(np.sum(driver.get_field(c, cell_centered=False) != oracle.field(c)))
        assert bad == 0, f"mirror192 {c}: {bad} words differ from the float32 oracle"
    for index, monitor in enumerate(flux):
        expected = oracle.flux_spectrum(index)
        got = monitor.get_flux_spectrum()
        assert np.max(np.abs(got - expected)) <= 1e-5 * max(np.max(np.abs(expected)), 1e-300), f"flux {index}"
    for index, monitor in enumerate(dft):
        for c in monitor.components:
            expected = oracle.dft(len(flux) + index, c)
            got = monitor.raw(c).reshape(expected.shape)
            # (after 120 steps the pulse has not reached every DFT volume: a transform
            # still below float32's normal range is compared at that floor)
            scale = max(float(np.max(np.abs(expected))), 1.2e-38)
            assert np.max(np.abs(got - expected)) <= 1e-5 * scale, f"dft {index} {c}"
    assert driver.engine.status.item() == 0
    driver.close()
