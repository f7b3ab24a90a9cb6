"""The CPU oracle against golden vectors recorded from the reference implementation.

The float32 oracle, configured through this package's host code (grid, PML tables,
source tables, monitor registration), must reproduce the reference's stored float32
words bit for bit after N steps, and its flux spectra and DFT accumulators to float32
rounding. The float64 oracle must agree with both to single-precision accuracy.
"""

import hashlib

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from oracle.oracle import Oracle, complex_accumulator, complex_flux_spectrum, problem_from_driver
from tests.golden.cases import CASES, SPHERE80, build_case
from tests import golden_io

FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


def run_case(case, precision="f32", steps=None):
    driver, flux, dft = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    oracle = Oracle(problem, precision)
    oracle.run(steps if steps is not None else case["steps"])
    return driver, oracle


def run_complex_case(case, precision="f32"):
    """A complex case at k = 0 as two real oracle runs (real parts, imaginary parts)."""
    driver, flux, dft = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    parts = []
    for part in ("real", "imag"):
        oracle = Oracle(problem, precision, part)
        oracle.run(case["steps"])
        parts.append(oracle)
    return driver, parts[0], parts[1]


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if c.get("complex") and not c.get("k_point")))
def test_complex_case_is_two_real_oracle_runs(name):
    """The reference's complex run at k = 0: its real words are one float32 oracle run
    driven by real(A), its imaginary words another driven by imag(A); its transforms are
    the two runs' sums, acc_re + i acc_im."""
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, re, im = run_complex_case(case)
    for c in FIELDS:
        assert np.array_equal(re.field(c), gold[c].real), f"{name} {c} real"
        assert np.array_equal(im.field(c), gold[c].imag), f"{name} {c} imag"
    nflux = len(driver._flux_monitors)
    for index in range(nflux):
        expected = gold[f"flux{index}"]
        got = complex_flux_spectrum(re, im, index)
        assert np.max(np.abs(got - expected)) <= 1e-5 * np.max(np.abs(expected)), f"{name} flux {index}"
    for index, monitor in enumerate(driver._dft_monitors):
        total = complex_accumulator(re, im, nflux + index)
        for q, c in enumerate(monitor.components):
            expected = gold[f"dft{index}_{c}"].reshape(len(monitor.frequencies), -1)
            assert np.max(np.abs(total[q] - expected)) <= 1e-5 * np.max(np.abs(expected)), f"{name} dft {c}"
    for m, (pr, pi) in enumerate(zip(re.polarization, im.polarization)):
        for q in pr:
            expected = gold[f"P{m}_{'Ex Ey Ez'.split()[q]}"]
            assert np.array_equal(pr[q][0], expected.real) and np.array_equal(pi[q][0], expected.imag)


def oracle_field(oracle, name):
    return oracle.field(name)


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if not c.get("complex")))
def test_float32_oracle_matches_reference_words(name):
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, oracle = run_case(case)
    for c in FIELDS:
        expected = gold[c]
        got = oracle_field(oracle, c)
        assert got.shape == expected.shape
        mismatched = int(np.sum(got != expected))
        assert mismatched == 0, f"{name} {c}: {mismatched} words differ from the reference"
    nflux = len(driver._flux_monitors)
    for index in range(nflux):
        expected = gold[f"flux{index}"]
        got = oracle.flux_spectrum(index)
        scale = np.max(np.abs(expected))
        assert np.max(np.abs(got - expected)) <= 1e-5 * scale, f"{name} flux {index}"
    for index, monitor in enumerate(driver._dft_monitors):
        for c in monitor.components:
            expected = gold[f"dft{index}_{c}"].reshape(len(monitor.frequencies), -1)
            got = oracle.dft(nflux + index, c)
            assert np.array_equal(got.astype(np.complex64), expected), f"{name} dft {c}"
    for m, pole in enumerate(oracle.polarization):
        for q, (p, _) in pole.items():
            assert np.array_equal(p, gold[f"P{m}_{'Ex Ey Ez'.split()[q]}"]), f"{name} P{m}"


@pytest.mark.parametrize("name", ["sphere_pml", "lorentz_slab", "mixed"])
def test_float64_oracle_agrees_to_single_precision(name):
    case = CASES[name]
    gold = golden_io.fields(name)
    _, oracle64 = run_case(case, "f64")
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        expected = gold[c].astype(np.float64)
        got = oracle64.field(c)
        rel = np.linalg.norm(got - expected) / max(np.linalg.norm(got), 1e-300)
        assert rel < 2e-5, f"{name} {c}: float32 reference vs float64 oracle rel-L2 {rel:.2e}"


def test_sphere80_digest_after_200_steps():
    """The full-size 80^3 sphere-under-PML workload: every word after 200 steps."""
    gold = golden_io.digest()
    driver, oracle = run_case(SPHERE80, steps=gold["steps"])
    assert driver._flux_monitors[0].decimation_factor == gold["decimation"]
    for c, expected in gold["sha256"].items():
        words = np.ascontiguousarray(oracle_field(oracle, c), dtype=np.float32)
        assert hashlib.sha256(words.tobytes()).hexdigest() == expected, c
    flux = oracle.flux_spectrum(0)
    expected = np.asarray(gold["flux"])
    assert np.max(np.abs(flux - expected)) <= 1e-5 * np.max(np.abs(expected))


def test_oracle_detects_a_planted_error():
    """A one-ulp change in one PML coefficient must show up in the words."""
    case = CASES["sphere_pml"]
    gold = golden_io.fields("sphere_pml")
    driver, flux, dft = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    kms, sinv, kps = problem.tables32[(1, 2)]
    kms = kms.copy()
    kms[1] = np.nextafter(kms[1], np.float32(2.0))
    problem.tables32[(1, 2)] = (kms, sinv, kps)
    oracle = Oracle(problem, "f32")
    oracle.run(case["steps"])
    assert any(int(np.sum(oracle.field(c) != gold[c])) for c in FIELDS)
