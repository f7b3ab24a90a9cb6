"""The stated tolerances on the extended paths, checked on the GPU against the float64
oracle at the bench's error cases: fields relative L2 <= 1e-5, flux <= 1e-4 (the folded
80^3 case, the complex 80^3 case at k = 0, the Bloch-periodic 48^3 case)."""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, workloads
from oracle.oracle import BlochPair, Oracle, complex_flux_spectrum, problem_from_driver

pytestmark = pytest.mark.gpu

COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _rel_l2(pairs):
    num = sum(float(np.sum(np.abs(a - b) ** 2)) for a, b in pairs)
    den = sum(float(np.sum(np.abs(b) ** 2)) for _, b in pairs)
    return np.sqrt(num / den)


def _run(name):
    steps = workloads.STEPS[name]
    gpu, flux, _ = workloads.build(name, FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build(name, FdtdDriver)
    return steps, gpu, flux, problem_from_driver(ref)


def test_folded_run_within_tolerance(gpu):
    steps, driver, flux, problem = _run("mirror80")
    oracle = Oracle(problem, "f64")
    oracle.run(steps)
    fields = [(driver.get_field(c, cell_centered=False).astype(np.float64), oracle.field(c)) for c in COMPONENTS]
    assert _rel_l2(fields) <= 1e-5
    expected = oracle.flux_spectrum(0)
    assert np.max(np.abs(flux[0].get_flux_spectrum() - expected)) <= 1e-4 * np.max(np.abs(expected))
    driver.close()


@pytest.mark.parametrize("name", ["complex80", "bloch48"])
def test_complex_runs_within_tolerance(gpu, name):
    steps, driver, flux, problem = _run(name)
    if name == "bloch48":
        pair = BlochPair(problem, "f64")
        pair.run(steps)
        re, im = pair.re, pair.im
    else:
        re, im = Oracle(problem, "f64", "real"), Oracle(problem, "f64", "imag")
        re.run(steps)
        im.run(steps)
    fields = [(driver.get_field(c, cell_centered=False).astype(np.complex128), re.field(c) + 1j * im.field(c))
              for c in COMPONENTS]
    assert _rel_l2(fields) <= 1e-5
    expected = complex_flux_spectrum(re, im, 0)
    assert np.max(np.abs(flux[0].get_flux_spectrum() - expected)) <= 1e-4 * np.max(np.abs(expected))
    driver.close()
