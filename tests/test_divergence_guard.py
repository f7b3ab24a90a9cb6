"""The divergence guard of dispersive runs (reference ``_DivergenceGuard``,
meep_gpu/driver.py:747-792; energy ``_field_energy`` :3634; interval 20 and limit 1e3,
:319-320).

On the host the guard is fed energy sequences (growth while the sources emit, a runaway
after they stop, decay, non-finite values). The reference's guard compares each sample
after the sources with the running maximum of every sample before it, so it stops a
jump of more than 1e3 times within one interval and an energy that is no longer finite.
On the GPU a driven Lorentz slab whose energy overflows float32 while every field word is
still finite is stopped at the guard's first sample, a passive one runs through, and the
device reduction equals the same sum formed on the host. Gain (negative sigma) is refused
as the reference refuses it.
"""

import math

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from meep_gpu_gb300.driver import STABILITY_CHECK_INTERVAL, STABILITY_GROWTH_LIMIT, DivergenceGuard, FdtdDivergence


class FakeDriver:
    def __init__(self, source_end, dt=0.5):
        self.step_count = 0
        self.dt = dt
        self._source_end = source_end

    @property
    def time(self):
        return self.step_count * self.dt

    def last_source_time(self):
        return self._source_end


def drive(energies, source_end=10.0, every=1):
    """Step a fake driver, feeding ``energies[k]`` at the k-th guard sample."""
    driver = FakeDriver(source_end)
    values = iter(energies)
    guard = DivergenceGuard(driver, energy=lambda: next(values))
    for _ in range(len(energies) * STABILITY_CHECK_INTERVAL):
        driver.step_count += 1
        guard.update()
    return driver, guard


def test_constants_are_the_references():
    assert STABILITY_CHECK_INTERVAL == 20 and STABILITY_GROWTH_LIMIT == 1e3


def test_growth_while_the_sources_emit_is_never_accused():
    # samples at t = 10, 20, ... 40 with the sources on until t = 100: peak only
    driver, guard = drive([1.0, 1e5, 1e9, 1e12], source_end=100.0)
    assert guard.samples == 4 and guard.peak == 1e12


def test_runaway_after_the_sources_raises_at_the_first_sample_past_the_limit():
    # sources stop at t = 10 (sample 1, peak 5); samples every 10 time units. Every
    # sample raises the peak it is compared with (the reference keeps the running max).
    with pytest.raises(FdtdDivergence, match="grew to 5.001e\\+03"):
        drive([5.0, 4.0, 5001.0, 1.0])
    driver, guard = drive([5.0, 4.0, 4999.0, 4.999e6])
    assert guard.peak == 4.999e6


def test_decay_after_the_sources_passes():
    driver, guard = drive([5.0, 3.0, 1.0, 0.5, 4999.0])
    assert guard.samples == 5


def test_non_finite_energy_raises():
    with pytest.raises(FdtdDivergence, match="not finite"):
        drive([1.0, math.inf])
    with pytest.raises(FdtdDivergence, match="not finite"):
        drive([math.nan])


def test_guard_samples_only_at_multiples_of_the_interval():
    calls = []
    driver = FakeDriver(1e9)
    guard = DivergenceGuard(driver, energy=lambda: calls.append(driver.step_count) or 1.0)
    for _ in range(65):
        driver.step_count += 1
        guard.update()
    assert calls == [20, 40, 60]


def lorentz_slab(sigma=1.5, amplitude=1.0, continuous=False):
    d = FdtdDriver((1.6, 1.4, 1.5), 10, force_complex_fields=False, boundaries="metallic")
    d.setup_pml(3)
    x, y, z = d.grid.meshgrid()
    slab = np.abs(x) < 0.2
    d.set_epsilon(np.where(slab, 2.25, 1.0))
    d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05), np.where(slab, sigma, 0.0))
    spec = {"component": "Ez", "center": (-0.4, 0.0, 0.0), "size": (0, 0, 0), "frequency": 0.8,
            "amplitude": amplitude}
    spec.update({"source_type": "continuous"} if continuous else {"source_type": "gaussian", "fwidth": 1.0})
    d.add_source(spec)
    return d


def test_gain_is_refused_as_the_reference_refuses_it():
    d = FdtdDriver((1.6, 1.4, 1.5), 10, force_complex_fields=False, boundaries="metallic")
    with pytest.raises(ValueError, match="negative sigma is gain"):
        d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05), -0.2)


@pytest.mark.gpu
def test_energy_overflow_is_stopped_while_the_field_is_finite(gpu):
    """A field driven past 1.8e19 overflows its float32 energy terms while every E word
    is still finite: the guard raises at its first sample, the E detector would not."""
    d = lorentz_slab(amplitude=1e24, continuous=True)
    with pytest.raises(FdtdDivergence, match="not finite"):
        d.run(num_steps=400)
    assert d.step_count == STABILITY_CHECK_INTERVAL
    assert not d.engine.nonfinite()
    assert np.isfinite(d.get_field("Ez", cell_centered=False)).all()
    d.close()


@pytest.mark.gpu
def test_passive_slab_runs_through(gpu):
    d = lorentz_slab()
    d.run(num_steps=1000, progress_interval=300)
    assert d.step_count == 1000
    d.close()


@pytest.mark.gpu
def test_device_energy_is_the_host_sum(gpu):
    d = lorentz_slab()
    d.run(num_steps=150)
    energy = d.field_energy()
    eps = 1.0 / d.engine.inv_eps[0].cpu().numpy().astype(np.float64)
    host = 0.0
    for c in ("x", "y", "z"):
        e = d.get_field("E" + c, cell_centered=False).astype(np.float64)
        b = d.get_field("B" + c, cell_centered=False).astype(np.float64)
        host += float(np.sum(e * e * eps)) + float(np.sum(b * b))
    assert energy > 0 and abs(energy - host) <= 1e-5 * host
    d.close()
