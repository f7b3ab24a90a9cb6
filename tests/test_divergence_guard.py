"""The divergence guard of dispersive runs (reference ``_DivergenceGuard``,
meep_gpu/driver.py:747-792; energy ``_field_energy`` :3634; interval 20 and limit 1e3,
:319-320).

On the host the guard is fed energy sequences; on the GPU a Lorentz slab with gain
(negative sigma) grows smoothly while staying finite and is stopped by the guard, a
passive one is not, and the device reduction equals the same sum formed on the host.
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


def gain_slab(sigma):
    d = FdtdDriver((1.6, 1.4, 1.5), 10, force_complex_fields=False, boundaries="metallic")
    d.setup_pml(3)
    x, y, z = d.grid.meshgrid()
    slab = np.abs(x) < 0.2
    d.set_epsilon(np.where(slab, 2.25, 1.0))
    d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05), np.where(slab, sigma, 0.0))
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.4, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.8, "fwidth": 1.0})
    return d


@pytest.mark.gpu
def test_gain_slab_is_stopped_while_finite(gpu):
    d = gain_slab(-0.2)
    with pytest.raises(FdtdDivergence, match="grew"):
        d.run(num_steps=2000)
    # the sources stop at t = 10 (step 200); the float32 oracle's energy passes 1e3 times
    # the peak at t = 20
    assert d.step_count == 400
    assert not d.engine.nonfinite()
    d.close()


@pytest.mark.gpu
def test_passive_slab_runs_through(gpu):
    d = gain_slab(1.5)
    d.run(num_steps=1000, progress_interval=300)
    assert d.step_count == 1000
    d.close()


@pytest.mark.gpu
def test_device_energy_is_the_host_sum(gpu):
    d = gain_slab(1.5)
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
