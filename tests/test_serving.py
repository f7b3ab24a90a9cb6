"""Serving: continuous batching of independent simulations.

CPU tests cover the request stream and the admission loop (with a stand-in server that
steps nothing). GPU tests check that every served result is the same alone and in the
mix: the batch computes each slot's float32 words exactly as the plain drop-in does, so
spectra and fields are compared bit for bit, and one served spectrum is held to the
float64 oracle at the stated flux tolerance (relative 1e-4 of the peak).
"""

import numpy as np
import pytest

from meep_gpu_gb300 import serving
from meep_gpu_gb300.serving import Request, make_stream


def test_stream_is_seeded_and_has_the_stated_distributions():
    a = make_stream(512, seed=0)
    b = make_stream(512, seed=0)
    assert [(r.side, r.eps, r.steps, r.arrival) for r in a] == [(r.side, r.eps, r.steps, r.arrival) for r in b]
    assert {r.side for r in a} == set(serving.SIDES)
    assert all(2.0 <= r.eps <= 12.0 for r in a)
    assert all(0.15 * r.side <= r.radius_cells <= 0.4 * r.side for r in a)
    assert all(1000 <= r.steps <= 4000 for r in a)
    gaps = np.diff([r.arrival for r in a])
    assert a[0].arrival == 0.0 and np.all(gaps >= 0)
    assert abs(gaps.mean() - 1 / 40) < 0.2 / 40  # Poisson(40/s)


def test_request_configuration_scales_with_the_cell():
    small = serving.build_request(Request(0, 32, 4.0, 8.0, 100, 0.0))
    large = serving.build_request(Request(1, 64, 4.0, 16.0, 100, 0.0))
    for driver, flux in (small, large):
        n = driver.grid.shape[0]
        assert driver.grid.shape == (n, n, n)
        assert flux.num_frequencies == serving.NFREQ
        # the plane sits at +L/4 and spans the PML-free interior
        assert flux.region[0] == 3 * n // 4 - 1
        assert flux.decimation_factor == 49
    assert serving.footprint_bytes(large[0]) > 7 * serving.footprint_bytes(small[0])


class _StandInServer:
    """The serve() contract without a GPU: a slot advances `rate` steps per launch."""

    def __init__(self, max_slots, budget, rate=50):
        self.max_slots = max_slots
        self.budget_bytes = budget
        self.slots = [None] * max_slots
        self.resident_bytes = 0
        self.rate = rate
        self.replays = 0
        self.peak_bytes = 0
        self.peak_active = 0
        self.admitted_order = []
        self.draining = []

    @property
    def active(self):
        return sum(s is not None for s in self.slots)

    def fits(self, nbytes, slots=1):
        return self.active + slots <= self.max_slots and (self.resident_bytes == 0 or self.resident_bytes + nbytes <= self.budget_bytes)

    def admit(self, job, now):
        slot = self.slots.index(None)
        job.slot, job.admitted = slot, now
        job.done_steps = 0
        self.slots[slot] = job
        self.resident_bytes += job.bytes
        self.admitted_order.append(job.request.index)
        self.peak_bytes = max(self.peak_bytes, self.resident_bytes)
        self.peak_active = max(self.peak_active, self.active)

    def commit(self):
        pass

    def launch(self, steps=None):
        self.replays += 1
        for job in self.slots:
            if job is not None:
                job.done_steps = min(job.request.steps, job.done_steps + self.rate)

    def mark(self):
        return _Event()

    def finish(self):
        for slot, job in enumerate(self.slots):
            if job is not None and job.done_steps >= job.request.steps:
                self.slots[slot] = None
                self.draining.append(job)

    def collect(self, now_fn, wait=False):
        out = []
        for job in self.draining:
            out.append(serving.Result(job.request.index, job.request.side, job.request.steps,
                                      np.zeros(1), job.request.arrival, job.admitted, now_fn()))
            self.resident_bytes -= job.bytes
        self.draining = []
        return out


class _Cfg:
    def __init__(self, nbytes):
        self.nbytes = nbytes


def test_admission_respects_slots_and_budget_and_backfills(monkeypatch):
    sizes = {0: 60, 1: 60, 2: 50, 3: 10, 4: 10, 5: 30, 6: 5}
    requests = [Request(i, 32, 4.0, 8.0, 100 + 40 * i, 0.0) for i in sizes]
    monkeypatch.setattr(serving, "footprint_bytes", lambda cfg: cfg.nbytes)
    server = _StandInServer(max_slots=3, budget=100)
    report = serving.serve(server, requests, realtime=False,
                           build=lambda r: (_Cfg(sizes[r.index]), None))
    assert sorted(r.index for r in report.results) == list(sizes)
    assert server.peak_bytes <= 100 and server.peak_active <= 3
    # the 50-byte request does not fit beside the first 60, so the 10-byte ones backfill
    assert server.admitted_order[:3] == [0, 3, 4]
    assert report.replays == server.replays > 0


class _Event:
    def synchronize(self):
        pass


def test_serving_loop_runs_without_a_device(monkeypatch):
    """The loop's own bookkeeping (no GPU): events are stand-ins, every request finishes."""
    monkeypatch.setattr(serving, "footprint_bytes", lambda cfg: cfg.nbytes)
    server = _StandInServer(max_slots=2, budget=1000, rate=70)
    requests = [Request(i, 32, 4.0, 8.0, 50 + 60 * i, 0.001 * i) for i in range(9)]
    report = serving.serve(server, requests, realtime=True, build=lambda r: (_Cfg(100), None))
    assert sorted(r.index for r in report.results) == list(range(9))
    assert all(r.done >= r.arrival for r in report.results)
    assert report.sims_per_second > 0


# ---------------------------------------------------------------------------------------
# GPU: served results against the plain drop-in and the float64 oracle

SMALL = [Request(0, 24, 6.0, 6.0, 150, 0.0), Request(1, 32, 3.0, 9.0, 233, 0.0),
         Request(2, 40, 11.0, 12.0, 187, 0.0), Request(3, 24, 2.5, 4.0, 301, 0.0),
         Request(4, 32, 8.0, 10.0, 97, 0.0), Request(5, 48, 4.0, 15.0, 140, 0.0)]


def plain(request, kernels, dft_accumulation="direct"):
    driver, flux = serving.build_request(request, kernels=kernels, dft_accumulation=dft_accumulation)
    driver.step_many(request.steps)
    spectrum = flux.get_flux_spectrum()
    fields = {c: driver.get_field(c, cell_centered=False) for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    driver.close()
    return spectrum, fields


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [True, False])
def test_served_spectra_equal_the_plain_solve(gpu, use_graph):
    """Two slots for six requests, 16 steps per replay: requests join as others leave,
    and slots end inside a replay; every spectrum equals the one-at-a-time solve's."""
    server = serving.BatchServer(gpu, max_slots=2, steps_per_replay=16, use_graph=use_graph)
    report = serving.serve(server, SMALL, realtime=False)
    server.close()
    got = report.spectra()
    assert sorted(got) == [r.index for r in SMALL]
    for request in SMALL:
        for kernels in ((0, 32, 4, 4), (1, 64, 8, 8)):
            expected, _ = plain(request, kernels)
            assert np.array_equal(got[request.index], expected), (request.index, kernels)
        # the plain drop-in's default (tensor-core) accumulation: the same spectrum to
        # float32 rounding order
        tensor, _ = plain(request, (0, 32, 4, 4), dft_accumulation="tensor")
        rel = np.max(np.abs(tensor - got[request.index])) / np.max(np.abs(got[request.index]))
        assert rel <= 1e-5, (request.index, rel)


@pytest.mark.gpu
def test_grouped_batches_serve_the_plain_spectra(gpu):
    """Three independent batches on their own streams (one slot each, six requests):
    every spectrum equals the one-at-a-time solve's."""
    server = serving.MultiBatchServer(gpu, groups=3, max_slots=3, steps_per_replay=16)
    assert len(server.servers) == 3 and server.max_slots >= 3
    report = serving.serve(server, SMALL, realtime=False)
    server.close()
    got = report.spectra()
    assert sorted(got) == [r.index for r in SMALL]
    for request in SMALL:
        expected, _ = plain(request, (0, 32, 4, 4))
        assert np.array_equal(got[request.index], expected), request.index


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(32, 4, 4), (64, 2, 8), (32, 8, 2), (64, 4, 1)])
def test_served_fields_equal_the_plain_solve(gpu, shape):
    """All slots at once under another launch shape: every field word equals the alone run."""
    import torch

    server = serving.BatchServer(gpu, max_slots=len(SMALL), steps_per_replay=32, shape=shape)
    jobs = []
    for request in SMALL:
        driver, flux = serving.build_request(request)
        job = serving._Job(request, driver, flux, serving.footprint_bytes(driver))
        server.admit(job, 0.0)
        jobs.append(job)
    server.commit()
    for _ in range(max(r.steps for r in SMALL) // 32 + 1):
        server.launch()
    steps = server.steps()
    server.stream.synchronize()
    for job in jobs:
        assert steps[job.slot] == job.request.steps
        expected_spectrum, expected = plain(job.request, (0, 32, 4, 4))
        assert np.array_equal(job.flux.get_flux_spectrum(), expected_spectrum), job.request.index
        for c, words in expected.items():
            assert np.array_equal(job.driver.get_field(c, cell_centered=False), words), (job.request.index, c)
    torch.cuda.synchronize()
    server.close()


@pytest.mark.gpu
def test_served_spectrum_against_the_float64_oracle(gpu):
    from oracle.oracle import Oracle, problem_from_driver

    request = Request(0, 32, 6.0, 9.0, 400, 0.0)
    server = serving.BatchServer(gpu, max_slots=2, steps_per_replay=64)
    report = serving.serve(server, [request], realtime=False)
    server.close()
    got = report.results[0].spectrum
    driver, _ = serving.build_request(request)
    oracle = Oracle(problem_from_driver(driver), "f64")
    oracle.run(request.steps)
    expected = oracle.flux_spectrum(0)
    rel = np.max(np.abs(got - expected)) / np.max(np.abs(expected))
    assert rel <= 1e-4, f"served flux vs float64 oracle {rel:.2e}"


@pytest.mark.gpu
def test_batch_autotuner_picks_a_candidate(gpu):
    server = serving.BatchServer(gpu, max_slots=4, max_side=48)
    shape = server.autotune(sides=(24, 48), steps=4)
    assert shape in serving.SHAPE_CANDIDATES
    report = serving.serve(server, SMALL[:3], realtime=False)
    server.close()
    for result in report.results:
        expected, _ = plain(SMALL[result.index], (0, 32, 4, 4))
        assert np.array_equal(result.spectrum, expected)


@pytest.mark.gpu
def test_batch_steps_every_golden_configuration_to_the_reference_words(gpu):
    """Slots of different kinds in one batch -- absorbers on some faces, periodic axes,
    Lorentz and Drude poles, extended and continuous sources -- each reach the reference's
    own words (the golden fixtures) after its step count, bit for bit."""
    from meep_gpu_gb300 import FdtdDriver, Susceptibility
    from tests import golden_io
    from tests.golden.cases import CASES, build_case

    # <= 2 monitors a slot; lossy runs, folds and 2-D / 1-D runs are not batched (refused
    # by name); a complex run takes two slots (its two parts), Bloch-phased or not
    names = [n for n in sorted(CASES) if n not in ("mixed", "tile_mixed", "complex_mixed")
             and not CASES[n].get("conductivity") and not CASES[n].get("bloch_monitors")
             and not CASES[n].get("symmetry") and not CASES[n].get("dims")]
    assert {"complex_sphere", "bloch_sphere", "bloch_magnetic", "magnetic"} <= set(names)
    slots = sum(2 if CASES[n].get("complex") else 1 for n in names)
    server = serving.BatchServer(gpu, max_slots=slots, steps_per_replay=16, max_side=72)
    jobs = []
    for name in names:
        driver, flux, dft = build_case(FdtdDriver, Susceptibility, CASES[name])
        request = Request(len(jobs), 0, 1.0, 0.0, CASES[name]["steps"], 0.0)
        job = serving._Job(request, driver, flux[0] if flux else None, serving.footprint_bytes(driver))
        server.admit(job, 0.0)
        jobs.append((name, job, flux, dft))
    server.commit()
    for _ in range(max(CASES[n]["steps"] for n in names) // 16 + 1):
        server.launch()
    server.stream.synchronize()
    for name, job, flux, dft in jobs:
        gold = golden_io.fields(name)
        for c in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz"):
            got = job.driver.get_field(c, cell_centered=False)
            assert np.array_equal(got, gold[c]), (name, c)
        for index, monitor in enumerate(flux):
            expected = gold[f"flux{index}"]
            assert np.max(np.abs(monitor.get_flux_spectrum() - expected)) <= 1e-5 * np.max(np.abs(expected)), name
    server.close()

