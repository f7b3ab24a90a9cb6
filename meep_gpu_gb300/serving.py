"""Continuous batching of independent FDTD simulations on one GPU.

The reference steps one simulation per process and GPU (``meep_gpu/driver.py:3419``,
``README.md:127``); a stream of independent requests there is a queue solved one at a
time. Here a :class:`BatchServer` keeps every admitted simulation's fields, PML state and
DFT accumulators resident in HBM as a slot of one batch (``mgb_batch_*`` in
``include/meepgb.h``) and advances all slots together with batched step kernels (one CTA
per work item of a launch shape the batch autotuner picks), replayed as a captured CUDA
graph of ``steps_per_replay`` steps. Requests that arrive
while others run are admitted as soon as a slot and the HBM budget allow (continuous
batching); finished slots are read out (flux spectrum) and freed between replays. Each
slot computes the same float32 words as the same simulation stepped alone, so a served
spectrum equals the plain drop-in's bit for bit.

The served workload (:func:`make_stream`): sphere-under-PML cubes of side
{32, 48, 64, 96, 128} cells at resolution 10, 8-cell PML, sphere eps ~ U[2, 12] and radius
~ U[0.15, 0.4] x side cells, an Ez Gaussian point source (fcen 0.15, df 0.1) at x = -L/4
and a 64-frequency x-normal flux plane at x = +L/4 spanning the PML-free interior, step
counts ~ U[1000, 4000], arrivals Poisson(40/s) -- seeded synthetic inputs, no dataset.
"""

from __future__ import annotations

import ctypes
import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .grid import Unsupported
from .sources import deposit_words

SIDES = (32, 48, 64, 96, 128)
RESOLUTION = 10
PML_CELLS = 8
NFREQ = 64
# Launch shapes (block_z, block_y, x_chunk, family) the batch autotuner times: family 2
# the prefetching marches, 4 the generic marches with the x chunk prefetched into L2.
SHAPE_CANDIDATES = ((32, 4, 4, 2), (32, 8, 4, 2), (32, 4, 8, 2), (32, 2, 8, 2), (64, 2, 4, 2),
                    (64, 4, 4, 2), (32, 8, 2, 2), (32, 4, 2, 2),
                    (32, 4, 4, 4), (32, 8, 4, 4), (32, 4, 8, 4), (32, 2, 8, 4), (64, 4, 4, 4),
                    (32, 4, 2, 4))
_SHAPE_CACHE: Dict[tuple, Tuple[int, ...]] = {}


@dataclass
class Request:
    """One served simulation: a sphere-under-PML cube and its flux spectrum."""

    index: int
    side: int
    eps: float
    radius_cells: float
    steps: int
    arrival: float  # seconds after the stream starts


def make_stream(count: int = 512, rate: float = 40.0, sides: Sequence[int] = SIDES,
                steps: Tuple[int, int] = (1000, 4000), seed: int = 0) -> List[Request]:
    """Seeded request stream: Poisson arrivals, uniform side, eps, radius and step count."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(count):
        side = int(rng.choice(np.asarray(sides)))
        out.append(Request(index=i, side=side, eps=float(rng.uniform(2.0, 12.0)),
                           radius_cells=float(rng.uniform(0.15, 0.4) * side),
                           steps=int(rng.integers(steps[0], steps[1] + 1)),
                           arrival=float(arrivals[i])))
    return out


def build_request(request: Request, driver_cls=None, **driver_kwargs):
    """Configure a driver for one request (host work only); returns ``(driver, flux)``."""
    if driver_cls is None:
        from .driver import FdtdDriver as driver_cls  # noqa: N813
    length = request.side / RESOLUTION
    d = driver_cls(cell_size=(length, length, length), resolution=RESOLUTION, courant=0.5,
                   force_complex_fields=False, boundaries="metallic", **driver_kwargs)
    d.setup_pml(PML_CELLS)
    x, y, z = d.grid.meshgrid()
    radius = request.radius_cells / RESOLUTION
    d.set_epsilon(np.where(x * x + y * y + z * z < radius * radius, request.eps, 1.0).astype(np.float32))
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-length / 4, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
    span = length - 2 * PML_CELLS / RESOLUTION
    flux = d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=NFREQ, center=(length / 4, 0.0, 0.0),
                              size=(0, span, span), decimation_factor=0)
    d.prepare()
    return d, flux


def footprint_bytes(driver) -> int:
    """Device bytes one simulation keeps resident (fields, materials, PML state, DFT)."""
    cells = driver.grid.total_cells
    volumes = 9 + len({id(a) for a in driver._inv_eps})
    if driver.pml is not None and driver.pml.is_active:
        volumes += 15  # B, f_w of H and E, fu of B and D: three components each
    total = 4 * volumes * cells
    for monitor in list(driver._flux_monitors) + list(driver._dft_monitors):
        total += 4 * len(monitor.components) * monitor.num_frequencies * 2 * monitor.cells
    total += 8 * sum(len(s.cells) for s in driver._sources) * 4096
    # a complex run keeps two parts (the material tables are shared, counted twice here)
    return 2 * total if driver.complex_fields else total


@dataclass
class _Job:
    request: Request
    driver: object
    flux: object
    bytes: int
    slot: int = -1
    engine: object = None
    slots: Tuple[int, ...] = ()  # every slot the job holds (two for a complex run)

    @property
    def slots_needed(self) -> int:
        """Slots the job steps in: one, or two for complex fields (its real and imaginary
        parts, which at k = 0 step independently)."""
        return 2 if getattr(self.driver, "complex_fields", False) else 1
    words: Optional[torch.Tensor] = None
    admitted: float = 0.0
    readback: object = None  # (pinned host spectrum, event) once its reduction is queued


@dataclass
class Result:
    index: int
    side: int
    steps: int
    spectrum: np.ndarray
    arrival: float
    admitted: float
    done: float

    @property
    def latency(self) -> float:
        """Time to spectrum: arrival to the host holding the spectrum."""
        return self.done - self.arrival


class BatchServer:
    """A slot table of resident simulations stepped together on one GPU.

    The host tracks every slot's step (each launch of G batch steps advances every
    running slot by G, up to its end), so the loop never waits on the device to learn
    which slots finish: right after queueing a replay it queues the flux reductions and
    read-backs of the slots that replay completes, frees their slots for the next
    commit, and collects the spectra once their events have completed.
    """

    def __init__(self, device: Optional[torch.device] = None, max_slots: int = 32,
                 budget_bytes: Optional[int] = None, steps_per_replay: int = 64,
                 use_graph: bool = True, shape: Optional[Tuple[int, int, int]] = None,
                 max_side: int = max(SIDES), max_monitor_cells: Optional[int] = None):
        if not torch.cuda.is_available():
            raise RuntimeError("meep_gpu_gb300 serving steps on a CUDA GPU and none is visible")
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.stream = torch.cuda.Stream(device=self.device)
        self.setup_stream = torch.cuda.Stream(device=self.device)
        self.max_slots = int(max_slots)
        self.steps_per_replay = int(steps_per_replay)
        self.use_graph = bool(use_graph)
        if budget_bytes is None:
            free, _total = torch.cuda.mem_get_info(self.device)
            budget_bytes = int(0.5 * free)
        self.budget_bytes = int(budget_bytes)
        self.resident_bytes = 0
        # work capacity: every slot as large as the largest admissible grid at the
        # smallest item (32 x 1 x 1 cells is below every candidate shape)
        items = math.ceil(max_side / 32) * max_side * max_side
        # a flux plane's region is two cells thick (the centred average's neighbours)
        plane = max_monitor_cells if max_monitor_cells is not None else 2 * max_side * max_side
        self.max_side = int(max_side)
        self.max_work = self.max_slots * items
        self.max_dft_work = self.max_slots * 2 * math.ceil(plane / 256)
        nbytes = self.lib.mgb_batch_bytes(self.max_slots, self.max_work, self.max_dft_work)
        self.tables = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        if self.tables.data_ptr() % 256:
            raise RuntimeError("batch table buffer is not 256-byte aligned")
        handle = ctypes.c_void_p()
        _lib.check(self.lib, self.lib.mgb_batch_create(self.max_slots, self.max_work, self.max_dft_work,
                                                       self.tables.data_ptr(), nbytes, ctypes.byref(handle)))
        self.handle = handle
        self.slots: List[Optional[_Job]] = [None] * self.max_slots
        self.draining: List[_Job] = []
        self.shape = (32, 4, 4, 2)
        if shape is not None:
            self.set_shape(shape)
        self.replays = 0

    # --- configuration ------------------------------------------------------------------
    def set_shape(self, shape: Sequence[int]) -> None:
        """(block_z, block_y, x_chunk[, family]): the CTA's (z, y) cells and x planes per
        item, and the marches it runs (family 2 by default, or 4)."""
        shape = tuple(int(v) for v in shape)
        if len(shape) == 3:
            shape = shape + (2,)
        _lib.check(self.lib, self.lib.mgb_batch_set_shape(self.handle, *shape[:3]))
        _lib.check(self.lib, self.lib.mgb_batch_set_family(self.handle, shape[3]))
        self.shape = shape

    def autotune(self, sides: Sequence[int] = SIDES, steps: int = 8) -> Tuple[int, int, int]:
        """Pick the fastest launch shape for a mix of the given sides and apply it.

        Runs on the empty server before any request is admitted: one zero-field,
        source-free simulation per side (same PML and monitor) fills the slots while
        ``steps`` batch steps are timed per candidate, then leaves. Cached per
        (sides, slots) for the process.
        """
        key = (tuple(sides), self.max_slots)
        if key in _SHAPE_CACHE:
            self.set_shape(_SHAPE_CACHE[key])
            return self.shape
        if self.active or self.draining:
            raise RuntimeError("the batch autotuner runs on an empty server")
        if len(sides) > self.max_slots or max(sides) > self.max_side:
            raise ValueError("the autotuning mix does not fit the server")
        jobs = []
        for i, side in enumerate(sides):
            req = Request(index=-1 - i, side=side, eps=4.0, radius_cells=0.3 * side,
                          steps=1 << 40, arrival=0.0)
            driver, flux = build_request(req)
            driver._sources.clear()
            job = _Job(req, driver, flux, footprint_bytes(driver))
            self.admit(job, now=0.0)
            jobs.append(job)
        best, best_ms = None, float("inf")
        for shape in SHAPE_CANDIDATES:
            try:
                self.set_shape(shape)
                self.commit()
            except _lib.MeepGBError:
                continue
            _lib.check(self.lib, self.lib.mgb_batch_step(self.handle, 2, 0, self.stream.cuda_stream))
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record(self.stream)
            _lib.check(self.lib, self.lib.mgb_batch_step(self.handle, steps, 0, self.stream.cuda_stream))
            end.record(self.stream)
            end.synchronize()
            ms = start.elapsed_time(end) / steps
            if ms < best_ms:
                best, best_ms = shape, ms
        for job in jobs:
            _lib.check(self.lib, self.lib.mgb_batch_clear_slot(self.handle, job.slot))
            self.slots[job.slot] = None
            self.resident_bytes -= job.bytes
        self.set_shape(best)
        self.commit()
        self.stream.synchronize()
        for job in jobs:
            job.driver.close()
        _SHAPE_CACHE[key] = best
        self.autotune_ms = best_ms
        return best

    # --- slots --------------------------------------------------------------------------
    @property
    def active(self) -> int:
        """Slots in use (a complex job holds two)."""
        return sum(job is not None for job in self.slots)

    def fits(self, nbytes: int, slots: int = 1) -> bool:
        """Free slots, and room in the HBM budget (slots still draining count)."""
        return (self.active + slots <= self.max_slots
                and (self.resident_bytes == 0 or self.resident_bytes + nbytes <= self.budget_bytes))

    def admit(self, job: _Job, now: float) -> None:
        """Make a job's device state (on the setup stream) and put it in free slots: one,
        or for complex fields two, its real and imaginary parts, each driven by its part
        of the currents (with a Bloch phase the two read each other across the phased
        faces, which a batch step allows: every slot's H half, then every slot's E half);
        the spectrum combines the two parts' transforms."""
        if job.driver.grid.has_symmetry:
            raise Unsupported("a batched slot does not carry mirror symmetry")
        free = [i for i, held in enumerate(self.slots) if held is None]
        if len(free) < job.slots_needed:
            raise RuntimeError("admit() needs free slots: check fits() first")
        with torch.cuda.stream(self.setup_stream):
            # the batch accumulates its monitors step by step (dft_batched)
            job.engine = job.driver.freeze(stream=self.stream, autotune=False, dft_accumulation="direct")
            plans = [job.engine.re, job.engine.im] if job.slots_needed == 2 else [job.engine]
            words = []
            for plan, part in zip(plans, ("real", "imag")):
                if job.driver.sources:
                    host = deposit_words(job.driver.sources, 0, job.request.steps, job.driver.grid.dt,
                                         part=part)
                    words.append(torch.from_numpy(host).to(self.device))
                else:
                    words.append(None)
        job.words = words
        for slot, plan, table in zip(free, plans, words):
            _lib.check(self.lib, self.lib.mgb_batch_set_slot(
                self.handle, slot, plan.handle, job.request.steps,
                table.data_ptr() if table is not None else None))
            self.slots[slot] = job
        job.slots = tuple(free[:len(plans)])
        job.slot = job.slots[0]
        job.admitted = now
        self.resident_bytes += job.bytes

    def commit(self) -> None:
        """Upload the slot changes; the batch stream first waits for the setup uploads."""
        self.stream.wait_stream(self.setup_stream)
        _lib.check(self.lib, self.lib.mgb_batch_commit(self.handle, self.stream.cuda_stream))

    def launch(self, steps: Optional[int] = None) -> None:
        """Queue one replay of ``steps`` batch steps (asynchronous)."""
        steps = self.steps_per_replay if steps is None else int(steps)
        _lib.check(self.lib, self.lib.mgb_batch_step(self.handle, steps, 1 if self.use_graph else 0,
                                                     self.stream.cuda_stream))
        self.replays += 1

    def mark(self) -> torch.cuda.Event:
        """An event at the end of the work queued so far on the batch stream."""
        event = torch.cuda.Event()
        event.record(self.stream)
        return event

    def steps(self) -> np.ndarray:
        """Every slot's step once the queued replays have run (-1 for empty slots)."""
        out = np.empty(self.max_slots, dtype=np.int64)
        _lib.check(self.lib, self.lib.mgb_batch_steps(self.handle, out.ctypes.data_as(_lib.c_int64_p)))
        return out

    def finish(self) -> int:
        """Queue read-outs of the slots the queued replays complete and free those slots."""
        steps = self.steps()
        count = 0
        for slot, job in enumerate(self.slots):
            if job is None or slot != job.slot or any(steps[s] < job.request.steps for s in job.slots):
                continue
            job.readback = job.engine.queue_flux_spectrum(job.flux)
            for held in job.slots:
                _lib.check(self.lib, self.lib.mgb_batch_clear_slot(self.handle, held))
                self.slots[held] = None
            self.draining.append(job)
            count += 1
        return count

    def collect(self, now_fn: Callable[[], float], wait: bool = False) -> List[Result]:
        """Spectra whose read-back has completed (all of them when ``wait``)."""
        results = []
        for job in list(self.draining):
            host, event = job.readback
            if wait:
                event.synchronize()
            elif not event.query():
                continue
            spectrum = host.numpy() * job.flux.measure * job.flux.weight
            results.append(Result(job.request.index, job.request.side, job.request.steps,
                                  spectrum, job.request.arrival, job.admitted, now_fn()))
            self.draining.remove(job)
            self.resident_bytes -= job.bytes
            job.driver.close()
            job.engine = None
            job.words = None
            job.readback = None
        return results

    def close(self) -> None:
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.stream.synchronize()
            self.lib.mgb_batch_destroy(self.handle)
            self.handle = None
        for job in list(self.slots) + list(self.draining):
            if job is not None:
                job.driver.close()
        self.slots = [None] * self.max_slots
        self.draining = []

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass


class _Marks:
    """Events at the end of the work queued on several batch streams."""

    def __init__(self, events):
        self.events = events

    def synchronize(self) -> None:
        for event in self.events:
            event.synchronize()

    def query(self) -> bool:
        return all(event.query() for event in self.events)


class MultiBatchServer:
    """Several batches, each on its own stream and CUDA graph, behind one server's calls.

    The slots of different batches are independent simulations, so nothing orders one
    batch's launches after another's: the GPU fills the tail of one batch's step launch
    with the other batches' work instead of idling SMs at every half. A request goes to
    the batch with the fewest resident cells that has room for it (both slots of a
    complex request to the same batch: with a Bloch phase its parts read each other).
    """

    def __init__(self, device: Optional[torch.device] = None, groups: int = 2, max_slots: int = 32,
                 budget_bytes: Optional[int] = None, steps_per_replay: int = 64, use_graph: bool = True,
                 shape: Optional[Tuple[int, int, int]] = None, max_side: int = max(SIDES),
                 max_monitor_cells: Optional[int] = None):
        groups = max(1, int(groups))
        if budget_bytes is None:
            free, _total = torch.cuda.mem_get_info(device)
            budget_bytes = int(0.5 * free)
        per_slots = max(2, -(-int(max_slots) // groups))
        self.servers = [BatchServer(device, max_slots=per_slots, budget_bytes=int(budget_bytes) // groups,
                                    steps_per_replay=steps_per_replay, use_graph=use_graph, shape=shape,
                                    max_side=max_side, max_monitor_cells=max_monitor_cells)
                        for _ in range(groups)]
        self.max_slots = per_slots * groups
        self.cells: List[int] = [0] * groups
        self.owner: Dict[int, int] = {}

    @property
    def active(self) -> int:
        return sum(server.active for server in self.servers)

    @property
    def draining(self) -> list:
        return [job for server in self.servers for job in server.draining]

    @property
    def replays(self) -> int:
        return sum(server.replays for server in self.servers)

    @property
    def shape(self):
        return self.servers[0].shape

    def autotune(self, sides: Sequence[int] = SIDES, steps: int = 8):
        shape = self.servers[0].autotune(sides, steps)
        for server in self.servers[1:]:
            server.set_shape(shape)
        return shape

    def fits(self, nbytes: int, slots: int = 1) -> bool:
        return any(server.fits(nbytes, slots) for server in self.servers)

    def admit(self, job: _Job, now: float) -> None:
        room = [g for g, server in enumerate(self.servers) if server.fits(job.bytes, job.slots_needed)]
        if not room:
            raise RuntimeError("admit() needs room in some batch: check fits() first")
        g = min(room, key=lambda at: self.cells[at])
        self.servers[g].admit(job, now)
        self.cells[g] += job.request.side ** 3
        self.owner[id(job)] = g

    def commit(self) -> None:
        for server in self.servers:
            if server.active:
                server.commit()

    def launch(self, steps: Optional[int] = None) -> None:
        for server in self.servers:
            if server.active:
                server.launch(steps)

    def mark(self) -> _Marks:
        return _Marks([server.mark() for server in self.servers])

    def finish(self) -> int:
        count = 0
        for g, server in enumerate(self.servers):
            before = set(id(job) for job in server.draining)
            count += server.finish()
            for job in server.draining:
                if id(job) not in before:
                    self.cells[g] -= job.request.side ** 3
        return count

    def collect(self, now_fn: Callable[[], float], wait: bool = False) -> List["Result"]:
        results = []
        for server in self.servers:
            results.extend(server.collect(now_fn, wait=wait))
        return results

    def close(self) -> None:
        for server in self.servers:
            server.close()


@dataclass
class Report:
    """Outcome of serving a stream: per-request results and the stream's throughput."""

    results: List[Result]
    wall_seconds: float
    first_arrival: float
    replays: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def sims_per_second(self) -> float:
        last = max(r.done for r in self.results)
        return len(self.results) / (last - self.first_arrival)

    def latency_percentile(self, q: float) -> float:
        return float(np.percentile([r.latency for r in self.results], q))

    def spectra(self) -> Dict[int, np.ndarray]:
        return {r.index: r.spectrum for r in self.results}


def serve(server: BatchServer, requests: Sequence[Request], realtime: bool = True,
          build: Callable = build_request, depth: int = 2) -> Report:
    """Serve a stream with continuous batching.

    Arrivals are honoured against the wall clock when ``realtime`` (else every request
    is present at time 0). Each turn: admit arrived requests in arrival order while a
    slot and the HBM budget allow (later, smaller requests may fill room the head of the
    queue does not fit), commit, queue one replay and the read-outs of the slots it
    completes, configure waiting requests on the host while the GPU works, and collect
    finished spectra. At most ``depth`` replays are queued ahead of the host.
    """
    order = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0  # noqa: E731
    arrived = 0
    waiting: deque = deque()
    prepared: Dict[int, _Job] = {}
    results: List[Result] = []
    inflight: deque = deque()
    replays0 = server.replays

    def job_for(request: Request) -> _Job:
        job = prepared.pop(request.index, None)
        if job is None:
            driver, flux = build(request)
            job = _Job(request, driver, flux, footprint_bytes(driver))
        return job

    while len(results) < len(order):
        t = now()
        while arrived < len(order) and (not realtime or order[arrived].arrival <= t):
            waiting.append(order[arrived])
            arrived += 1
        for request in list(waiting):
            if server.active >= server.max_slots:
                break
            job = job_for(request)
            if server.fits(job.bytes, job.slots_needed):
                server.admit(job, now())
                waiting.remove(request)
            else:
                prepared[request.index] = job
        if server.active > 0:
            server.commit()
            server.launch()
            inflight.append(server.mark())
            server.finish()
        # configure a few waiting (or about to arrive) requests while the GPU works
        budget = 2
        for request in list(waiting) + order[arrived:arrived + 2]:
            if budget == 0:
                break
            if request.index not in prepared and request.arrival <= now() + 0.05:
                prepared[request.index] = job_for(request)
                budget -= 1
        while len(inflight) > depth or (inflight and server.active == 0 and not waiting):
            inflight.popleft().synchronize()
        # with nothing left to step, wait for the remaining read-backs instead of polling
        results.extend(server.collect(now, wait=server.active == 0 and not waiting))
        if server.active == 0 and not server.draining and arrived < len(order) and not waiting:
            time.sleep(max(0.0, min(order[arrived].arrival - now(), 0.005)))
    return Report(results, now(), order[0].arrival, server.replays - replays0)
def solve_plain(requests: Sequence[Request], realtime: bool = True, build: Callable = build_request,
                kernels=None) -> Report:
    """The same stream solved one request at a time through the plain drop-in driver."""
    order = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0  # noqa: E731
    results = []
    for request in order:
        if realtime:
            wait = request.arrival - now()
            if wait > 0:
                time.sleep(wait)
        driver, flux = build(request, kernels=kernels) if kernels is not None else build(request)
        started = now()
        driver.step_many(request.steps)
        spectrum = flux.get_flux_spectrum()
        results.append(Result(request.index, request.side, request.steps, spectrum, request.arrival,
                              started, now()))
        driver.close()
    return Report(results, now(), order[0].arrival)
