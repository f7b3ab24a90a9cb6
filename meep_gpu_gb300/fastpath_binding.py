"""The reference-side binding: the reference driver's fast-path seam served by this engine.

The reference's ``FdtdDriver.step`` consults a plan at each sub-step slot —
``plan.dispatch(slot, fields) -> bool`` for the slots of ``DRIVER_SLOTS``
(``meep_gpu/fastpath.py:575``; consults ``driver.py:3533-3584``), True meaning "the whole
sub-step ran", False "nothing ran, the array call follows" (``fastpath.py:4631``) — and
builds that plan once per configuration freeze with ``plan_fast_path(fields, pml, grid,
sources, chunk_layout)`` (``fastpath.py:6986``; call ``driver.py:3509``). This module
provides the same two names over ``libmeepgb``:

* :func:`build_desc` reads the reference's own objects (its ``Grid``, ``PML``,
  ``ChunkLayout``, ``Fields`` and bound sources) by their attribute names into the
  tables the library's descriptor carries (:class:`DescTables`): dimensions, boundary
  kinds, ``dt/dx``, the 18 PML vectors, the one-rank membership runs, the inverse
  permittivity words, the poles' realnum constants and sigma volumes, and every
  source's ``src_vol`` deposit entries. :func:`host_tables` forms the same tables from
  a ``meep_gpu_gb300.FdtdDriver``'s host configuration (what its engine uploads), so
  the two can be compared entry for entry.
* :func:`plan_fast_path` maps the reference's configuration onto an engine and returns a
  :class:`GB300Plan`. Its ``dispatch("step_B", fields)`` runs one whole step on the GPU
  (both halves, the sources, the wall passes, the poles); every other slot answers True.
  With ``mirror=True`` (the default) the plan writes the stepped words back into the
  reference's ``Fields`` arrays at the slots that close each family — B and H at
  ``update_H``, D and E at ``update_E``, P at ``update_P`` — so whatever the reference's
  driver does between the consults (its source deposits and wall passes on its own
  arrays, its monitors after the step) reads the engine's words, and its arrays equal
  the engine's at every step boundary. ``claims_sources`` / ``claims_monitors`` say the
  engine already deposits the sources and can accumulate the monitors: a driver that
  honours them skips its own passes and the write-back (``mirror=False``).

Nothing here imports the reference. Arrays on a CuPy device are read through
``.get()``; host NumPy arrays directly.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

from .conductivity import CONDUCTIVITY_COMPONENTS
from .dispersion import Susceptibility
from .grid import AXIS_NAMES, Mirror, Unsupported

DRIVER_SLOTS: Tuple[str, ...] = ("step_B", "fill_B", "update_H", "step_D", "fill_D", "update_E", "update_P")
FAR_FILL_PASSES: Tuple[str, ...] = ("fill_folded_far_ghosts_B", "fill_folded_far_ghosts_D")
E_NAMES = ("Ex", "Ey", "Ez")


def _host(array) -> Optional[np.ndarray]:
    if array is None:
        return None
    if hasattr(array, "get") and not isinstance(array, np.ndarray):
        array = array.get()
    return np.asarray(array)


def _runs(line: np.ndarray) -> Tuple[int, int, int, int]:
    """The [a0, a1) U [b0, b1) record of a membership line (empty runs are [0, 0))."""
    line = np.asarray(line, dtype=bool)
    edges = np.flatnonzero(np.diff(np.concatenate([[0], line.astype(np.int8), [0]])))
    pairs = list(zip(edges[0::2], edges[1::2]))
    if len(pairs) > 2:
        raise Unsupported(f"a membership line with {len(pairs)} runs (the record holds two)")
    words = [0, 0, 0, 0]
    for slot, (start, stop) in enumerate(pairs):
        words[2 * slot], words[2 * slot + 1] = int(start), int(stop)
    return tuple(words)  # type: ignore[return-value]


def canonical_runs(words) -> Tuple[int, int, int, int]:
    """A membership record with its empty runs written [0, 0) and the others in order."""
    pairs = sorted((int(a), int(b)) for a, b in (tuple(words[0:2]), tuple(words[2:4])) if b > a)
    pairs += [(0, 0)] * (2 - len(pairs))
    return (pairs[0][0], pairs[0][1], pairs[1][0], pairs[1][1])


@dataclass
class DescTables:
    """What the library's descriptor (``mgb_sim_desc``) carries for one configuration."""

    shape: Tuple[int, int, int]
    metallic: Tuple[bool, bool, bool]
    dtdx: np.float32
    pml_active: bool
    # (lattice 0 integer / 1 half-integer, axis) -> (kms, sinv, kps), 1-D float32
    pml: Dict[Tuple[int, int], Tuple[np.ndarray, np.ndarray, np.ndarray]] = field(default_factory=dict)
    # (lattice, axis) -> (a0, a1, b0, b1)
    runs: Dict[Tuple[int, int], Tuple[int, int, int, int]] = field(default_factory=dict)
    inv_eps: Tuple[np.ndarray, ...] = ()
    # per pole: ((two_minus_od, gamma1, omega0dtsqr, gamma1inv) float32, {component: sigma or None})
    poles: List[Tuple[Tuple[np.float32, ...], Dict[str, Optional[np.ndarray]]]] = field(default_factory=list)
    # per source, deposit order: (component, linear cells int64, amplitudes complex128)
    sources: List[Tuple[str, np.ndarray, np.ndarray]] = field(default_factory=list)

    def compare(self, other: "DescTables") -> List[str]:
        """Every entry where the two tables differ (empty: identical words)."""
        diffs: List[str] = []
        for name in ("shape", "metallic", "pml_active"):
            if getattr(self, name) != getattr(other, name):
                diffs.append(f"{name}: {getattr(self, name)} != {getattr(other, name)}")
        if np.float32(self.dtdx) != np.float32(other.dtdx):
            diffs.append(f"dtdx: {self.dtdx!r} != {other.dtdx!r}")
        if self.pml_active:
            for key, vectors in self.pml.items():
                for label, a, b in zip(("kms", "sinv", "kps"), vectors, other.pml.get(key, (None,) * 3)):
                    if b is None or not np.array_equal(a, b):
                        diffs.append(f"pml {label} {key}")
            for key, runs in self.runs.items():
                if other.runs.get(key) != runs:
                    diffs.append(f"runs {key}: {runs} != {other.runs.get(key)}")
        for q, (a, b) in enumerate(zip(self.inv_eps, other.inv_eps)):
            if not np.array_equal(a, b):
                diffs.append(f"inv_eps {E_NAMES[q]}: {int(np.sum(a != b))} words")
        if len(self.poles) != len(other.poles):
            diffs.append(f"{len(self.poles)} poles != {len(other.poles)}")
        for m, ((ca, sa), (cb, sb)) in enumerate(zip(self.poles, other.poles)):
            if tuple(np.float32(v) for v in ca) != tuple(np.float32(v) for v in cb):
                diffs.append(f"pole {m} constants {ca} != {cb}")
            for c in E_NAMES:
                x, y = sa.get(c), sb.get(c)
                if (x is None) != (y is None) or (x is not None and not np.array_equal(x, y)):
                    diffs.append(f"pole {m} sigma {c}")
        if len(self.sources) != len(other.sources):
            diffs.append(f"{len(self.sources)} sources != {len(other.sources)}")
        for s, ((ca, xa, aa), (cb, xb, ab)) in enumerate(zip(self.sources, other.sources)):
            if ca != cb or not np.array_equal(xa, xb) or not np.array_equal(aa, ab):
                diffs.append(f"source {s} ({ca}/{cb}) deposit entries")
        return diffs


# --- the reference's objects -> tables ---------------------------------------------------
def _reference_runs(grid, chunk_layout) -> Dict[Tuple[int, int], Tuple[int, int, int, int]]:
    runs = {}
    for axis in range(3):
        for lattice in (0, 1):
            line = chunk_layout.membership(axis, bool(lattice)) if chunk_layout is not None else None
            if line is None:
                raise Unsupported(f"the chunk division is not separable along {AXIS_NAMES[axis]}")
            runs[(lattice, axis)] = canonical_runs(_runs(_host(line)))
    return runs


def build_desc(fields, pml, grid, sources, chunk_layout=None) -> DescTables:
    """The descriptor tables of the reference's frozen configuration, read from its own
    ``Fields`` / ``PML`` / ``Grid`` / sources / ``ChunkLayout`` (reference ``fields.py:390``,
    ``pml.py:324``, ``grid.py``, ``sources.py:1585`` ``bind_src_vols``, ``chunk_map.py:897``)."""
    shape = tuple(int(n) for n in grid.shape)
    pml_active = pml is not None and bool(getattr(pml, "is_active", True))
    tables = DescTables(shape=shape, metallic=tuple(bool(grid.is_metallic(a)) for a in range(3)),
                        dtdx=np.float32(grid.dt / grid.dx), pml_active=pml_active)
    if pml_active:
        for axis, name in enumerate(AXIS_NAMES):
            for lattice, suffix in ((0, ""), (1, "_h")):
                tables.pml[(lattice, axis)] = tuple(
                    np.ascontiguousarray(_host(getattr(pml, f"{v}_{name}{suffix}")), dtype=np.float32).reshape(-1)
                    for v in ("kms", "sinv", "kps"))
        layout = chunk_layout if chunk_layout is not None else getattr(fields, "chunk_layout", None)
        tables.runs = _reference_runs(grid, layout)
    tables.inv_eps = tuple(np.ascontiguousarray(_host(fields.inverse_epsilon_for(c)), dtype=np.float32)
                           for c in E_NAMES)
    for state in getattr(fields, "polarizations", None) or ():
        k = state.constants
        constants = (k.two_minus_od, k.gamma1, k.omega0dtsqr, k.gamma1inv)
        sigma = {c: (None if state.sigma.get(c) is None else np.asarray(_host(state.sigma[c]), dtype=np.float32))
                 for c in E_NAMES}
        tables.poles.append((constants, sigma))
    ny, nz = shape[1], shape[2]
    for source in sources or ():
        cells, amps = [], []
        for entry in source._src_vol:
            ix, iy, iz = (np.asarray(_host(a), dtype=np.int64).reshape(-1) for a in (entry.ix, entry.iy, entry.iz))
            cells.append((ix * ny + iy) * nz + iz)
            amps.append(np.asarray(_host(entry.amps), dtype=np.complex128).reshape(-1))
        tables.sources.append((str(source.component), np.concatenate(cells) if cells else np.zeros(0, np.int64),
                               np.concatenate(amps) if amps else np.zeros(0, np.complex128)))
    return tables


def host_tables(driver) -> DescTables:
    """The same tables as this engine's host code forms them for ``driver`` (a
    ``meep_gpu_gb300.FdtdDriver``; resolved with ``prepare()`` first): what its engine uploads."""
    driver.prepare()
    grid = driver.grid
    pml = driver.pml
    pml_active = pml is not None and pml.is_active
    tables = DescTables(shape=tuple(grid.shape), metallic=tuple(bool(grid.is_metallic(a)) for a in range(3)),
                        dtdx=np.float32(grid.dt / grid.dx), pml_active=pml_active)
    if pml_active:
        for key, axis_tables in pml.tables.items():
            tables.pml[key] = tuple(np.ascontiguousarray(v, dtype=np.float32).reshape(-1)
                                    for v in (axis_tables.kms, axis_tables.sinv, axis_tables.kps))
        tables.runs = {key: canonical_runs(runs) for key, runs in pml.records.items()}
    tables.inv_eps = tuple(np.ascontiguousarray(v, dtype=np.float32) for v in driver._inv_eps)
    for susceptibility, volumes in driver._poles:
        k = susceptibility.realnum_constants(grid.dt)
        constants = (k.two_minus_od, k.gamma1, k.omega0dtsqr, k.gamma1inv)
        tables.poles.append((constants, {c: (None if v is None else np.asarray(v, dtype=np.float32))
                                         for c, v in zip(E_NAMES, volumes)}))
    ny, nz = grid.shape[1], grid.shape[2]
    for source in driver.sources:
        cells = np.asarray(source.cells, dtype=np.int64).reshape(-1, 3)
        tables.sources.append((source.component, (cells[:, 0] * ny + cells[:, 1]) * nz + cells[:, 2],
                               np.asarray(source.amps, dtype=np.complex128).reshape(-1)))
    return tables


# --- the reference's configuration -> this engine's driver ----------------------------------
def _boundaries(grid) -> Tuple[str, str, str]:
    kinds = []
    for axis, pair in enumerate(grid.boundaries):
        low, high = (pair, pair) if isinstance(pair, str) else tuple(pair)
        if low != high:
            raise Unsupported(f"different boundary kinds on the two {AXIS_NAMES[axis]} faces")
        kinds.append(str(low))
    return tuple(kinds)  # type: ignore[return-value]


def _mirrors(grid) -> Tuple[Mirror, ...]:
    out = []
    for symmetry in getattr(grid, "symmetry", None) or ():
        axis = getattr(symmetry, "axis", None)
        name = axis if isinstance(axis, str) else AXIS_NAMES[int(axis)]
        out.append(Mirror(name.upper(), int(getattr(symmetry, "phase", 1))))
    return tuple(out)


def _source_spec(source) -> Dict[str, Any]:
    """The add_source mapping of one reference source: a ``GaussianPulsedSource`` or
    ``ContinuousSource`` (electric), or a ``VolumeSource`` (any family) whose envelope is a
    ``GaussianEnvelope`` or ``ContinuousEnvelope`` (reference ``sources.py:2427``, :1849, :1892)."""
    kind = type(source).__name__
    waveform = source
    if kind == "VolumeSource":
        waveform = source.envelope
        kind = {"GaussianEnvelope": "GaussianPulsedSource",
                "ContinuousEnvelope": "ContinuousSource"}.get(type(waveform).__name__, type(waveform).__name__)
    spec: Dict[str, Any] = {"component": str(source.component), "center": tuple(source.center),
                            "size": tuple(source.size), "amplitude": complex(source.amplitude)}
    if getattr(source, "amp_func", None) is not None:
        spec["amp_func"] = source.amp_func
    if getattr(source, "is_integrated", False) or getattr(waveform, "is_integrated", False):
        raise Unsupported("integrated sources are not stepped by this engine")
    if kind == "GaussianPulsedSource":
        spec.update(source_type="gaussian", frequency=float(waveform.frequency), fwidth=float(waveform.fwidth),
                    start_time=float(waveform.start_time), cutoff=float(waveform.cutoff))
    elif kind == "ContinuousSource":
        spec.update(source_type="continuous", frequency=float(waveform.frequency),
                    start_time=float(waveform.start_time), end_time=float(waveform.end_time),
                    width=float(waveform.width), slowness=float(waveform.slowness))
    else:
        raise Unsupported(f"a {kind} is not stepped by this engine")
    if spec["amplitude"].imag == 0.0:
        spec["amplitude"] = spec["amplitude"].real
    return spec


def driver_for(fields, pml, grid, sources, gpu_id: int = 0):
    """A ``meep_gpu_gb300.FdtdDriver`` configured as the reference's frozen run (not frozen)."""
    from .driver import FdtdDriver

    if getattr(fields, "has_nonlinearity", False) or getattr(fields, "has_offdiagonal_epsilon", False):
        raise Unsupported("nonlinear or off-diagonal-epsilon runs are not stepped by this engine")
    if getattr(grid, "cylindrical", False):
        raise Unsupported("cylindrical runs are not stepped by this engine")
    driver = FdtdDriver(tuple(grid.cell_size), grid.resolution, courant=grid.courant,
                        force_complex_fields=bool(fields.force_complex_fields), symmetry=_mirrors(grid),
                        k_point=tuple(grid.k_point), boundaries=_boundaries(grid), gpu_id=gpu_id,
                        dimensions=int(getattr(grid, "dimensions", 3)))
    driver.set_epsilon_components(*(np.asarray(_host(fields.epsilon_for(c)), dtype=np.float32) for c in E_NAMES))
    if pml is not None and getattr(pml, "is_active", True):
        driver.setup_pml(tuple(tuple(pair) for pair in pml.thickness_by_face), order=int(pml.order))
    for state in getattr(fields, "polarizations", None) or ():
        s = state.susceptibility
        driver.add_susceptibility(Susceptibility(frequency=float(s.frequency), gamma=float(s.gamma), kind=s.kind),
                                  {c: (None if state.sigma.get(c) is None else np.asarray(_host(state.sigma[c])))
                                   for c in E_NAMES})
    if getattr(fields, "has_conductivity", False) or getattr(fields, "has_magnetic_conductivity", False):
        volumes = {c: _host(fields.conductivity_for(c)) for c in CONDUCTIVITY_COMPONENTS}
        driver.set_conductivity({c: volumes[c] for c in ("Dx", "Dy", "Dz")}, absorber_included=True)
        driver.set_b_conductivity({c: volumes[c] for c in ("Bx", "By", "Bz")})
    for source in sources or ():
        driver.add_source(_source_spec(source))
    absent = tuple(getattr(fields, "absent_components", ()) or ())
    if absent:
        driver.set_absent_components(absent)
    return driver


class GB300Plan:
    """One frozen configuration's dispatch set on this engine (the reference's
    ``FastPathPlan``, ``fastpath.py:4512``): every slot is claimed, and the whole step
    runs when ``step_B`` is consulted."""

    table = "gb300"
    slots = DRIVER_SLOTS
    claims_sources = True
    claims_monitors = False

    def __init__(self, fields, driver, first_step: int = 0, mirror: bool = True):
        self.fields = fields
        self.driver = driver
        self.mirror = bool(mirror)
        self.launches: Dict[str, int] = {slot: 0 for slot in DRIVER_SLOTS}
        driver.step_count = int(first_step)
        self._upload()

    def _stored(self):
        for family in ("E", "D", "H", "B"):
            for axis in "xyz":
                yield family + axis, getattr(self.fields, family + axis, None)

    def _upload(self) -> None:
        """Start the engine from the words the reference's arrays hold (zero at a freeze
        before the first step; a plan rebuilt mid-run continues from them)."""
        import torch

        engine = self.driver.freeze(autotune=True)
        loaded = False
        for name, array in self._stored():
            host = _host(array)
            if host is None or not np.any(host):
                continue
            loaded = True
            if engine is not None and hasattr(engine, "fields") and name[0] in "EDH":
                engine.fields[name].copy_(torch.from_numpy(np.ascontiguousarray(host, dtype=np.float32)))
        if loaded and self.driver.pml is not None:
            raise Unsupported("a plan rebuilt mid-run under a PML (its auxiliaries are not carried over)")

    def dispatches_a_kernel(self) -> bool:
        return True

    def dispatch(self, slot: str, fields) -> bool:
        """Run ``slot`` (the whole step at ``step_B``) or answer False for the array path."""
        if fields is not self.fields:
            return False
        if slot not in DRIVER_SLOTS and slot not in FAR_FILL_PASSES:
            return False
        if slot == "step_B":
            self.driver.step_many(1)
        if slot in self.launches:
            self.launches[slot] += 1
        if self.mirror:
            if slot == "update_H":
                self._write_back("BH")
            elif slot == "update_E":
                self._write_back("DE")
            elif slot == "update_P":
                self._write_back_polarization()
        return True

    def _write_back(self, families: str) -> None:
        for family in families:
            for axis in "xyz":
                target = getattr(self.fields, family + axis, None)
                if target is None:
                    continue
                words = self.driver.get_field(family + axis, cell_centered=False)
                if hasattr(target, "set") and not isinstance(target, np.ndarray):
                    target.set(words)
                else:
                    target[...] = words

    def _write_back_polarization(self) -> None:
        engine = self.driver.engine
        states = getattr(self.fields, "polarizations", None) or ()
        if not states or not hasattr(engine, "pole_tensors"):
            return
        box = engine.pbox
        current = self.driver.step_count % 2
        for m, state in enumerate(states):
            for q, name in enumerate(E_NAMES):
                if q not in engine.pole_tensors[m] or state.P.get(name) is None:
                    continue
                _, p0, p1 = engine.pole_tensors[m][q]
                now, before = (p0, p1) if current == 0 else (p1, p0)
                for target, words in ((state.P[name], now), (state.P_prev[name], before)):
                    full = np.zeros(target.shape, dtype=np.float32)
                    full[box[0]:box[1], box[2]:box[3], box[4]:box[5]] = words.cpu().numpy()
                    target[...] = full

    def report(self) -> Dict[str, Any]:
        return {"table": self.table, "slots": list(self.slots), "launches": dict(self.launches),
                "mirror": self.mirror, "claims_sources": self.claims_sources}

    def close(self) -> None:
        self.driver.close()


def plan_fast_path(fields, pml, grid, sources=None, chunk_layout=None, *, first_step: int = 0,
                   mirror: bool = True, gpu_id: int = 0) -> Optional[GB300Plan]:
    """The reference's ``plan_fast_path`` (``fastpath.py:6986``) on this engine: a
    :class:`GB300Plan`, or None (the array path) when the configuration is one this
    engine refuses. ``first_step`` is the driver's step count at the freeze."""
    try:
        driver = driver_for(fields, pml, grid, sources, gpu_id=gpu_id)
    except Unsupported:
        return None
    try:
        return GB300Plan(fields, driver, first_step=first_step, mirror=mirror)
    except Unsupported:
        driver.close()
        return None
