"""Python front end of the CPU oracle (``liboracle.so``). TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline arm use this
module, to check or time the CUDA engine; the product (``meep_gpu_gb300``) never
imports it. The oracle steps full-volume arrays with plain C loops that restate the
reference's array path (``meep_gpu/stepping.py``, ``dispersion.py``, ``sources.py``,
``dft.py``) operation for operation, in float32 (bit-comparable with the reference) or
in float64 (the same equations in double, the error floor every float32 result is
quoted against).

A :class:`Problem` is the full description of one run: it is built from a configured
(not yet stepped) ``meep_gpu_gb300.FdtdDriver`` by :func:`problem_from_driver`, or from
a golden fixture recorded from the reference (``tests/golden``).
"""

from __future__ import annotations

import ctypes
import math
import subprocess
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "liboracle.so"
COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def build() -> Path:
    """Compile ``liboracle.so`` with the committed Makefile (gcc)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIBRARY


_LIB: Optional[ctypes.CDLL] = None


def load() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        sources = [HERE / "fdtd_oracle.c", HERE / "fdtd_oracle_impl.h", HERE / "Makefile"]
        if not LIBRARY.exists() or any(p.stat().st_mtime > LIBRARY.stat().st_mtime for p in sources):
            build()
        _LIB = ctypes.CDLL(str(LIBRARY))
    return _LIB


P = ctypes.c_void_p


def _state_type(real) -> type:
    class Pole(ctypes.Structure):
        _fields_ = [("two_minus_od", real), ("gamma1", real), ("omega0dtsqr", real),
                    ("gamma1inv", real), ("sigma", P * 3), ("p", P * 3), ("pp", P * 3)]

    class State(ctypes.Structure):
        _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                    ("metallic", ctypes.c_int * 3), ("dtdx", real), ("pml", ctypes.c_int),
                    ("kms", (P * 3) * 2), ("sinv", (P * 3) * 2), ("kps", (P * 3) * 2),
                    ("member", (P * 3) * 2),
                    ("E", P * 3), ("D", P * 3), ("B", P * 3), ("H", P * 3),
                    ("fwH", P * 3), ("fwE", P * 3), ("fuB", P * 3), ("fuD", P * 3),
                    ("inv_eps", P * 3), ("scratch", P), ("drive", P * 3),
                    ("npoles", ctypes.c_int), ("poles", Pole * 8),
                    ("nsrc", ctypes.c_int), ("src_cell", P), ("src_comp", P),
                    ("h_separated", ctypes.c_int),
                    ("condfac", (P * 3) * 2), ("condinv", (P * 3) * 2), ("keeps", (P * 3) * 2),
                    ("fcond", (P * 3) * 2), ("fold", ctypes.c_int * 3),
                    ("full", ctypes.c_int * 3), ("bloch", ctypes.c_int), ("bmode", ctypes.c_int * 3),
                    ("bre", real * 3), ("bim", real * 3), ("part", ctypes.c_int),
                    ("pE", P * 3), ("pH", P * 3), ("invariant", ctypes.c_int)]
    return State


_STATE = {"f32": _state_type(ctypes.c_float), "f64": _state_type(ctypes.c_double)}
_DTYPE = {"f32": np.float32, "f64": np.float64}


@dataclass
class MonitorSpec:
    kind: str                      # "flux" or "dft"
    region: Tuple[int, ...]
    components: Tuple[str, ...]
    omegas: np.ndarray
    scale: float
    decimation: int
    weights: Optional[np.ndarray] = None   # flux: float32 per-cell weights
    measure: float = 1.0
    weight: float = 1.0


@dataclass
class Problem:
    shape: Tuple[int, int, int]
    metallic: Tuple[int, int, int]
    dt: float
    dx: float
    pml: bool
    tables32: Dict[Tuple[int, int], Tuple[np.ndarray, np.ndarray, np.ndarray]]
    tables64: Dict[Tuple[int, int], Tuple[np.ndarray, np.ndarray, np.ndarray]]
    member: Dict[Tuple[int, int], np.ndarray]
    inv_eps32: Sequence[np.ndarray]
    inv_eps64: Sequence[np.ndarray]
    poles: List[dict]              # {"c32": (4,), "c64": (4,), "sigma": [vol|None]*3}
    src_cells: np.ndarray          # int64 linear indices
    src_comps: np.ndarray          # int32
    words: Callable[[int, int], np.ndarray]
    monitors: List[MonitorSpec] = field(default_factory=list)
    # float32 sigma volume per lossy D / B component ("Dx" .. "Bz"), and the PML faces in
    # cells ((low, high) per axis) the one-rank chunks are cut by
    conductivity: Dict[str, np.ndarray] = field(default_factory=dict)
    faces: Tuple[Tuple[float, float], ...] = ((0.0, 0.0),) * 3
    # mirror planes: the phase (+1 / -1) of each folded axis, 0 elsewhere, and the
    # unfolded counts
    mirror: Tuple[int, int, int] = (0, 0, 0)
    full: Tuple[int, int, int] = (0, 0, 0)
    # Bloch phases per axis: None, or eikna as (re, im) in float64
    bloch: Tuple[Optional[Tuple[float, float]], ...] = (None, None, None)
    # MEEP's window per axis in cells, and whether each axis wraps (None: the stored
    # counts, and every non-metallic axis)
    owned: Optional[Tuple[int, int, int]] = None
    wraps: Optional[Tuple[bool, bool, bool]] = None
    # bit a: axis a is translationally invariant (a 2-D or 1-D run)
    invariant: int = 0


YEE = {"Dx": (1, 0, 0), "Dy": (0, 1, 0), "Dz": (0, 0, 1),
       "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0)}


def keeps_volume(shape, metallic, faces, iyee, sigma: np.ndarray, owned=None, wraps=None) -> np.ndarray:
    """Per cell of one component lattice: does the one-rank chunk owning it keep a
    conductivity array? (meep_gpu/chunk_map.py ``ChunkLayout.one_rank`` :384,
    ``owner_volume`` :649, ``loop_rows`` :675, ``conductive_chunks`` :720.)

    Per axis the chunk boxes are [0, 2s_lo], [2s_lo, 2n - 2s_hi], [2n - 2s_hi, 2n] in
    doubled offsets (s = int(cells + 1.5) for a face with a layer). A chunk keeps the
    array when any sample of its loop volume (doubled lo + shift .. hi + shift) is
    nonzero; a cell belongs to the chunk whose box holds its doubled coordinate
    (lo < p <= hi), a wall row that no chunk owns taking its nearest owned row's.
    ``owned``: MEEP's window per axis in cells (the stored count but on a folded periodic
    axis, which stores one row past it); ``wraps``: whether the axis wraps (default: not
    metallic).
    """
    owned = tuple(shape) if owned is None else tuple(owned)
    wraps = tuple(not m for m in metallic) if wraps is None else tuple(wraps)
    boxes, coords = [], []
    for axis in range(3):
        n = shape[axis]
        w = owned[axis]
        low, high = faces[axis]
        cut_lo = 2 * min(w, int(low + 1.5)) if low > 0 else 0
        cut_hi = 2 * w - 2 * min(w, int(high + 1.5)) if high > 0 else 2 * w
        edges = [(0, cut_lo), (cut_lo, cut_hi), (cut_hi, 2 * w)]
        boxes.append([e for e in edges if e[0] < e[1]])
        p = 2 * np.arange(n) + iyee[axis]
        if wraps[axis]:
            p = np.where(p <= 0, p + 2 * n, p)
        inside = (p > 0) & (p <= 2 * w)
        owned_at = np.flatnonzero(inside)
        for row in np.flatnonzero(~inside):
            p[row] = p[owned_at[np.argmin(np.abs(owned_at - row))]]
        coords.append(p)
    out = np.zeros(shape, dtype=bool)
    for bx in boxes[0]:
        for by in boxes[1]:
            for bz in boxes[2]:
                rows = []
                for axis, (lo, hi) in enumerate((bx, by, bz)):
                    n = shape[axis]
                    r = np.arange(lo // 2, hi // 2 + 1)
                    rows.append(r % n if wraps[axis] else np.clip(r, 0, n - 1))
                if not np.any(sigma[np.ix_(*rows)] != 0):
                    continue
                sel = [(c > lo) & (c <= hi) for c, (lo, hi) in zip(coords, (bx, by, bz))]
                out |= sel[0][:, None, None] & sel[1][None, :, None] & sel[2][None, None, :]
    return out


def problem_from_driver(driver) -> Problem:
    """The oracle's description of a configured ``meep_gpu_gb300.FdtdDriver`` (host data only)."""
    from meep_gpu_gb300.dft import FluxMonitor
    from meep_gpu_gb300.pml import identity_tables
    from meep_gpu_gb300.sources import deposit_scales, deposit_words

    driver.prepare()
    grid = driver.grid
    pml = driver.pml if (driver.pml is not None and driver.pml.is_active) else None
    tables = pml.tables if pml is not None else identity_tables(grid)
    tables32 = {key: (t.kms, t.sinv, t.kps) for key, t in tables.items()}
    tables64 = {key: (t.kms64, t.sinv64, t.kps64) for key, t in tables.items()}
    member = {}
    for lattice in (0, 1):
        for axis in range(3):
            member[(lattice, axis)] = (pml.membership(lattice, axis) if pml is not None
                                       else np.zeros(grid.shape[axis], dtype=bool))
    inv32 = driver._inv_eps
    eps = driver._eps
    inv64 = [1.0 / e.astype(np.float64) for e in eps]
    poles = []
    for susceptibility, sigmas in driver._poles:
        c32 = susceptibility.realnum_constants(grid.dt)
        c64 = susceptibility.float64_constants(grid.dt)
        poles.append({"c32": tuple(float(v) for v in c32), "c64": tuple(c64), "sigma": sigmas})
    cells, comps = [], []
    for source in driver._sources:
        for (i, j, k) in source.cells:
            cells.append((i * grid.ny + j) * grid.nz + k)
            comps.append(source.comp_index)
    sources = list(driver._sources)
    monitors = []
    for m in list(driver._flux_monitors) + list(driver._dft_monitors):
        flux = isinstance(m, FluxMonitor)
        monitors.append(MonitorSpec(
            kind="flux" if flux else "dft", region=tuple(m.region), components=tuple(m.components),
            omegas=m.omegas, scale=m.scale, decimation=m.decimation_factor,
            weights=m.weights.reshape(-1) if flux else None,
            measure=m.measure if flux else 1.0, weight=m.weight if flux else 1.0))
    conductivity = {name: v for name, v in driver.conductivity_volumes().items() if v is not None}
    # a deposit on a lossy D or B component is scaled by its condinv word (sources.py:1357)
    condinv = {}
    for index, name in enumerate(("Dx", "Dy", "Dz", "Bx", "By", "Bz")):
        sigma = conductivity.get(name)
        if sigma is not None:
            condinv[index] = (1.0 / (1.0 + (sigma.astype(np.float64) * grid.dt) * 0.5)).astype(np.float32)
    scales = deposit_scales(sources, condinv)
    return Problem(shape=grid.shape, metallic=tuple(int(grid.is_metallic(a)) for a in range(3)),
                   dt=grid.dt, dx=grid.dx, pml=pml is not None, tables32=tables32,
                   tables64=tables64, member=member, inv_eps32=inv32, inv_eps64=inv64,
                   poles=poles, src_cells=np.array(cells, dtype=np.int64),
                   src_comps=np.array(comps, dtype=np.int32),
                   words=lambda first, steps, part="real": deposit_words(sources, first, steps, grid.dt,
                                                                           scales, part),
                   monitors=monitors, conductivity=conductivity,
                   faces=tuple(pml.faces) if pml is not None else ((0.0, 0.0),) * 3,
                   mirror=tuple(grid.mirror_phase(a) or 0 for a in range(3)),
                   full=tuple(grid.shape_full),
                   bloch=tuple(None if grid.bloch_phase(a) is None else grid.eikna(a) for a in range(3)),
                   owned=tuple(grid.owned_cells(a) for a in range(3)),
                   wraps=tuple(grid.axis_wraps(a) for a in range(3)),
                   invariant=sum(1 << a for a in range(3) if getattr(grid, "is_invariant", lambda _: False)(a)))


class Oracle:
    """One run of the CPU oracle over a :class:`Problem`, in ``precision`` f32 or f64.

    ``part="imag"`` runs a complex run's imaginary fields (driven by imag(A)): at k = 0
    the two parts of a complex run step independently, so a complex run is two real runs.
    """

    def __init__(self, problem: Problem, precision: str = "f32", part: str = "real"):
        if precision not in _DTYPE:
            raise ValueError("precision is 'f32' or 'f64'")
        self.problem = problem
        self.precision = precision
        self.part = part
        self.lib = load()
        dtype = _DTYPE[precision]
        self.dtype = dtype
        shape = tuple(problem.shape)
        self._keep: List[np.ndarray] = []
        z = lambda: np.zeros(shape, dtype=dtype)  # noqa: E731
        self.fields: Dict[str, np.ndarray] = {}
        for fam in ("E", "D", "B", "H", "fwH", "fwE", "fuB", "fuD", "drive"):
            for axis in "xyz":
                self.fields[fam + axis] = z()
        if not problem.pml:
            for axis in "xyz":
                self.fields["H" + axis] = self.fields["B" + axis]
        self.scratch = z()
        s = _STATE[precision]()
        s.nx, s.ny, s.nz = shape
        s.metallic[:] = list(problem.metallic)
        s.fold[:] = list(problem.mirror)
        s.invariant = int(problem.invariant)
        s.full[:] = list(problem.full) if any(problem.mirror) else list(shape)
        s.part = 1 if part == "imag" else 0
        s.bloch = 1 if any(b is not None for b in problem.bloch) else 0
        for a, phase in enumerate(problem.bloch):
            if phase is None:
                continue
            re_, im_ = phase
            # the library's connection rule: a copy within 1e-13 of +1, a negation of -1
            if abs(im_) < 1e-13 and abs(re_ - 1.0) < 1e-13:
                s.bmode[a] = 1
            elif abs(im_) < 1e-13 and abs(re_ + 1.0) < 1e-13:
                s.bmode[a] = 2
            else:
                s.bmode[a] = 3
                s.bre[a] = float(np.float32(re_)) if precision == "f32" else re_
                s.bim[a] = float(np.float32(im_)) if precision == "f32" else im_
        s.dtdx = float(np.float32(problem.dt / problem.dx)) if precision == "f32" else problem.dt / problem.dx
        s.pml = 1 if problem.pml else 0
        tables = problem.tables32 if precision == "f32" else problem.tables64
        for (lattice, axis), (kms, sinv, kps) in tables.items():
            for name, arr in (("kms", kms), ("sinv", sinv), ("kps", kps)):
                getattr(s, name)[lattice][axis] = self._ptr(np.ascontiguousarray(arr, dtype=dtype))
            s.member[lattice][axis] = self._ptr(np.ascontiguousarray(problem.member[(lattice, axis)], dtype=np.uint8))
        for q, axis in enumerate("xyz"):
            for fam in ("E", "D", "B", "H", "fwH", "fwE", "fuB", "fuD", "drive"):
                getattr(s, fam)[q] = self.fields[fam + axis].ctypes.data
        inv = problem.inv_eps32 if precision == "f32" else problem.inv_eps64
        for q in range(3):
            s.inv_eps[q] = self._ptr(np.ascontiguousarray(inv[q], dtype=dtype))
        s.scratch = self.scratch.ctypes.data
        s.npoles = len(problem.poles)
        self.polarization: List[Dict[int, Tuple[np.ndarray, np.ndarray]]] = []
        for m, pole in enumerate(problem.poles):
            const = pole["c32"] if precision == "f32" else pole["c64"]
            entry = s.poles[m]
            entry.two_minus_od, entry.gamma1, entry.omega0dtsqr, entry.gamma1inv = const
            kept = {}
            for q in range(3):
                sigma = pole["sigma"][q]
                if sigma is None:
                    entry.sigma[q] = None
                    continue
                entry.sigma[q] = self._ptr(np.ascontiguousarray(sigma, dtype=dtype))
                p, pp = z(), z()
                kept[q] = (p, pp)
                entry.p[q] = p.ctypes.data
                entry.pp[q] = pp.ctypes.data
            self.polarization.append(kept)
        s.nsrc = int(problem.src_cells.size)
        s.src_cell = self._ptr(np.ascontiguousarray(problem.src_cells, dtype=np.int64))
        s.src_comp = self._ptr(np.ascontiguousarray(problem.src_comps, dtype=np.int32))
        s.h_separated = 0
        self.fcond: Dict[str, np.ndarray] = {}
        for name, sigma in problem.conductivity.items():
            side = 0 if name[0] == "B" else 1
            q = "xyz".index(name[1])
            if precision == "f32":
                values = np.ascontiguousarray(sigma, dtype=np.float32)
                dt2 = np.float32(np.float32(problem.dt) * np.float32(0.5))
                fac = (np.float32(1.0) - values * dt2).astype(np.float32)
                inv = (1.0 / (1.0 + (values.astype(np.float64) * problem.dt) * 0.5)).astype(np.float32)
            else:
                wide = np.asarray(sigma, dtype=np.float64)
                fac = 1.0 - wide * (problem.dt / 2.0)
                inv = 1.0 / (1.0 + wide * (problem.dt / 2.0))
            s.condfac[side][q] = self._ptr(np.ascontiguousarray(fac, dtype=dtype))
            s.condinv[side][q] = self._ptr(np.ascontiguousarray(inv, dtype=dtype))
            if problem.pml:
                keeps = keeps_volume(shape, problem.metallic, problem.faces, YEE[name], sigma,
                                     problem.owned, problem.wraps)
                s.keeps[side][q] = self._ptr(np.ascontiguousarray(keeps, dtype=np.uint8))
                self.fcond[name] = z()
                s.fcond[side][q] = self.fcond[name].ctypes.data
        self.state = s
        self.step_count = 0
        self.accumulators: List[np.ndarray] = []
        for mon in problem.monitors:
            cells = int(np.prod([mon.region[2 * a + 1] - mon.region[2 * a] for a in range(3)]))
            self.accumulators.append(np.zeros((len(mon.components), mon.omegas.size, 2, cells), dtype=dtype))
        self._step_fn = getattr(self.lib, f"oracle_step_{precision}")
        self._step_fn.argtypes = [P, P]
        self._half_fn = getattr(self.lib, f"oracle_half_{precision}")
        self._half_fn.argtypes = [P, P, ctypes.c_int]
        self._dft_fn = getattr(self.lib, f"oracle_dft_{precision}")
        self._dft_fn.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_longlong, P]

    def _ptr(self, array: np.ndarray) -> int:
        self._keep.append(array)
        return array.ctypes.data

    def run(self, nsteps: int) -> None:
        if self.state.bloch:
            raise RuntimeError("a Bloch-phased run steps its two parts together: use BlochPair")
        nsrc = int(self.problem.src_cells.size)
        words = self.problem.words(self.step_count, nsteps, self.part) if nsrc else None
        empty = np.zeros(1)
        for t in range(nsteps):
            row = np.ascontiguousarray(words[t]) if nsrc else empty
            self._step_fn(ctypes.addressof(self.state), row.ctypes.data)
            self.step_count += 1
            for mon, acc in zip(self.problem.monitors, self.accumulators):
                if self.step_count % mon.decimation:
                    continue
                region = (ctypes.c_int * 6)(*mon.region)
                comps = np.array([COMPONENTS.index(c) for c in mon.components], dtype=np.int32)
                omegas = np.ascontiguousarray(mon.omegas, dtype=np.float64)
                self._dft_fn(ctypes.addressof(self.state), ctypes.addressof(region), len(comps),
                             comps.ctypes.data, omegas.size, omegas.ctypes.data, mon.scale,
                             self.problem.dt, self.step_count, acc.ctypes.data)

    def accumulate(self) -> None:
        """The monitors' accumulation after a completed step (step_count already advanced)."""
        for mon, acc in zip(self.problem.monitors, self.accumulators):
            if self.step_count % mon.decimation:
                continue
            region = (ctypes.c_int * 6)(*mon.region)
            comps = np.array([COMPONENTS.index(c) for c in mon.components], dtype=np.int32)
            omegas = np.ascontiguousarray(mon.omegas, dtype=np.float64)
            self._dft_fn(ctypes.addressof(self.state), ctypes.addressof(region), len(comps),
                         comps.ctypes.data, omegas.size, omegas.ctypes.data, mon.scale,
                         self.problem.dt, self.step_count, acc.ctypes.data)

    def field(self, name: str) -> np.ndarray:
        return self.fields[name]

    def polarization_array(self, pole: int, q: int) -> np.ndarray:
        return self.polarization[pole][q][0]

    def flux_spectrum(self, index: int) -> np.ndarray:
        """``sum w * Re(Ea conj(Hb) - Eb conj(Ha)) * dA * weight`` in float64."""
        mon = self.problem.monitors[index]
        acc = self.accumulators[index].astype(np.float64)
        ea = acc[0, :, 0] + 1j * acc[0, :, 1]
        eb = acc[1, :, 0] + 1j * acc[1, :, 1]
        ha = acc[2, :, 0] + 1j * acc[2, :, 1]
        hb = acc[3, :, 0] + 1j * acc[3, :, 1]
        w = mon.weights.astype(np.float64)
        s = np.real(ea * np.conj(hb) - eb * np.conj(ha)) @ w
        return s * mon.measure * mon.weight

    def dft(self, index: int, component: str) -> np.ndarray:
        mon = self.problem.monitors[index]
        acc = self.accumulators[index][mon.components.index(component)]
        return acc[:, 0] + 1j * acc[:, 1]


def complex_accumulator(real: "Oracle", imag: "Oracle", index: int) -> np.ndarray:
    """A complex run's transform ``acc_re + i * acc_im`` from its two parts' oracles:
    complex ``[ncomp][nf][cells]``."""
    parts = []
    for oracle in (real, imag):
        acc = oracle.accumulators[index].astype(np.float64)
        parts.append(acc[:, :, 0] + 1j * acc[:, :, 1])
    return parts[0] + 1j * parts[1]


def complex_flux_spectrum(real: "Oracle", imag: "Oracle", index: int) -> np.ndarray:
    """``sum w * Re(Ea conj(Hb) - Eb conj(Ha)) * dA * weight`` of a complex run."""
    mon = real.problem.monitors[index]
    total = complex_accumulator(real, imag, index)
    ea, eb, ha, hb = total[0], total[1], total[2], total[3]
    w = mon.weights.astype(np.float64)
    return (np.real(ea * np.conj(hb) - eb * np.conj(ha)) @ w) * mon.measure * mon.weight


class BlochPair:
    """A Bloch-phased complex run on the oracle: the real and imaginary parts, each
    reading the other's E and H across the phased faces, stepped half by half (H of both,
    then E of both) as the reference's complex run steps (reference ``stepping.py:2544``,
    ``part_products.py:186``)."""

    def __init__(self, problem: Problem, precision: str = "f32"):
        self.re = Oracle(problem, precision, "real")
        self.im = Oracle(problem, precision, "imag")
        for own, other in ((self.re, self.im), (self.im, self.re)):
            for q, axis in enumerate("xyz"):
                own.state.pE[q] = other.fields["E" + axis].ctypes.data
                own.state.pH[q] = other.fields["H" + axis].ctypes.data
        self.problem = problem
        self.step_count = 0

    def run(self, nsteps: int) -> None:
        nsrc = int(self.problem.src_cells.size)
        words = {part: (self.problem.words(self.step_count, nsteps, part) if nsrc else None)
                 for part in ("real", "imag")}
        empty = np.zeros(1)
        for t in range(nsteps):
            rows = {part: (np.ascontiguousarray(words[part][t]) if nsrc else empty) for part in words}
            for half in (0, 1):
                for oracle, part in ((self.re, "real"), (self.im, "imag")):
                    oracle._half_fn(ctypes.addressof(oracle.state), rows[part].ctypes.data, half)
            self.step_count += 1
            for oracle in (self.re, self.im):
                oracle.step_count += 1
                oracle.accumulate()

    def field(self, name: str) -> np.ndarray:
        return self.re.field(name) + 1j * self.im.field(name)
