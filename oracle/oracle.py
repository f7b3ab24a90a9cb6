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
                    ("npoles", ctypes.c_int), ("poles", Pole * 4),
                    ("nsrc", ctypes.c_int), ("src_cell", P), ("src_comp", P),
                    ("h_separated", ctypes.c_int)]
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


def problem_from_driver(driver) -> Problem:
    """The oracle's description of a configured ``meep_gpu_gb300.FdtdDriver`` (host data only)."""
    from meep_gpu_gb300.dft import FluxMonitor
    from meep_gpu_gb300.pml import identity_tables
    from meep_gpu_gb300.sources import deposit_words

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
    return Problem(shape=grid.shape, metallic=tuple(int(grid.is_metallic(a)) for a in range(3)),
                   dt=grid.dt, dx=grid.dx, pml=pml is not None, tables32=tables32,
                   tables64=tables64, member=member, inv_eps32=inv32, inv_eps64=inv64,
                   poles=poles, src_cells=np.array(cells, dtype=np.int64),
                   src_comps=np.array(comps, dtype=np.int32),
                   words=lambda first, steps: deposit_words(sources, first, steps, grid.dt),
                   monitors=monitors)


class Oracle:
    """One run of the CPU oracle over a :class:`Problem`, in ``precision`` f32 or f64."""

    def __init__(self, problem: Problem, precision: str = "f32"):
        if precision not in _DTYPE:
            raise ValueError("precision is 'f32' or 'f64'")
        self.problem = problem
        self.precision = precision
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
        self.state = s
        self.step_count = 0
        self.accumulators: List[np.ndarray] = []
        for mon in problem.monitors:
            cells = int(np.prod([mon.region[2 * a + 1] - mon.region[2 * a] for a in range(3)]))
            self.accumulators.append(np.zeros((len(mon.components), mon.omegas.size, 2, cells), dtype=dtype))
        self._step_fn = getattr(self.lib, f"oracle_step_{precision}")
        self._step_fn.argtypes = [P, P]
        self._dft_fn = getattr(self.lib, f"oracle_dft_{precision}")
        self._dft_fn.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_longlong, P]

    def _ptr(self, array: np.ndarray) -> int:
        self._keep.append(array)
        return array.ctypes.data

    def run(self, nsteps: int) -> None:
        nsrc = int(self.problem.src_cells.size)
        words = self.problem.words(self.step_count, nsteps) if nsrc else None
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
