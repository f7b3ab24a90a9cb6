"""UPML coefficient tables and the one-rank PML membership the kernels select forms by.

Coefficients follow the reference's ``meep_gpu/pml.py`` (``PML._compute_coefficients``
:720, ``_compute_sigma_profile`` :631, ``_graded_sigma`` :469, ``prefac`` :436,
``half_cell_extent`` :132), which restate MEEP's ``structure_chunk::use_pml``:
quadratic grading, kappa = 1, R = 1e-15, ``sigma * dt / 2`` baked in, and per axis and
Yee lattice (integer / half-integer) the three float32 vectors

    kms = kappa - sigma,  sinv = 1 / (kappa + sigma),  kps = kappa + sigma.

Membership follows ``meep_gpu/chunk_map.py:180`` (``one_rank_line``): MEEP picks the
split-field recurrence per structure CHUNK, and on one rank the low and high PML
chunks span ``int(cells + 1.5)`` array cells from each wall. A cell whose chunk
carries an axis's layer steps the recurrence (with its auxiliary array) even where its
own sigma is zero; every other cell steps the auxiliary-free form, which is exact
because every coefficient outside the membership is exactly 1.0 (checked here).

The membership on each (lattice, axis) is at most two runs ``[a0, a1) U [b0, b1)``,
the same four words per (lattice, axis) as the reference's ``chunk_bounds_record``
(``chunk_map.py:897``). The device stores every auxiliary array as a full grid volume
of which only the cells whose coordinate along the array's axis lies in those runs are
ever read or written: a cell's auxiliary word sits at the cell's own offset, and the
untouched cells move no bytes.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Dict, List, Tuple

import numpy as np

from .grid import AXIS_NAMES, Grid, Unsupported

Faces = Tuple[Tuple[float, float], Tuple[float, float], Tuple[float, float]]

INTEGER, HALF = 0, 1


def half_cell_extent(cells: float) -> int:
    """How deep one face reaches, in half cells: MEEP's ``(int)(dx * 2a + 0.5)`` (pml.py:132)."""
    return int(2.0 * float(cells) + 0.5)


def normalize_thickness(thickness: Any) -> Faces:
    """Per-axis ``(low, high)`` thickness in cells from the reference's spellings.

    A scalar covers all six faces; a 3-sequence gives each axis (scalar or
    ``(low, high)``); a mapping ``{'x': t, 'y': {'low': a, 'high': b}}`` names axes.
    """
    def side_pair(value: Any) -> Tuple[float, float]:
        if isinstance(value, dict):
            unknown = set(value) - {"low", "high"}
            if unknown:
                raise ValueError(f"unknown PML sides {sorted(unknown)!r}")
            pair = (float(value.get("low", 0.0)), float(value.get("high", 0.0)))
        elif isinstance(value, (tuple, list)):
            if len(value) != 2:
                raise ValueError(f"a per-side PML thickness needs (low, high), got {value!r}")
            pair = (float(value[0]), float(value[1]))
        else:
            pair = (float(value), float(value))
        for side in pair:
            if not math.isfinite(side) or side < 0:
                raise ValueError(f"PML thickness must be finite and >= 0, got {value!r}")
        return pair

    if isinstance(thickness, dict):
        unknown = set(thickness) - set(AXIS_NAMES)
        if unknown:
            raise ValueError(f"unknown PML axes {sorted(unknown)!r}")
        return tuple(side_pair(thickness.get(name, 0.0)) for name in AXIS_NAMES)  # type: ignore[return-value]
    if isinstance(thickness, (tuple, list)):
        if len(thickness) != 3:
            raise ValueError(f"a per-axis PML thickness needs three entries, got {thickness!r}")
        return tuple(side_pair(v) for v in thickness)  # type: ignore[return-value]
    return (side_pair(thickness),) * 3  # type: ignore[return-value]


def one_rank_line(n_cells: int, faces: Tuple[float, float], lattice: int, wraps: bool) -> np.ndarray:
    """Per stored cell: is it owned by a one-rank chunk that carries this axis's layer?

    The chunk beside each face spans ``int(cells + 1.5)`` array cells; integer
    samples of a chunk ``[c0, c1]`` are owned at ``c0+2 .. c1`` (its upper plane belongs
    to it) and half-integer samples at ``c0+1 .. c1-1``, MEEP's owned-corner rule.
    On a wrapping axis stored integer cell 0 is the image of the high wall plane.
    """
    low, high = faces
    inside = np.zeros(n_cells, dtype=bool)
    if low > 0:
        span = min(n_cells, int(low + 1.5))
        if lattice == HALF:
            inside[0:span] = True
        else:
            inside[1:min(n_cells, span + 1)] = True
    if high > 0:
        span = min(n_cells, int(high + 1.5))
        if lattice == HALF:
            inside[n_cells - span:] = True
        else:
            inside[max(0, n_cells - span + 1):] = True
            if wraps:
                inside[0] = True
    return inside


def runs_of(line: np.ndarray) -> Tuple[int, int, int, int]:
    """The membership line as ``(a0, a1, b0, b1)``: a low run and a high run.

    An absent low run is ``(0, 0)``; an absent high run is ``(n, n)``. A line that
    is not the union of at most two runs (one may start at 0, one must end at n when
    both exist) is refused.
    """
    n = line.size
    edges = np.flatnonzero(np.diff(np.concatenate(([0], line.astype(np.int8), [0]))))
    runs = [(int(edges[i]), int(edges[i + 1])) for i in range(0, edges.size, 2)]
    if not runs:
        return (0, 0, n, n)
    if len(runs) == 1:
        start, stop = runs[0]
        if stop == n and start > 0:
            return (0, 0, start, stop)
        return (start, stop, n, n)
    if len(runs) == 2 and runs[1][1] == n:
        return (runs[0][0], runs[0][1], runs[1][0], runs[1][1])
    raise Unsupported(f"PML membership {runs} is not two runs; only the one-rank division is stepped")


def slab_rows(record: Tuple[int, int, int, int]) -> int:
    a0, a1, b0, b1 = record
    return (a1 - a0) + (b1 - b0)


def slab_index(record: Tuple[int, int, int, int], index: np.ndarray) -> np.ndarray:
    """Compact slab row of each axis position (-1 outside both runs)."""
    a0, a1, b0, b1 = record
    index = np.asarray(index)
    out = np.full(index.shape, -1, dtype=np.int64)
    low = (index >= a0) & (index < a1)
    high = (index >= b0) & (index < b1)
    out[low] = index[low] - a0
    out[high] = (a1 - a0) + index[high] - b0
    return out


@dataclass(frozen=True)
class AxisTables:
    """The three coefficient vectors of one (axis, lattice), in both precisions."""

    kms: np.ndarray
    sinv: np.ndarray
    kps: np.ndarray
    kms64: np.ndarray
    sinv64: np.ndarray
    kps64: np.ndarray
    sigma64: np.ndarray


class PML:
    """Graded UPML on any subset of the six faces, with the one-rank membership."""

    def __init__(self, grid: Grid, thickness: Any, order: int = 2, R_asymptotic: float = 1e-15):
        if order < 1:
            raise ValueError(f"PML grading order must be at least 1, got {order}")
        if not 0.0 < R_asymptotic < 1.0:
            raise ValueError(f"R_asymptotic must lie in (0, 1), got {R_asymptotic}")
        self.grid = grid
        self.order = int(order)
        self.R_asymptotic = float(R_asymptotic)
        self.faces: Faces = self._resolve_invariant_faces(
            self._resolve_mirror_faces(normalize_thickness(thickness), thickness), thickness)
        for axis, n in enumerate(grid.shape):
            low, high = self.faces[axis]
            if low + high > n:
                raise ValueError(
                    f"PML thickness (low={low}, high={high}) does not fit on the "
                    f"{AXIS_NAMES[axis]} axis ({n} cells)")
        self.tables: Dict[Tuple[int, int], AxisTables] = {}
        self.records: Dict[Tuple[int, int], Tuple[int, int, int, int]] = {}
        for axis in range(3):
            for lattice in (INTEGER, HALF):
                self.tables[(lattice, axis)] = self._axis_tables(axis, lattice)
                line = one_rank_line(grid.shape[axis], self.faces[axis], lattice,
                                     grid.axis_wraps(axis))
                self.records[(lattice, axis)] = runs_of(line)
                self._check_unit_outside(axis, lattice, line)

    def _resolve_invariant_faces(self, faces: Faces, request: Any) -> Faces:
        """No layer on an invariant axis (z of a 2-D run, x and y of a 1-D one: it has no
        faces). A request that puts one there, a scalar thickness included, is refused as
        the reference refuses it (``driver.py:2248``): name the axes the run resolves."""
        for axis in range(3):
            if self.grid.is_invariant(axis) and faces[axis] != (0.0, 0.0):
                raise ValueError(f"the PML puts {faces[axis]} cells on the {AXIS_NAMES[axis]} axis, which "
                                 f"dimensions={self.grid.dimensions} makes translationally invariant: it has "
                                 "no face to absorb at; request the layers on the axes the run resolves")
        return faces

    def _resolve_mirror_faces(self, faces: Faces, request: Any) -> Faces:
        """No layer on the low face of a folded axis: its cell 0 straddles the mirror plane,
        a boundary condition, not a wall. A scalar request means every face that can carry
        a layer and skips it; a request naming that face is refused (reference
        ``pml.py:387`` ``_resolve_mirror_faces``)."""
        uniform = not isinstance(request, (dict, tuple, list))
        resolved = list(faces)
        for axis in range(3):
            low, high = faces[axis]
            if not self.grid.is_mirrored(axis) or low == 0:
                continue
            if not uniform:
                raise ValueError(
                    f"PML requested at the {AXIS_NAMES[axis]} low face ({low} cells), but the "
                    f"{AXIS_NAMES[axis].upper()} axis is mirror-symmetric: cell 0 lies on the mirror "
                    f"plane, which is a boundary condition, not an absorber. Ask for the high face "
                    f"only, e.g. {{'{AXIS_NAMES[axis]}': {{'high': {low}}}}}.")
            resolved[axis] = (0.0, high)
        return tuple(resolved)  # type: ignore[return-value]

    @property
    def is_active(self) -> bool:
        return any(low > 0 or high > 0 for low, high in self.faces)

    def prefac(self, cells: float) -> float:
        """``-ln(R) / (4 * dx_pml * 1/(order+1))`` for one face (pml.py:436)."""
        dx_pml = cells * self.grid.dx
        if dx_pml <= 0:
            return 0.0
        profile_integral = 1.0 / (self.order + 1)
        return float(-np.log(self.R_asymptotic) / (4.0 * dx_pml * profile_integral))

    def graded_sigma64(self, axis: int, lattice: int, scale_factor: float) -> np.ndarray:
        """Float64 ``scale_factor * prefac * u**order`` at each stored sample of one lattice.

        MEEP's ``pml_x`` distance rule on the half-cell index ``i = 2j + lattice``
        (index 0 of a wrapping integer lattice is the upper wall's image, ``2n``).
        """
        n = self.grid.shape[axis]
        sig = np.zeros(n, dtype=np.float64)
        half_index = 2 * np.arange(n) + lattice
        if self.grid.axis_wraps(axis):
            half_index = (half_index - 1) % (2 * n) + 1
        # the upper wall is MEEP's window top, 2 * owned cells: on a folded periodic axis
        # the stored rows run one cell past it (reference pml.py:600 _wall_high)
        wall_high = 2 * self.grid.owned_cells(axis)
        for wall, n_pml in ((0, self.faces[axis][0]), (wall_high, self.faces[axis][1])):
            if n_pml <= 0:
                continue
            scale = scale_factor * self.prefac(n_pml)
            extent = half_cell_extent(n_pml)
            distance = np.abs(half_index - wall)
            overhang = extent - 2.0 * n_pml
            u = 1.0 + (overhang - distance) / (2.0 * n_pml)
            inside = distance < extent
            sig[inside] = scale * u[inside] ** self.order
        return sig

    def _axis_tables(self, axis: int, lattice: int) -> AxisTables:
        sigma64 = self.graded_sigma64(axis, lattice, 0.5 * self.grid.dt)
        sig = sigma64.astype(np.float32)
        kap = np.ones_like(sig)
        sinv = np.float32(1.0) / (kap + sig)
        kms = kap - sig
        kps = kap + sig
        return AxisTables(kms=kms, sinv=sinv, kps=kps,
                          kms64=1.0 - sigma64, sinv64=1.0 / (1.0 + sigma64),
                          kps64=1.0 + sigma64, sigma64=sigma64)

    def _check_unit_outside(self, axis: int, lattice: int, line: np.ndarray) -> None:
        table = self.tables[(lattice, axis)]
        outside = ~line
        if lattice == INTEGER and self.grid.is_metallic(axis):
            # The wall plane is not owned: its curl is masked and its word held at zero.
            outside[0] = False
        for name in ("kms", "sinv", "kps"):
            values = getattr(table, name)[outside]
            if values.size and not np.all(values == np.float32(1.0)):
                raise Unsupported(
                    f"PML {name} is not 1 outside the {AXIS_NAMES[axis]} membership; the "
                    "auxiliary-free form would not be exact there")

    def record(self, lattice: int, axis: int) -> Tuple[int, int, int, int]:
        return self.records[(lattice, axis)]

    def membership(self, lattice: int, axis: int) -> np.ndarray:
        a0, a1, b0, b1 = self.records[(lattice, axis)]
        line = np.zeros(self.grid.shape[axis], dtype=bool)
        line[a0:a1] = True
        line[b0:b1] = True
        return line

    def __repr__(self) -> str:
        return f"PML(faces={self.faces}, order={self.order}, R={self.R_asymptotic:.0e})"


def no_pml_records(grid: Grid) -> Dict[Tuple[int, int], Tuple[int, int, int, int]]:
    """Empty membership on every (lattice, axis), for a run with no absorber."""
    return {(lattice, axis): (0, 0, grid.shape[axis], grid.shape[axis])
            for lattice in (INTEGER, HALF) for axis in range(3)}


def identity_tables(grid: Grid) -> Dict[Tuple[int, int], AxisTables]:
    tables = {}
    for axis in range(3):
        n = grid.shape[axis]
        ones32 = np.ones(n, dtype=np.float32)
        ones64 = np.ones(n, dtype=np.float64)
        for lattice in (INTEGER, HALF):
            tables[(lattice, axis)] = AxisTables(ones32, ones32, ones32, ones64, ones64, ones64,
                                                 np.zeros(n))
    return tables


# Which auxiliary a component's PML form keys on, and on which lattice: the curl
# recurrence of B and D on the component's dsigu axis (MEEP's cycle X->Y->Z, dsig =
# next axis, dsigu = the one after; reference stepping.py:253-261), the constitutive
# accumulation of H and E on the component's own axis (stepping.py:266-267).
CURL_AXES = {0: (1, 2), 1: (2, 0), 2: (0, 1)}  # component axis -> (dsig, dsigu)


def curl_aux_key(field: str, comp: int) -> Tuple[int, int]:
    """(lattice, axis) of the curl auxiliary ``fu`` for B or D component ``comp``."""
    lattice = HALF if field == "B" else INTEGER
    return (lattice, CURL_AXES[comp][1])


def constitutive_aux_key(field: str, comp: int) -> Tuple[int, int]:
    """(lattice, axis) of the constitutive auxiliary ``f_w`` (and stored H) for H or E."""
    lattice = INTEGER if field == "H" else HALF
    return (lattice, comp)


def aux_shape(grid: Grid, record: Tuple[int, int, int, int], axis: int) -> Tuple[int, int, int]:
    shape: List[int] = list(grid.shape)
    shape[axis] = slab_rows(record)
    return tuple(shape)  # type: ignore[return-value]
