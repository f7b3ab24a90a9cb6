"""D and B conductivity: MEEP's ``D_conductivity`` / ``B_conductivity`` and ``mp.Absorber``.

A conductivity sigma on a D (or B) component replaces its curl update ``f -= curl`` by
MEEP's ``f = ((condfac * f) - curl) * condinv`` (step_generic.cpp:87-97), with

    condfac = 1 - sigma * dt/2   (float32, from dt2 = float32(dt) * 0.5)
    condinv = 1 / (1 + sigma * dt/2)   (double, rounded once)

as the reference forms them (``meep_gpu/fields.py:822`` ``_set_conductivity_side``).
Under a PML the lossy curl has four forms chosen per structure chunk
(``meep_gpu/stepping.py:2844`` ``_apply_conductive_pml_update``): whether the chunk
carries the component's dsig and dsigu layers, and whether it keeps a conductivity array
for the component at all (``meep_gpu/chunk_map.py:720`` ``conductive_chunks``: MEEP
deletes a chunk's array when every sample of its loop volume is zero). On one rank the
chunks are the product of (low PML, interior, high PML) pieces per axis
(``ChunkLayout.one_rank``, ``chunk_map.py:384``); this module gives every stored row
its piece and every component a 27-bit mask of the chunks that keep it.

``mp.Absorber`` is a graded conductivity added to both sides (``meep_gpu/absorber.py``):
per face a table ``prof[i] = prefac * (i/N)^2`` over N half-pixels
(``absorber_profile`` :112, MEEP's ``set_cond_profile``), looked up linearly at each
component's own Yee coordinate and summed over faces (``_sigma_along_axis`` :155,
``absorber_conductivity`` :268).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Dict, Mapping, Optional, Sequence, Tuple

import numpy as np

from .grid import AXIS_NAMES, IYEE, Grid, Unsupported

D_COMPONENTS = ("Dx", "Dy", "Dz")
B_COMPONENTS = ("Bx", "By", "Bz")
CONDUCTIVITY_COMPONENTS = D_COMPONENTS + B_COMPONENTS
# A source in a run whose conductivity reaches into a PML stays this many cells inside
# every absorbing face (meep_gpu/driver.py:313, :2520).
SOURCE_CLEARANCE_CELLS = 2.0
DEFAULT_R_ASYMPTOTIC = 1e-15
# integral of the quadratic profile u^2 over [0, 1]
QUADRATIC_PROFILE_INTEGRAL = 1.0 / 3.0
LOW, INTERIOR, HIGH = 0, 1, 2


@dataclass(frozen=True)
class AbsorberLayer:
    """One ``mp.Absorber`` face (``meep_gpu/absorber.py:68``): a thickness in length
    units on the ``"low"`` or ``"high"`` side of axis 0/1/2."""

    thickness: float
    axis: int
    side: str
    R_asymptotic: float = DEFAULT_R_ASYMPTOTIC

    def __post_init__(self) -> None:
        if self.axis not in (0, 1, 2):
            raise ValueError(f"absorber axis must be 0, 1 or 2, got {self.axis!r}")
        if self.side not in ("low", "high"):
            raise ValueError(f"absorber side must be 'low' or 'high', got {self.side!r}")
        if not math.isfinite(self.thickness) or self.thickness <= 0.0:
            raise ValueError(f"absorber thickness must be finite and > 0, got {self.thickness!r}")
        if not math.isfinite(self.R_asymptotic) or not 0.0 < self.R_asymptotic < 1.0:
            raise ValueError(f"absorber R_asymptotic must lie in (0, 1), got {self.R_asymptotic!r}")


def absorber_profile(thickness: float, resolution: float,
                     R_asymptotic: float = DEFAULT_R_ASYMPTOTIC) -> Tuple[int, np.ndarray]:
    """``(N, prof)``: N = int(L / (half a pixel) + 0.5) and prof[i] = prefac * (i/N)^2
    with prefac = -ln(R) / (4 L * 1/3), the table MEEP samples at half-pixel spacing."""
    half_pixel = 0.5 / resolution
    count = int(thickness / half_pixel + 0.5)
    if count < 1:
        raise ValueError(f"absorber thickness {thickness!r} spans less than half a half-pixel at "
                         f"resolution {resolution!r}; its profile table would be empty")
    prefac = (-math.log(R_asymptotic)) / (4.0 * thickness * QUADRATIC_PROFILE_INTEGRAL)
    index = np.arange(count + 1, dtype=np.float64)
    return count, prefac * (index / count) ** 2


def _layer_sigma(coordinates: np.ndarray, layer: AbsorberLayer, half_length: float,
                 resolution: float) -> np.ndarray:
    """One face's sigma at the given coordinates: inside the layer u = N * depth / L,
    linear interpolation between prof[int(u)] and prof[int(u) + 1], prof[N] past the end."""
    count, profile = absorber_profile(layer.thickness, resolution, layer.R_asymptotic)
    thickness = float(layer.thickness)
    if layer.side == "high":
        edge = half_length - thickness
        inside = coordinates >= edge
        depth = count * (coordinates - edge) / thickness
    else:
        edge = thickness - half_length
        inside = coordinates <= edge
        depth = count * (edge - coordinates) / thickness
    out = np.zeros(coordinates.shape, dtype=np.float64)
    if not np.any(inside):
        return out
    u = np.where(inside, depth, 0.0)
    lower = np.floor(u).astype(np.int64)
    frac = u - lower
    past = lower >= count
    lower = np.minimum(lower, count - 1)
    value = profile[lower] * (1.0 - frac) + profile[lower + 1] * frac
    out[...] = np.where(inside, np.where(past, profile[count], value), 0.0)
    return out


def snapped_lengths(grid: Grid) -> Tuple[float, float, float]:
    """The unfolded cell lengths snapped to the grid, n * dx (the reference's
    Grid.Lx/Ly/Lz); on a folded axis the full cell's, so a low-face absorber there never
    reaches a stored cell (reference ``absorber.py:174``)."""
    return tuple(n * grid.dx for n in grid.shape_full)  # type: ignore[return-value]


def _axis_coordinates(grid: Grid, axis: int, shift: int) -> np.ndarray:
    """Coordinates of the stored rows of one Yee sub-lattice, as MEEP forms them from one
    doubled integer (``doubled * dx/2``). On a wrapping axis the integer row 0 is the
    image of the top wall plane and takes that plane's coordinate (``absorber.py:218``)."""
    n = grid.shape[axis]
    index = np.arange(n, dtype=np.int64)
    if shift == 0 and grid.axis_wraps(axis):
        index = np.concatenate(([n], np.arange(1, n, dtype=np.int64)))
    doubled = grid.origin_doubled(axis) + 2 * index + shift
    return doubled * (0.5 * float(grid.dx))


def absorber_conductivity(grid: Grid, layers: Sequence[AbsorberLayer]) -> Dict[str, np.ndarray]:
    """Six float64 sigma volumes (Dx..Dz, Bx..Bz) for a set of absorber faces, each
    sampled at its component's own Yee position and summed over the faces; empty for no
    layers."""
    if not layers:
        return {}
    resolution = 1.0 / float(grid.dx)
    lengths = snapped_lengths(grid)
    per_axis: list = [[None, None], [None, None], [None, None]]
    for layer in layers:
        for shift in (0, 1):
            contribution = _layer_sigma(_axis_coordinates(grid, layer.axis, shift), layer,
                                        lengths[layer.axis] / 2.0, resolution)
            existing = per_axis[layer.axis][shift]
            per_axis[layer.axis][shift] = contribution if existing is None else existing + contribution
    shape = grid.shape
    volumes: Dict[str, np.ndarray] = {}
    for component in CONDUCTIVITY_COMPONENTS:
        shifts = IYEE[component]
        total = np.zeros(shape, dtype=np.float64)
        for axis in range(3):
            line = per_axis[axis][shifts[axis]]
            if line is None:
                continue
            view = [1, 1, 1]
            view[axis] = shape[axis]
            total = total + line.reshape(view)
        volumes[component] = total
    return volumes


def coefficients(sigma: np.ndarray, dt: float) -> Tuple[np.ndarray, np.ndarray]:
    """``(condfac, condinv)`` float32 volumes of one float32 sigma volume."""
    values = np.ascontiguousarray(sigma, dtype=np.float32)
    dt2 = np.float32(np.float32(dt) * np.float32(0.5))
    condfac = (np.float32(1.0) - values * dt2).astype(np.float32)
    wide = values.astype(np.float64)
    condinv = (1.0 / (1.0 + (wide * float(dt)) * 0.5)).astype(np.float32)
    return condfac, condinv


# --- one-rank chunks --------------------------------------------------------------------
def axis_pieces(n: int, faces: Tuple[float, float]) -> Tuple[Tuple[int, int, int], ...]:
    """The chunk pieces along one axis as ``(piece, lo, hi)`` in doubled offsets from the
    low wall: a face's chunk spans ``int(cells + 1.5)`` cells (``chunk_map.py:384``)."""
    low, high = faces
    low_hi = 2 * min(n, int(low + 1.5)) if low > 0 else 0
    high_lo = 2 * n - 2 * min(n, int(high + 1.5)) if high > 0 else 2 * n
    if low_hi > high_lo:
        raise Unsupported("the two PML chunks of an axis overlap; a conductivity under such a PML is not stepped")
    pieces = ((LOW, 0, low_hi), (INTERIOR, low_hi, high_lo), (HIGH, high_lo, 2 * n))
    return tuple(p for p in pieces if p[1] < p[2])


def piece_line(n: int, faces: Tuple[float, float], lattice: int, wraps: bool,
               owned: Optional[int] = None) -> np.ndarray:
    """The piece owning each stored row of one sub-lattice (0 integer, 1 half).

    A row at doubled offset p belongs to the piece with lo < p <= hi (MEEP's ``owns``).
    The integer row 0 is the wall: on a wrapping axis it is the image of the top wall
    (p = 2n), on a metallic or folded one it is not owned and takes its neighbour row 1's
    chunk. The pieces span MEEP's window, ``owned`` cells (the stored count unless a
    folded periodic axis stores one row past it, the far ghost slot, which takes the top
    piece).
    """
    owned = n if owned is None else owned
    pieces = axis_pieces(owned, faces)
    line = np.empty(n, dtype=np.int8)
    for r in range(n):
        p = 2 * r + lattice
        if p == 0:
            p = 2 * n if wraps else 2
        p = min(p, 2 * owned)
        line[r] = next(piece for piece, lo, hi in pieces if lo < p <= hi)
    return line


def piece_rows(n: int, lo: int, hi: int, wraps: bool) -> np.ndarray:
    """The stored rows of a piece's loop volume: its owned samples plus the one beyond
    (``chunk_map.py:675`` ``loop_rows``): rows lo/2 .. hi/2, wrapped or clipped."""
    rows = np.arange(lo // 2, hi // 2 + 1, dtype=np.int64)
    return rows % n if wraps else np.clip(rows, 0, n - 1)


def keeps_mask(grid: Grid, faces, sigma: np.ndarray) -> int:
    """Bit (x * 9 + y * 3 + z) set for each chunk whose loop volume holds a nonzero sigma."""
    per_axis = [axis_pieces(grid.owned_cells(a), faces[a]) for a in range(3)]
    mask = 0
    nonzero = sigma != 0
    for px, xlo, xhi in per_axis[0]:
        rx = piece_rows(grid.nx, xlo, xhi, grid.axis_wraps(0))
        for py, ylo, yhi in per_axis[1]:
            ry = piece_rows(grid.ny, ylo, yhi, grid.axis_wraps(1))
            for pz, zlo, zhi in per_axis[2]:
                rz = piece_rows(grid.nz, zlo, zhi, grid.axis_wraps(2))
                if np.any(nonzero[np.ix_(rx, ry, rz)]):
                    mask |= 1 << (px * 9 + py * 3 + pz)
    return mask


def reaches_a_pml(grid: Grid, faces, volumes: Mapping[str, Optional[np.ndarray]]) -> bool:
    """Whether any conductivity is nonzero inside an absorbing face, padded by one cell
    (``meep_gpu/driver.py:2452`` ``_conductivity_reaches_a_pml``)."""
    for sigma in volumes.values():
        if sigma is None:
            continue
        inside = np.zeros(grid.shape, dtype=bool)
        for axis in range(3):
            low, high = faces[axis]
            n = grid.shape[axis]
            top = grid.owned_cells(axis)  # the high face sits at MEEP's window top
            line = np.zeros(n, dtype=bool)
            if low:
                line[:min(int(math.ceil(low)) + 1, n)] = True
            if high:
                line[max(top - int(math.ceil(high)) - 1, 0):] = True
            view = [1, 1, 1]
            view[axis] = n
            inside |= line.reshape(view)
        if np.any(inside & (sigma != 0)):
            return True
    return False


def require_source_clear(grid: Grid, faces, center: Sequence[float], size: Sequence[float]) -> None:
    """Refuse a source closer than ``SOURCE_CLEARANCE_CELLS`` to a PML face (the caller
    checks first that the conductivity reaches a PML; ``driver.py:2520``)."""
    margin = SOURCE_CLEARANCE_CELLS * grid.dx
    lengths = snapped_lengths(grid)
    violations = []
    for axis in range(3):
        low_cells, high_cells = faces[axis]
        low = center[axis] - size[axis] / 2.0
        high = center[axis] + size[axis] / 2.0
        if low_cells:
            limit = -lengths[axis] / 2.0 + low_cells * grid.dx + margin
            violations.append((limit - low, axis, "low", low, limit))
        if high_cells:
            limit = lengths[axis] / 2.0 - high_cells * grid.dx - margin
            violations.append((high - limit, axis, "high", high, limit))
    offending = [v for v in violations if v[0] > 1e-12]
    if not offending:
        return
    amount, axis, side, endpoint, limit = max(offending)
    raise ValueError(
        f"A source in a run combining a conductivity with PML must stay at least "
        f"{SOURCE_CLEARANCE_CELLS:g} grid cells ({margin:g} length units) inside every absorbing "
        f"face. Its {AXIS_NAMES[axis]}-{side} endpoint {endpoint:g} crosses the limit {limit:g} "
        f"by {amount:g}. Move or shrink the source.")


def coerce(value: Any, shape: Tuple[int, int, int], side: str) -> Optional[np.ndarray]:
    """One conductivity entry as a float32 volume, or None for no loss (None, or zero
    everywhere); scalars, grid-shaped volumes and MEEP's (n+1)-padded volumes are taken
    (``driver.py:1808`` ``_coerce_conductivity``)."""
    if value is None:
        return None
    probe = np.asarray(value)
    if np.iscomplexobj(probe):
        raise ValueError(f"{side} conductivity must be real: MEEP's sigma_{side} is a real loss rate")
    values = probe.astype(np.float64)
    if values.ndim == 0:
        uniform = float(values)
        if not math.isfinite(uniform) or uniform < 0.0:
            raise ValueError(f"{side} conductivity must be finite and >= 0, got {value!r}; a negative "
                             f"conductivity is gain")
        if uniform == 0.0:
            return None
        return np.full(shape, uniform, dtype=np.float32)
    if values.ndim != 3:
        raise ValueError(f"{side} conductivity must be a scalar or a 3-D array, got {values.ndim} dimensions")
    if values.shape == tuple(shape):
        trimmed = values
    elif values.shape == tuple(n + 1 for n in shape):
        trimmed = values[:-1, :-1, :-1]
    else:
        raise ValueError(f"{side} conductivity shape {values.shape} matches neither the grid shape "
                         f"{tuple(shape)} nor the boundary-padded shape {tuple(n + 1 for n in shape)}")
    if not np.all(np.isfinite(trimmed)) or np.any(trimmed < 0.0):
        raise ValueError(f"{side} conductivity must be finite and >= 0 in every cell; a negative value is gain")
    if not np.any(trimmed != 0.0):
        return None
    return np.ascontiguousarray(trimmed.astype(np.float32))


def compose(components: Tuple[str, ...], material: Optional[Mapping[str, Optional[np.ndarray]]],
            absorber: Mapping[str, np.ndarray]) -> Dict[str, Optional[np.ndarray]]:
    """Material sigma plus the absorber ramp per component, summed in float64 and rounded
    once to float32 (``driver.py:1955`` ``_compose_conductivity_side``)."""
    out: Dict[str, Optional[np.ndarray]] = {}
    for component in components:
        own = None if material is None else material.get(component)
        ramp = absorber.get(component)
        if ramp is None:
            out[component] = own
        elif own is None:
            out[component] = np.ascontiguousarray(ramp.astype(np.float32))
        else:
            out[component] = np.ascontiguousarray((own.astype(np.float64) + ramp).astype(np.float32))
    return out
