"""The Yee grid of one simulation: cell counts, spacing, time step, registration.

Follows the reference's ``meep_gpu/grid.py`` (``Grid``, :288 ``meep_cell_count``,
:426-438 dx/dt/counts, :1095 ``origin_doubled``, :1292 ``_create_coordinates``) for
the subset this engine steps: three resolved dimensions, real fields, no mirror
symmetry, and per-axis boundaries that are either MEEP metallic walls or plain
periodic wrap (Bloch vector zero).

Registration: cell ``i`` of a component with Yee shift ``s`` on an axis sits at the
doubled coordinate ``origin_doubled + 2*i + s``; ``origin_doubled`` is ``-(n - n % 2)``,
MEEP's centred origin (odd counts start half a cell higher).
"""

from __future__ import annotations

import math
from typing import Any, Sequence, Tuple

import numpy as np

AXIS_NAMES = ("x", "y", "z")
METALLIC = "metallic"
PERIODIC = "periodic"

# Yee shift of every component on (x, y, z), MEEP's iyee_shift
# (reference meep_gpu/fields.py:218-223).
IYEE = {
    "Ex": (1, 0, 0), "Ey": (0, 1, 0), "Ez": (0, 0, 1),
    "Dx": (1, 0, 0), "Dy": (0, 1, 0), "Dz": (0, 0, 1),
    "Hx": (0, 1, 1), "Hy": (1, 0, 1), "Hz": (1, 1, 0),
    "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0),
}


class Unsupported(ValueError):
    """A configuration outside what this engine steps, refused by name before any launch."""


def cell_count(length: float, resolution: float) -> int:
    """MEEP's ``int(size * a + 0.5)`` (reference grid.py:288)."""
    return int(length * resolution + 0.5)


def normalize_boundaries(boundaries: Any) -> Tuple[str, str, str]:
    """Per-axis boundary kind from the reference's spellings (grid.py ``_normalize_boundaries``).

    ``None`` is periodic on every axis (the reference driver's default); a single
    string applies to all three axes; a mapping or a 3-sequence names each axis.
    """
    if boundaries is None:
        return (PERIODIC,) * 3
    if isinstance(boundaries, str):
        kinds = (boundaries,) * 3
    elif isinstance(boundaries, dict):
        kinds = tuple(boundaries.get(name, PERIODIC) for name in AXIS_NAMES)
        unknown = set(boundaries) - set(AXIS_NAMES)
        if unknown:
            raise ValueError(f"unknown boundary axes {sorted(unknown)!r}")
    else:
        kinds = tuple(boundaries)
        if len(kinds) != 3:
            raise ValueError(f"boundaries needs one entry per axis, got {boundaries!r}")
    for kind in kinds:
        if kind not in (METALLIC, PERIODIC):
            raise Unsupported(
                f"boundary {kind!r} is not stepped by this engine; use 'metallic' or 'periodic'")
    return tuple(kinds)  # type: ignore[return-value]


class Grid:
    """Cell counts, spacing, dt and registration of one 3-D simulation."""

    def __init__(self, cell_size: Sequence[float], resolution: float, courant: float = 0.5,
                 boundaries: Any = None):
        if len(tuple(cell_size)) != 3:
            raise ValueError(f"cell_size needs three lengths, got {cell_size!r}")
        self.cell_size = tuple(float(v) for v in cell_size)
        self.resolution = float(resolution)
        if not (self.resolution > 0 and math.isfinite(self.resolution)):
            raise ValueError(f"resolution must be positive, got {resolution!r}")
        self.courant = float(courant)
        self.dx = 1.0 / self.resolution
        self.dt = self.courant / self.resolution
        counts = tuple(cell_count(length, self.resolution) for length in self.cell_size)
        if min(counts) < 2:
            raise Unsupported(
                f"every axis needs at least 2 cells (got {counts}); reduced-dimension runs "
                "are not stepped by this engine")
        self.nx, self.ny, self.nz = counts
        self.boundaries = normalize_boundaries(boundaries)

    # --- registration -------------------------------------------------------------
    @property
    def shape(self) -> Tuple[int, int, int]:
        return (self.nx, self.ny, self.nz)

    @property
    def total_cells(self) -> int:
        return self.nx * self.ny * self.nz

    def count(self, axis: int) -> int:
        return self.shape[axis]

    def is_metallic(self, axis: int) -> bool:
        return self.boundaries[axis] == METALLIC

    def axis_wraps(self, axis: int) -> bool:
        return self.boundaries[axis] == PERIODIC

    def origin_doubled(self, axis: int) -> int:
        """MEEP's little corner on one axis in doubled units (reference grid.py:1095)."""
        n = self.shape[axis]
        return -(n - n % 2)

    def axis_origin(self, axis: int) -> float:
        return self.origin_doubled(axis) * self.dx / 2

    def axis_coordinates(self, axis: int) -> np.ndarray:
        """Cell-centre coordinates as float32, ``origin + (i + 0.5) dx`` (grid.py:1292)."""
        n = self.shape[axis]
        start = self.axis_origin(axis) + self.dx / 2
        return np.linspace(start, start + (n - 1) * self.dx, n, dtype=np.float32)

    @property
    def x(self) -> np.ndarray:
        return self.axis_coordinates(0)

    @property
    def y(self) -> np.ndarray:
        return self.axis_coordinates(1)

    @property
    def z(self) -> np.ndarray:
        return self.axis_coordinates(2)

    def meshgrid(self):
        """Cell-centre coordinates in (x, y, z) index order, as the reference's ``Grid.meshgrid``."""
        return np.meshgrid(self.x, self.y, self.z, indexing="ij")

    def __repr__(self) -> str:
        return (f"Grid({self.nx}x{self.ny}x{self.nz}, res={self.resolution:g}, "
                f"dt={self.dt:g}, boundaries={self.boundaries})")
