"""The Yee grid of one simulation: cell counts, spacing, time step, registration.

Follows the reference's ``meep_gpu/grid.py`` (``Grid``, :288 ``meep_cell_count``,
:426-438 dx/dt/counts, :1095 ``origin_doubled``, :1292 ``_create_coordinates``) for
the subset this engine steps: three resolved dimensions, per-axis boundaries that are
either MEEP metallic walls or periodic wraps (Bloch-phased where the axis has a nonzero
``k_point`` component), and mirror planes (``Mirror``) folding metallic axes.

Registration: cell ``i`` of a component with Yee shift ``s`` on an axis sits at the
doubled coordinate ``origin_doubled + 2*i + s``; ``origin_doubled`` is ``-(n - n % 2)``,
MEEP's centred origin (odd counts start half a cell higher), and ``-2`` on a folded
axis (MEEP's ``grid_volume::halve``: cell 0 one cell below the plane at doubled 0).
"""

from __future__ import annotations

import ctypes
import ctypes.util
import math
from typing import Any, Optional, Sequence, Tuple

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


MIRROR_AXES = ("X", "Y", "Z")


class Mirror:
    """One mirror plane through the cell centre: the axis it is normal to and its phase
    (reference ``grid.py:100``; MEEP's ``mp.Mirror(direction, phase)``). ``phase`` +1 is
    an even mirror, -1 an odd one; a mirror is an involution, so nothing else is taken."""

    __slots__ = ("axis", "phase")

    def __init__(self, axis: str, phase: int = 1):
        name = str(axis).upper()
        if name not in MIRROR_AXES:
            raise ValueError(f"mirror axis must be one of {list(MIRROR_AXES)}, got {axis!r}")
        if phase not in (1, -1) or isinstance(phase, bool):
            raise ValueError(f"mirror phase must be +1 (even) or -1 (odd), got {phase!r}")
        self.axis = name
        self.phase = int(phase)

    @property
    def axis_index(self) -> int:
        return MIRROR_AXES.index(self.axis)

    def __eq__(self, other) -> bool:
        return isinstance(other, Mirror) and (self.axis, self.phase) == (other.axis, other.phase)

    def __hash__(self) -> int:
        return hash((self.axis, self.phase))

    def __repr__(self) -> str:
        return f"Mirror({self.axis!r}, phase={self.phase:+d})"


def normalize_mirrors(symmetry: Any) -> Tuple[Optional[Mirror], Optional[Mirror], Optional[Mirror]]:
    """The plane on each axis, or None (reference ``grid.py:155``): a bare axis name is an
    even mirror; two planes on one axis are refused."""
    planes: list = [None, None, None]
    for entry in tuple(symmetry or ()):
        plane = entry if isinstance(entry, Mirror) else Mirror(entry)
        clash = planes[plane.axis_index]
        if clash is not None:
            raise ValueError(f"two mirror planes normal to {plane.axis}: {clash!r} and {plane!r}")
        planes[plane.axis_index] = plane
    return tuple(planes)  # type: ignore[return-value]


def mirror_parity(component: str, axis: int, phase: int = 1) -> int:
    """The sign a component takes under the mirror normal to ``axis`` (MEEP's
    ``symmetry::phase_shift``; reference ``fields.py:121``): a vector (E, D) is odd about
    the plane it is normal to and even otherwise, a pseudovector (H, B) the opposite, and
    the plane's phase multiplies both."""
    direction = "xyz".index(component[1])
    if component[0] in "ED":
        return -phase if direction == axis else phase
    return phase if direction == axis else -phase


_LIBM = None


def sincos(x: float) -> Tuple[float, float]:
    """``(sin x, cos x)`` from one libm ``sincos`` call, as a compiled ``exp`` of an
    imaginary argument takes them (reference ``readback.py:170``)."""
    global _LIBM
    if _LIBM is None:
        _LIBM = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    if hasattr(_LIBM, "sincos"):
        s, c = ctypes.c_double(), ctypes.c_double()
        _LIBM.sincos(ctypes.c_double(float(x)), ctypes.byref(s), ctypes.byref(c))
        return float(s.value), float(c.value)
    return math.sin(x), math.cos(x)


def cmul(a: Tuple[float, float], b: Tuple[float, float]) -> Tuple[float, float]:
    """Complex product, each operation rounded on its own: ``(ac - bd, ad + bc)``."""
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def creciprocal(c: float, d: float) -> Tuple[float, float]:
    """``1 / (c + i d)`` by Smith's algorithm (the complex division a C runtime without
    fast-math performs; no rescaling is needed for the unit-modulus phases it serves)."""
    if not (1e-150 < math.hypot(c, d) < 1e150):
        raise ValueError("a Bloch phase power must be of moderate modulus")
    if abs(c) < abs(d):
        ratio = c / d
        denom = (c * ratio) + d
        return ((1.0 * ratio + 0.0) / denom, (0.0 * ratio - 1.0) / denom)
    ratio = d / c
    denom = (d * ratio) + c
    return ((0.0 * ratio + 1.0) / denom, (0.0 - 1.0 * ratio) / denom)


def cpow_int(x: Tuple[float, float], n: int) -> Tuple[float, float]:
    """``pow(complex, int)`` by repeated squaring, and the reciprocal of the power for a
    negative exponent (the integer power a GCC-built C++ runtime takes)."""
    if n < 0:
        return creciprocal(*cpow_int(x, -n))
    y = x if n % 2 else (1.0, 0.0)
    n >>= 1
    while n:
        x = cmul(x, x)
        if n % 2:
            y = cmul(y, x)
        n >>= 1
    return y


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
    """Cell counts, spacing, dt and registration of one simulation: 3-D, 2-D with z
    translationally invariant, or 1-D along z with x and y invariant (reference
    ``grid.py:337``): MEEP leaves an invariant axis out of its loops, so every difference
    along it reads the same sample twice; here that is one stored cell with a periodic
    wrap, whose difference is the same exact zero."""

    def __init__(self, cell_size: Sequence[float], resolution: float, courant: float = 0.5,
                 boundaries: Any = None, k_point: Sequence[float] = (0.0, 0.0, 0.0),
                 symmetry: Any = (), dimensions: int = 3):
        if len(tuple(cell_size)) != 3:
            raise ValueError(f"cell_size needs three lengths, got {cell_size!r}")
        self.cell_size = tuple(float(v) for v in cell_size)
        self.resolution = float(resolution)
        if not (self.resolution > 0 and math.isfinite(self.resolution)):
            raise ValueError(f"resolution must be positive, got {resolution!r}")
        self.courant = float(courant)
        self.dx = 1.0 / self.resolution
        self.dt = self.courant / self.resolution
        if dimensions not in (1, 2, 3) or isinstance(dimensions, bool):
            raise Unsupported(f"dimensions {dimensions!r}: 3-D, 2-D (z invariant) and 1-D (along z) "
                              "runs are stepped by this engine")
        self.dimensions = int(dimensions)
        # the axes MEEP's loops carry (reference sources.py:770 _meep_directions): 2-D
        # drops z, 1-D keeps z alone
        self.directions = {3: (0, 1, 2), 2: (0, 1), 1: (2,)}[self.dimensions]
        self.invariant_axes = tuple(a not in self.directions for a in range(3))
        for axis in range(3):
            if self.invariant_axes[axis] and self.cell_size[axis] != 0.0:
                raise ValueError(f"dimensions={self.dimensions} makes {AXIS_NAMES[axis]} translationally "
                                 f"invariant: its cell_size must be 0 (an invariant axis has no extent), "
                                 f"got {self.cell_size[axis]!r}")
        counts = tuple(1 if self.invariant_axes[a] else cell_count(self.cell_size[a], self.resolution)
                       for a in range(3))
        self.shape_full = counts
        self.nx_full, self.ny_full, self.nz_full = counts
        self.boundaries = normalize_boundaries(boundaries)
        for axis in range(3):
            if self.boundaries[axis] != METALLIC:
                continue
            if self.invariant_axes[axis]:
                raise ValueError(f"the {AXIS_NAMES[axis]} axis is invariant at dimensions={self.dimensions}: "
                                 "it has no outer face, so it cannot be metallic (a wall there zeroes the "
                                 "components whose Yee shift on it is 0); leave it periodic")
            if counts[axis] < 2:
                raise ValueError(f"the {AXIS_NAMES[axis]} axis is metallic and holds {counts[axis]} cell(s): "
                                 "MEEP makes a one-cell direction periodic (fields.cpp, unit directions); "
                                 "declare it periodic or give it more cells")
        if min(counts) < 1:
            raise ValueError(f"every carried axis needs at least one cell, got {counts}")
        self.mirrors = normalize_mirrors(symmetry)
        for axis in range(3):
            if self.mirrors[axis] is not None and self.invariant_axes[axis]:
                raise ValueError(f"a mirror plane normal to the invariant {AXIS_NAMES[axis]} axis")
        # MEEP's halve(): n - n//2 + 1 owned cells on a folded axis, from one cell below the
        # plane (reference grid.py:604, vec.cpp halve); a folded periodic axis stores one
        # more, MEEP's big_corner plane and the far ghost slot past it
        self.nx, self.ny, self.nz = (
            self.owned_cells(a) + (0 if self.mirrors[a] is None or self.is_metallic(a) else 1)
            for a in range(3))
        for axis in range(3):
            if self.mirrors[axis] is not None and self.shape[axis] < 4:
                raise Unsupported(f"a folded axis needs at least 4 stored cells, {AXIS_NAMES[axis]} has "
                                  f"{self.shape[axis]}")
        self.k_point = tuple(float(k) for k in k_point)
        if len(self.k_point) != 3 or not all(math.isfinite(k) for k in self.k_point):
            raise ValueError(f"k_point needs three finite components, got {k_point!r}")
        for axis, k in enumerate(self.k_point):
            if k != 0.0 and not self.axis_wraps(axis):
                raise ValueError(
                    f"k_point component {AXIS_NAMES[axis]} = {k!r} on an axis declared "
                    f"{self.boundaries[axis]!r}: a Bloch phase says what the field is one lattice "
                    f"vector away, and a perfect-electric-conductor wall terminates the axis "
                    f"instead of repeating it. Make the axis periodic or set its k component to 0.")
        if self.has_symmetry and any(k != 0.0 for k in self.k_point):
            raise Unsupported("a nonzero k_point together with mirror symmetry is not stepped by this "
                              "engine (a folded axis carries no Bloch phase)")
        self.bloch_phases = tuple(self._bloch_phase(self.k_point[a], counts[a]) for a in range(3))
        self.has_bloch = any(p is not None for p in self.bloch_phases)

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
        return self.boundaries[axis] == PERIODIC and self.mirrors[axis] is None

    def is_invariant(self, axis: int) -> bool:
        """Whether the axis is translationally invariant (z of a 2-D run)."""
        return self.invariant_axes[axis]

    def nosize_direction(self, axis: int) -> bool:
        """MEEP's ``fields::nosize_direction`` (reference ``grid.py:1237``): a one-cell
        periodic axis stands for the whole direction, so a zero-extent source request
        there is not a delta function (its amplitude is not scaled by the resolution)."""
        return self.axis_wraps(axis) and self.shape_full[axis] == 1

    @property
    def has_symmetry(self) -> bool:
        return any(plane is not None for plane in self.mirrors)

    def is_mirrored(self, axis: int) -> bool:
        return self.mirrors[axis] is not None

    def owned_cells(self, axis: int) -> int:
        """MEEP's cell count of the axis (reference ``grid.py:1343``): the halved count
        ``n - n//2 + 1`` on a folded axis, the full count elsewhere. It differs from the
        stored count only on a folded periodic axis, which stores one cell more."""
        n = self.shape_full[axis]
        return n - n // 2 + 1 if self.mirrors[axis] is not None else n

    def far_reflect_row(self, axis: int) -> Optional[int]:
        """On a folded periodic axis, the stored row the far ghost slot (the last shift-1
        slot) and the sample past the top image about the second mirror at doubled
        ``n_full`` (reference ``stepping.py:2361``): ``n_full - stored + 2``; else None."""
        if self.mirrors[axis] is None or self.is_metallic(axis):
            return None
        return self.shape_full[axis] - self.shape[axis] + 2

    def mirror_phase(self, axis: int) -> Optional[int]:
        """The declared phase of the axis's plane, None on an unfolded axis."""
        plane = self.mirrors[axis]
        return None if plane is None else plane.phase

    def parity(self, component: str, axis: int) -> int:
        """``mirror_parity`` of a component about the axis's plane (the axis must be folded)."""
        return mirror_parity(component, axis, self.mirrors[axis].phase)

    def origin_doubled(self, axis: int) -> int:
        """MEEP's little corner on one axis in doubled units (reference grid.py:1095):
        ``-(n - n % 2)`` of the full count, ``-2`` on a folded axis."""
        if self.mirrors[axis] is not None:
            return -2
        n = self.shape_full[axis]
        return -(n - n % 2)

    def full_origin_doubled(self, axis: int) -> int:
        """The unfolded cell's little corner (the user volume)."""
        n = self.shape_full[axis]
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

    def _bloch_phase(self, k: float, n: int) -> Optional[complex]:
        """MEEP's ``eikna`` of one axis, ``exp(i k (2 pi / a) n)`` with the argument
        associated as MEEP forms it (reference ``grid.py:1009``): None at k = 0, exactly -1
        at the zone edge."""
        if k == 0.0:
            return None
        if k * n == 0.5 * self.resolution:
            return complex(-1.0, 0.0)
        sin_a, cos_a = sincos(k * ((2 * math.pi / self.resolution) * n))
        return complex(cos_a, sin_a)

    def bloch_phase(self, axis: int) -> Optional[complex]:
        """``f(x + L) = bloch_phase * f(x)`` on a phased axis; None where k is 0."""
        return self.bloch_phases[axis]

    def eikna(self, axis: int) -> Tuple[float, float]:
        phase = self.bloch_phases[axis]
        return (1.0, 0.0) if phase is None else (phase.real, phase.imag)

    def __repr__(self) -> str:
        folds = "" if not self.has_symmetry else f", symmetry={[m for m in self.mirrors if m]}"
        return (f"Grid({self.nx}x{self.ny}x{self.nz}, res={self.resolution:g}, "
                f"dt={self.dt:g}, boundaries={self.boundaries}{folds})")
