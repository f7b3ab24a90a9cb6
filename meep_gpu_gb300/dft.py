"""DFT field monitors and flux planes: registration, weights and read-out.

Registration follows the reference's ``meep_gpu/dft.py``: every axis of a monitor
volume takes its cells from MEEP's ``vec2diel_floor``/``vec2diel_ceil`` ladder of
the requested bounds on the centred lattice (``_boundary_weight_ladder`` :604,
``_axis_ladder`` :857, ``_register_volume`` :1259), and the flux surface weights are
the ladder's Simpson tapers per axis (``_fractional_cell_weights`` :1208,
``_volume_boundary_weights`` :2753). A plane requested between two rows of cell
centres is bracketed by both and linearly interpolated, MEEP's zero-thickness rule.

Accumulation (done on the device by ``dft_accumulate`` in the CUDA library) is
MEEP's ``update_dft`` as the reference runs it (``DFTMonitor.update`` :2197,
``FluxMonitor.update`` :3031, ``_phase_factors`` :316, ``_apply_yee_interpolation``
:352): on steps with ``step % d == 0`` (post-increment count), E is sampled at
``t = step*dt`` and H at ``t - dt/2``, each averaged onto cell centres along every
axis where its Yee shift is 0 (x, then y, then z), and
``acc += complex64(exp(i w t) * dt*d/sqrt(2 pi)) * sample``. The phase is formed in
float64 on the device from the exact time, so it does not drift over long runs.

The flux reduction (``FluxMonitor._integrate_flux`` :3107) is
``sum_w Re(E_a conj(H_b) - E_b conj(H_a)) * dA * weight`` over the tangential pair,
summed in float64 by the device.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, List, Optional, Sequence, Tuple

import numpy as np

from .grid import AXIS_NAMES, Grid, Unsupported
from .sources import loop_weight

ELECTRIC = ("Ex", "Ey", "Ez")
MAGNETIC = ("Hx", "Hy", "Hz")
COMPONENTS = ELECTRIC + MAGNETIC

# Per-monitor accumulator budget (the reference caps each monitor at 4 GiB, dft.py:125).
ACCUMULATOR_BUDGET_BYTES = 4 * 1024 ** 3


def normalize_frequencies(frequencies: Any = None, frequency: Any = None, fcen: Optional[float] = None,
                          df: Optional[float] = None, nfreq: Optional[int] = None) -> Tuple[float, ...]:
    """Monitor frequencies from any of the reference's spellings (``meep_frequency_span`` :137)."""
    given = [x for x in (frequencies, frequency) if x is not None]
    if fcen is not None:
        if given:
            raise ValueError("give either frequencies or fcen/df/nfreq, not both")
        count = int(nfreq if nfreq is not None else 1)
        if count < 1 or count != (nfreq if nfreq is not None else 1):
            raise ValueError(f"nfreq must be a positive whole number, got {nfreq!r}")
        width = float(df if df is not None else 0.0)
        if not math.isfinite(width) or width < 0:
            raise ValueError(f"df must be finite and >= 0, got {df!r}")
        if count == 1:
            values = [float(fcen)]
        else:
            values = list(np.linspace(float(fcen) - 0.5 * width, float(fcen) + 0.5 * width, count))
    else:
        if not given:
            raise ValueError("a monitor needs frequencies (or fcen/df/nfreq)")
        if len(given) == 2 and tuple(np.atleast_1d(given[0])) != tuple(np.atleast_1d(given[1])):
            raise ValueError("frequency and frequencies disagree")
        values = [float(v) for v in np.atleast_1d(given[0])]
    if not values or any(not math.isfinite(v) for v in values):
        raise ValueError(f"monitor frequencies must be finite, got {values!r}")
    return tuple(float(v) for v in values)


def weight_ladder(where_min: float, where_max: float, resolution: float, parity: int = 1):
    """Doubled-coordinate ladder bounds and Simpson tapers of one axis (MEEP loop_in_chunks)."""
    a = resolution
    yee_c = (1 - parity) * 0.5 / a
    is_doubled = 1 + 2 * math.floor((where_min + yee_c) * a - 0.5) - (1 - parity)
    ie_doubled = 1 + 2 * math.ceil((where_max + yee_c) * a - 0.5) - (1 - parity)
    w0 = 1.0 - where_min * a + 0.5 * is_doubled
    w1 = 1.0 + where_max * a - 0.5 * ie_doubled
    num_doubled = ie_doubled - is_doubled
    if num_doubled >= 3 * 2:
        taper = (w0 * w0 / 2, 1 - (1 - w0) * (1 - w0) / 2, w1 * w1 / 2, 1 - (1 - w1) * (1 - w1) / 2)
    elif num_doubled == 2 * 2:
        s1 = 1 - (1 - w0) * (1 - w0) / 2 - (1 - w1) * (1 - w1) / 2
        taper = (w0 * w0 / 2, s1, w1 * w1 / 2, s1)
    elif where_min == where_max:
        taper = (w0, w1, w1, w0)
    elif num_doubled == 1 * 2:
        s0 = w0 * w0 / 2 - (1 - w1) * (1 - w1) / 2
        e0 = w1 * w1 / 2 - (1 - w0) * (1 - w0) / 2
        taper = (s0, e0, e0, s0)
    else:
        taper = (1.0, 1.0, 1.0, 1.0)
    return is_doubled, ie_doubled, taper


def axis_ladder(grid: Grid, axis: int, where_min: float, where_max: float):
    """(first stored cell, cell count, tapers) of one axis's centred ladder."""
    is_doubled, ie_doubled, taper = weight_ladder(where_min, where_max, grid.resolution)
    count = (ie_doubled - is_doubled) // 2 + 1
    first = int(round((is_doubled - grid.origin_doubled(axis) - 1) / 2.0))
    return first, count, taper


def folded_site(grid: Grid, axis: int, parity: int, site: int):
    """Where a monitor reads site ``site`` (stored-index convention, doubled coordinate
    ``-2 + 2*site + parity``) of a component with Yee shift ``parity`` on a folded axis
    (reference ``dft.py:1004`` ``folded_axis_sites``, MEEP's sn loop): ``(row, flipped)``
    -- a stored row, read with the component's parity when flipped -- or ``"zero"`` (a
    metallic wall) or None (no chunk serves it). The device sampling maps sites the same
    way."""
    full = grid.shape_full[axis]
    stored = grid.shape[axis]
    metallic = grid.is_metallic(axis)
    low = -(full - full % 2)
    lattice = 2 * full
    doubled = -2 + 2 * site + parity
    flipped = False
    if doubled < low + 2 - parity or doubled > low + lattice - parity:
        if metallic:
            return "zero" if parity == 0 and doubled == low else None
        doubled += lattice if doubled < low + 2 - parity else -lattice
        if doubled < low + 2 - parity or doubled > low + lattice - parity:
            return None
    if doubled < -parity:
        doubled = -doubled
        flipped = True
    row = (doubled + 2 - parity) // 2
    if row >= stored:
        if metallic:
            return "zero" if parity == 0 and row == stored else None
        doubled = lattice - doubled  # the second mirror at doubled n_full
        flipped = not flipped
        row = (doubled + 2 - parity) // 2
        if not 0 <= row < stored:
            return None
    return row, flipped


def volume_bounds(center: Sequence[float], size: Sequence[float], what: str):
    center = tuple(float(v) for v in center)
    size = tuple(float(v) for v in size)
    if len(center) != 3 or len(size) != 3:
        raise ValueError(f"{what} needs a three-component center and size")
    if any(not math.isfinite(v) for v in center) or any(not math.isfinite(v) or v < 0 for v in size):
        raise ValueError(f"{what} needs a finite center and a finite, non-negative size")
    return tuple((center[d] - size[d] / 2, center[d] + size[d] / 2) for d in range(3))


def register_volume(grid: Grid, center: Sequence[float], size: Sequence[float], what: str):
    """Half-open stored-index region ``(x0, x1, y0, y1, z0, z1)`` a monitor volume covers.

    Non-wrapping axes clamp the ladder to the stored grid, a folded one to the unfolded
    cell (its sites below the plane are read from their mirror images, with the
    component's parity, by the device sampling). On a wrapping axis the
    ladder is kept whole even where it reaches past a face: its cells past the face
    sample the lattice images of stored cells (MEEP's lattice-shift gather,
    ``loop_in_chunks``; reference ``dft.py:927`` ``_lattice_gather``), which the device
    sampling folds back, with the Bloch factor on a phased axis.
    """
    bounds = volume_bounds(center, size, what)
    region: List[int] = []
    for axis in range(3):
        first, count, _ = axis_ladder(grid, axis, *bounds[axis])
        n = grid.shape[axis]
        if grid.axis_wraps(axis):
            if first < -n or first + count > 2 * n:
                raise Unsupported(f"{what} reaches more than one period past the {AXIS_NAMES[axis]} face")
            region += [first, first + count]
            continue
        if grid.is_mirrored(axis):
            # a folded axis serves the sites below the plane from their images (reference
            # dft.py:1004 folded_axis_sites): the region keeps the ladder's cell-centre
            # sites some chunk serves, which may start below the stored cells
            served = [r for r in range(first, first + count) if folded_site(grid, axis, 1, r) is not None]
            if not served:
                raise ValueError(f"{what} lies outside the cell on the {AXIS_NAMES[axis]} axis")
            if served[-1] - served[0] + 1 != len(served):
                raise RuntimeError(f"{what}: the served sites of the folded {AXIS_NAMES[axis]} axis "
                                   "are not one interval")
            region += [served[0], served[-1] + 1]
            continue
        lo, hi = max(first, 0), min(first + count, n)
        if hi <= lo:
            raise ValueError(f"{what} lies outside the cell on the {AXIS_NAMES[axis]} axis")
        region += [lo, hi]
    return tuple(region)


def axis_weights(grid: Grid, axis: int, where_min: float, where_max: float, start: int,
                 count: int) -> np.ndarray:
    """Float32 taper weight of every region cell along one axis (0 outside the ladder)."""
    first, ladder_count, (s0, s1, e0, e1) = axis_ladder(grid, axis, where_min, where_max)
    weights = np.zeros(count, dtype=np.float32)
    for index in range(ladder_count):
        cell = first + index - start
        if 0 <= cell < count:
            weights[cell] = loop_weight(index, ladder_count, s0, s1, e0, e1)
    return weights


class _Monitor:
    """Shared state of a DFT accumulator: frequencies, decimation, region, device buffer."""

    kind = "dft"

    def __init__(self, grid: Grid, frequencies: Tuple[float, ...], decimation: int):
        self.grid = grid
        self.frequencies = tuple(frequencies)
        self.decimation_factor = int(decimation)
        self.region: Optional[Tuple[int, ...]] = None
        self.components: Tuple[str, ...] = ()
        self.accumulator = None  # device tensor [ncomp][nfreq][2][cells], float32
        self._engine = None

    @property
    def num_frequencies(self) -> int:
        return len(self.frequencies)

    @property
    def omegas(self) -> np.ndarray:
        return 2 * np.pi * np.asarray(self.frequencies, dtype=np.float64)

    @property
    def scale(self) -> float:
        return self.grid.dt * self.decimation_factor / math.sqrt(2 * math.pi)

    @property
    def region_shape(self) -> Tuple[int, int, int]:
        x0, x1, y0, y1, z0, z1 = self.region
        return (x1 - x0, y1 - y0, z1 - z0)

    @property
    def cells(self) -> int:
        return int(np.prod(self.region_shape))

    def _configure_decimation(self, factor: int) -> None:
        if self._engine is not None:
            raise RuntimeError("cannot change a monitor's decimation after accumulation started")
        self.decimation_factor = int(factor)

    def _check_budget(self) -> None:
        size = self.cells * self.num_frequencies * len(self.components) * 8
        if size > ACCUMULATOR_BUDGET_BYTES:
            raise ValueError(f"monitor accumulators need {size} bytes, above the 4 GiB budget")

    def raw(self, component: str) -> np.ndarray:
        """Complex64 host copy of one component's accumulator, shape ``(nf,) + region``."""
        if component not in self.components:
            raise ValueError(f"component {component!r} is not monitored ({self.components})")
        if self._engine is None:
            return np.zeros((self.num_frequencies,) + self.region_shape, dtype=np.complex64)
        values = self._engine.read_accumulator(self, self.components.index(component))
        return values.reshape((self.num_frequencies,) + self.region_shape)


class DFTMonitor(_Monitor):
    """Cell-centred DFT of chosen components over a region (reference dft.py:1960)."""

    kind = "dft"

    def __init__(self, grid: Grid, frequencies, components: Sequence[str], decimation: int):
        super().__init__(grid, frequencies, decimation)
        for c in components:
            if c not in COMPONENTS:
                raise Unsupported(f"DFT component {c!r} is not stepped (E and H components only)")
        self.components = tuple(components)

    def set_region_from_volume(self, center, size) -> None:
        self.region = register_volume(self.grid, center, size, "DFT region")
        self._check_budget()

    def set_region(self, region: Sequence[int]) -> None:
        region = tuple(int(v) for v in region)
        for axis in range(3):
            if not 0 <= region[2 * axis] < region[2 * axis + 1] <= self.grid.shape[axis]:
                raise ValueError(f"DFT region {region} is not inside the grid")
        self.region = region
        self._check_budget()

    def get_dft(self, component: str, freq_index: int = 0) -> np.ndarray:
        return self.raw(component)[freq_index]


@dataclass(frozen=True)
class FluxPlaneDft:
    """One flux plane's accumulated E and H transforms, host copies detached from the run
    (reference ``dft.py:2618``): ``{"Ex"/"Ey"/"Ez": (nf,) + region complex64}`` and the
    same for H."""

    E: dict
    H: dict
    frequencies: tuple


@dataclass(frozen=True)
class FluxDftData:
    """What a flux monitor's ``get_dft_data()`` returns (reference ``dft.py:2638``,
    MEEP's ``sim.get_flux_data``): one :class:`FluxPlaneDft` per plane, to be handed to
    ``load_dft_data`` / ``load_minus_dft_data`` of a monitor built the same way."""

    planes: tuple


class FluxMonitor(_Monitor):
    """Poynting flux through an axis-aligned plane (reference dft.py:2814).

    Only the tangential pair of E and of H is accumulated: the normal components
    never enter the flux. In the saved transforms (:meth:`get_dft_data`) they are
    zero, and loading ignores them.
    """

    kind = "flux"

    def __init__(self, grid: Grid, frequencies, center, size, direction: Optional[int],
                 weight: float, decimation: int):
        super().__init__(grid, frequencies, decimation)
        self.center = tuple(float(v) for v in center)
        self.size = tuple(float(v) for v in size)
        if direction is None:
            if self.size[0] == 0 or self.size[0] < grid.dx:
                direction = 0
            elif self.size[1] == 0 or self.size[1] < grid.dx:
                direction = 1
            else:
                direction = 2
        if direction not in (0, 1, 2):
            raise ValueError(f"flux direction must be 0, 1 or 2, got {direction!r}")
        self.direction = int(direction)
        self.weight = float(weight)
        a, b = (self.direction + 1) % 3, (self.direction + 2) % 3
        self.components = (ELECTRIC[a], ELECTRIC[b], MAGNETIC[a], MAGNETIC[b])
        self.region = register_volume(grid, self.center, self.size, "flux plane")
        starts = self.region[0::2]
        counts = self.region_shape
        bounds = volume_bounds(self.center, self.size, "flux plane")
        per_axis = [axis_weights(grid, d, bounds[d][0], bounds[d][1], starts[d], counts[d])
                    for d in range(3)]
        self.weights = (per_axis[0][:, None, None] * per_axis[1][None, :, None]
                        * per_axis[2][None, None, :]).astype(np.float32)
        self.measure = grid.dx ** sum(1 for extent in self.size if extent > 0)
        self._check_budget()

    def get_flux_spectrum(self) -> np.ndarray:
        if self._engine is None:
            return np.zeros(self.num_frequencies)
        return self._engine.flux_spectrum(self)

    def get_flux(self, freq_index: int = 0) -> float:
        return float(self.get_flux_spectrum()[freq_index])

    # --- saved transforms: the two-run normalisation idiom ----------------------------
    def _shape(self) -> Tuple[int, ...]:
        return (self.num_frequencies,) + self.region_shape

    def _tangential(self) -> dict:
        """The accumulated tangential transforms (complex64, ``(nf,) + region``)."""
        if self._engine is not None:
            return {name: self.raw(name) for name in self.components}
        pending = getattr(self, "_pending", None)
        if pending is not None:
            return {name: pending[name].copy() for name in self.components}
        return {name: np.zeros(self._shape(), dtype=np.complex64) for name in self.components}

    def get_dft_data(self) -> FluxDftData:
        """This plane's accumulated transforms (reference ``FluxMonitor.get_dft_data``
        :3261, MEEP's ``sim.get_flux_data``), as host copies."""
        blocks = self._tangential()
        full = {name: blocks.get(name, np.zeros(self._shape(), dtype=np.complex64)) for name in COMPONENTS}
        return FluxDftData(planes=(FluxPlaneDft(E={n: full[n] for n in ELECTRIC},
                                                H={n: full[n] for n in MAGNETIC},
                                                frequencies=tuple(self.frequencies)),))

    def load_dft_data(self, data: FluxDftData) -> None:
        """Replace this plane's transforms with ``data`` (MEEP's ``load_flux_data``: the
        stored words are replaced, not added to). Checked as the reference checks it
        (``dft.py:2660`` ``_load_flux_planes``): one plane, the same frequencies, all six
        components, each block of this plane's shape; a refusal changes nothing."""
        where = "FluxMonitor.load_dft_data"
        if not isinstance(data, FluxDftData):
            raise TypeError(f"{where} takes the object a flux monitor's get_dft_data() returned "
                            f"(FluxDftData), got {type(data).__name__}")
        if len(data.planes) != 1:
            raise ValueError(f"{where} was given data for {len(data.planes)} flux plane(s) but this "
                             f"monitor has 1")
        record = data.planes[0]
        if len(record.frequencies) != self.num_frequencies:
            raise ValueError(f"{where}: the data holds {len(record.frequencies)} frequencies and this "
                             f"monitor accumulates {self.num_frequencies}")
        for saved, mine in zip(record.frequencies, self.frequencies):
            if not math.isclose(float(saved), float(mine), rel_tol=1e-12, abs_tol=0.0):
                raise ValueError(f"{where}: the data was accumulated at frequencies {record.frequencies} "
                                 f"and this monitor accumulates {self.frequencies}")
        for side, names, block in (("E", ELECTRIC, record.E), ("H", MAGNETIC, record.H)):
            if set(block) != set(names):
                raise ValueError(f"{where}: the data's {side} components are {sorted(block)}, "
                                 f"expected {sorted(names)}")
            for name in names:
                if np.asarray(block[name]).shape != self._shape():
                    raise ValueError(f"{where}: {name} in the data has shape {np.asarray(block[name]).shape} "
                                     f"and this monitor's plane is {self._shape()}")
        incoming = {}
        for name in self.components:
            block = record.E[name] if name in record.E else record.H[name]
            incoming[name] = np.ascontiguousarray(np.asarray(block), dtype=np.complex64)
        if self._engine is None:
            self._pending = incoming  # written into the accumulators when the run freezes
            return
        self._write(incoming)

    def _write(self, blocks: dict) -> None:
        for q, name in enumerate(self.components):
            self._engine.write_accumulator(self, q, blocks[name].reshape(self.num_frequencies, self.cells))

    def scale_dfts(self, scale: complex) -> None:
        """Multiply every accumulated transform by ``scale`` (``dft_flux::scale_dfts``:
        both the E and the H side)."""
        factor = complex(scale)
        blocks = self._tangential()
        scaled = {name: (block * factor).astype(np.complex64) for name, block in blocks.items()}
        if self._engine is None:
            self._pending = scaled
            return
        self._write(scaled)

    def load_minus_dft_data(self, data: FluxDftData) -> None:
        """``load_dft_data`` then negate (MEEP's ``load_minus_flux_data``): the second
        run's accumulators start at -E1, -H1, so its flux is that of the field
        difference, ``Re[(E2 - E1) x conj(H2 - H1)]``."""
        self.load_dft_data(data)
        self.scale_dfts(-1.0)

    def reset(self) -> None:
        """Zero every accumulator (buffered samples included)."""
        self._pending = None
        if self._engine is not None:
            for q in range(len(self.components)):
                self._engine.write_accumulator(self, q, None)


def automatic_decimation(dt: float, monitor_frequencies: Sequence[float], sources) -> int:
    """MEEP's ``decimation_factor == 0``: ``floor(1/(dt*(f_mon_max + f_src_max)))`` (driver.py:3101)."""
    source_max = 0.0
    for source in sources:
        band = getattr(source.waveform, "bandwidth_max", None)
        if band is None:
            continue
        source_max = max(source_max, band)
    monitor_max = max((abs(float(f)) for f in monitor_frequencies), default=0.0)
    if monitor_max <= 0.0 or source_max <= 0.0:
        return 1
    return max(1, int(math.floor(1.0 / (dt * (monitor_max + source_max)))))


def absorbing_cells(cells: float) -> int:
    """Whole cells one PML face grades: ``ceil(half_cell_extent / 2)``."""
    from .pml import half_cell_extent
    return (half_cell_extent(cells) + 1) // 2
