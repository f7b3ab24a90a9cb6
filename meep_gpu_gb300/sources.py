"""Electric current sources: MEEP's waveforms, deposition tables and per-step deposit words.

Waveforms follow the reference's ``meep_gpu/sources.py``: the Gaussian dipole
(``_gaussian_dipole`` :615, hard cut at ``_gaussian_cutoff_time`` :603), the CW dipole
(``_continuous_dipole`` :580), the amplitude factor ``1/(-2*pi*i*f)`` (``_amp_factor``
:177) and the current as a forward difference of the dipole (``_forward_difference``
:1765). The deposition table (which cells, which complex amplitude) restates MEEP's
``add_volume_source`` / ``loop_in_chunks`` weight ladder as the reference transcribes it
(``_source_geometry`` :787, ``_compute_boundary_weights`` :654, ``_ivec_loop_weight_1d``
:698, ``_src_vol_pieces`` :1061) for one chunk and a zero Bloch vector.

The deposit itself is MEEP's ``f -= real(amp * current) * dt`` in double on a float32
word (``_deposit`` :1357, ``host_writes.subtract_double`` :140). The host forms, for
every step and table point, the float64 subtrahend ``((amp_re*c_re) - (amp_im*c_im))*dt``
with every product rounded on its own (written out per part, so no platform contracts
it), and the device kernel performs ``float(double(D) - A)``. A current that is bitwise
``(+0, +0)`` deposits ``+0``, which leaves every float32 word unchanged, as the
reference's early return does.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .grid import AXIS_NAMES, IYEE, Grid, Unsupported, cmul, cpow_int

ELECTRIC = ("Ex", "Ey", "Ez")
MAGNETIC = ("Hx", "Hy", "Hz")
_COMPONENT_ALIASES = {"Ex": "Ex", "Ey": "Ey", "Ez": "Ez", "Dx": "Ex", "Dy": "Ey", "Dz": "Ez",
                      "Hx": "Hx", "Hy": "Hy", "Hz": "Hz", "Bx": "Hx", "By": "Hy", "Bz": "Hz"}


def amp_factor(frequency: float) -> Tuple[float, float]:
    """``1/(-2*pi*i*f)`` as CPython's complex division evaluates it: ``(-0.0, 1/(2*pi*f))``."""
    if not math.isfinite(frequency) or frequency == 0.0:
        raise ValueError(f"source frequency must be finite and nonzero, got {frequency!r}")
    denominator = (-2.0 * np.pi) * frequency
    return (-0.0 if frequency > 0 else 0.0, (-1.0) / denominator)


def _cmul(a: Tuple[float, float], b: Tuple[float, float]) -> Tuple[float, float]:
    """Complex product with every product rounded on its own: ``(ac - bd, ad + bc)``."""
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def _carrier(omega: float, t: float) -> Tuple[float, float]:
    value = complex(np.exp(-1j * omega * t))
    return (value.real, value.imag)


def gaussian_cutoff_time(cutoff: float, width: float) -> float:
    """MEEP shrinks the hard cut until the envelope is representable, rounded to float32."""
    cutoff_time = cutoff * width
    while math.exp(-cutoff_time * cutoff_time / (2 * width * width)) < 1e-100:
        cutoff_time *= 0.9
    return float(np.float32(cutoff_time))


@dataclass
class GaussianWaveform:
    """MEEP ``gaussian_src_time``: a Gaussian envelope about ``start + cutoff/fwidth``."""

    frequency: float
    fwidth: float
    start_time: float = 0.0
    cutoff: float = 5.0

    def __post_init__(self):
        if not (self.fwidth > 0 and math.isfinite(self.fwidth)):
            raise ValueError(f"fwidth must be positive, got {self.fwidth!r}")
        self.omega = 2 * np.pi * self.frequency
        self.amp = amp_factor(self.frequency)
        self.width = 1.0 / self.fwidth
        self.peak_time = self.start_time + self.cutoff * self.width
        self.cutoff_time = gaussian_cutoff_time(self.cutoff, self.width)

    @property
    def bandwidth_max(self) -> float:
        """``|f| + fwidth/2``, what MEEP's automatic DFT decimation reads."""
        return abs(float(self.frequency)) + 0.5 * float(self.fwidth)

    def dipole(self, t: float) -> Tuple[float, float]:
        t_rel = t - self.peak_time
        if np.float32(abs(t_rel)) > self.cutoff_time:
            return (0.0, 0.0)
        envelope = math.exp(-t_rel * t_rel / (2 * self.width * self.width))
        phase = _carrier(self.omega, t_rel)
        scaled = _cmul(phase, (envelope, 0.0))
        return _cmul(scaled, self.amp)


@dataclass
class ContinuousWaveform:
    """MEEP ``continuous_src_time``: a CW carrier with an optional tanh turn-on/off."""

    frequency: float
    start_time: float = 0.0
    end_time: float = 1e20
    width: float = 0.0
    slowness: float = 3.0

    def __post_init__(self):
        self.omega = 2 * np.pi * self.frequency
        self.amp = amp_factor(self.frequency)

    bandwidth_max = None

    def dipole(self, t: float) -> Tuple[float, float]:
        rtime = np.float32(t)
        if rtime < np.float32(self.start_time) or rtime > np.float32(self.end_time):
            return (0.0, 0.0)
        carrier = _carrier(self.omega, t)
        value = _cmul(carrier, self.amp)
        if self.width == 0.0:
            return value
        ts = (t - self.start_time) / self.width - self.slowness
        te = (self.end_time - t) / self.width - self.slowness
        ramp = (1.0 + math.tanh(ts)) * (1.0 + math.tanh(te)) * 0.25
        return _cmul(value, (ramp, 0.0))


@dataclass
class CustomWaveform:
    """MEEP ``custom_src_time``: the caller's ``func(t) -> complex`` inside a float32 window."""

    func: Callable[[float], complex]
    start_time: float = -1e20
    end_time: float = 1e20
    bandwidth_max = None

    def dipole(self, t: float) -> Tuple[float, float]:
        rtime = np.float32(t)
        if rtime < np.float32(self.start_time) or rtime > np.float32(self.end_time):
            return (0.0, 0.0)
        value = complex(self.func(t))
        return (value.real, value.imag)


def current(waveform, t: float, dt: float) -> Tuple[float, float]:
    """MEEP ``src_time::current``: ``(dipole(t + dt) - dipole(t)) / dt`` per part."""
    late = waveform.dipole(t + dt)
    early = waveform.dipole(t)
    return ((late[0] - early[0]) / dt, (late[1] - early[1]) / dt)


# --- deposition table -------------------------------------------------------------------

def vec2diel_floor(pt: float, a: float) -> int:
    return 1 + 2 * int(np.floor(pt * a - 0.5))


def vec2diel_ceil(pt: float, a: float) -> int:
    return 1 + 2 * int(np.ceil(pt * a - 0.5))


def boundary_weights(where_min: float, where_max: float, is_d: int, ie_d: int,
                     a: float) -> Tuple[float, float, float, float]:
    """MEEP ``compute_boundary_weights``: Simpson tapers ``(s0, s1, e0, e1)``; case order matters."""
    w0 = 1.0 - where_min * a + 0.5 * is_d
    w1 = 1.0 + where_max * a - 0.5 * ie_d
    num_doubled = ie_d - is_d
    if num_doubled >= 3 * 2:
        return (w0 * w0 / 2, 1 - (1 - w0) * (1 - w0) / 2, w1 * w1 / 2, 1 - (1 - w1) * (1 - w1) / 2)
    if num_doubled == 2 * 2:
        s1 = 1 - (1 - w0) * (1 - w0) / 2 - (1 - w1) * (1 - w1) / 2
        return (w0 * w0 / 2, s1, w1 * w1 / 2, s1)
    if where_min == where_max:
        return (w0, w1, w1, w0)
    if num_doubled == 1 * 2:
        s0 = w0 * w0 / 2 - (1 - w1) * (1 - w1) / 2
        e0 = w1 * w1 / 2 - (1 - w0) * (1 - w0) / 2
        return (s0, e0, e0, s0)
    return (1.0, 1.0, 1.0, 1.0)


def loop_weight(i: int, n: int, s0: float, s1: float, e0: float, e1: float) -> float:
    """MEEP ``IVEC_LOOP_WEIGHT1x``: weight of position ``i`` in a run of ``n``."""
    if 1 < i < n - 2:
        return 1.0
    if i == 0:
        return s0
    if i == 1:
        return s1
    if i == n - 1:
        return e0
    if i == n - 2:
        return e1
    return 1.0


def _chunk_weights(start: int, end: int, is_d: int, ie_d: int, taper) -> Tuple[float, float, float, float]:
    """The end weights of a clipped run ``[start, end]`` (source-frame doubled ends): the
    request's tapers where the run meets the request's ends, 1 elsewhere, and the
    narrow-range minima (MEEP's ``loop_in_chunks``)."""
    s0, s1, e0, e1 = taper
    ws0 = ws1 = we0 = we1 = 1.0
    if start == is_d:
        ws0, ws1 = s0, s1
    elif start == is_d + 2:
        ws0 = s1
    if end == ie_d:
        we0, we1 = e0, e1
    elif end == ie_d - 2:
        we0 = e1
    if end == start:
        w = min(ws0, we0)
        ws0 = we0 = ws1 = we1 = w
    elif end == start + 2:
        w = min(ws0, we1)
        ws0 = we1 = w
        w = min(ws1, we0)
        ws1 = we0 = w
    elif end == start + 4:
        w = min(ws1, we1)
        ws1 = we1 = w
    return ws0, ws1, we0, we1


def chunk_boxes(grid: Grid, faces) -> List[Tuple[Tuple[int, int, int], Tuple[int, int, int]]]:
    """The one-rank chunk boxes (doubled corners): per axis the low PML piece, the interior
    and the high PML piece, x outermost (reference ``chunk_map.py:384``); one box
    spanning the window without a PML."""
    from .conductivity import axis_pieces
    per_axis = []
    for d in range(3):
        io = grid.origin_doubled(d)
        # MEEP's window is owned cells long (a folded periodic axis stores one more)
        pieces = axis_pieces(grid.owned_cells(d), faces[d] if faces is not None else (0.0, 0.0))
        per_axis.append([(io + lo, io + hi) for _piece, lo, hi in pieces])
    return [((bx[0], by[0], bz[0]), (bx[1], by[1], bz[1]))
            for bx in per_axis[0] for by in per_axis[1] for bz in per_axis[2]]


def deposition_pieces(grid: Grid, component: str, center: Sequence[float], size: Sequence[float],
                      amplitude: complex = 1.0,
                      amp_func: Optional[Callable[[float, float, float], complex]] = None,
                      boxes=None) -> List[Tuple[int, List[Tuple[int, int, int]], List[complex]]]:
    """MEEP's ``src_vol`` pieces of one source, in ``add_volume_source`` order:
    ``(chunk, cells, amplitudes)`` per (lattice shift, chunk) (reference ``sources.py:1061``
    ``_src_vol_pieces``, :787 ``_source_geometry``).

    The request's doubled-coordinate bounds on the component's lattice, the Simpson
    tapers of the request, the owned window ``[origin + 2 - iyee, origin + 2n - iyee]``
    (the plane on a metallic high wall takes no deposit), one pass per lattice shift on
    a periodic axis (with ``amp * conj(ph)``, ``ph`` the product of ``eikna^shift`` on a
    Bloch-phased run), the amplitude ``amplitude * a`` per zero-extent axis, and per
    chunk the pass clipped to the chunk's owned corners with its own end weights.
    ``boxes``: the chunk boxes (:func:`chunk_boxes`), or None for one box spanning the
    window.
    """
    comp = _COMPONENT_ALIASES.get(component)
    if comp is None:
        raise Unsupported(f"source component {component!r} is not one of Ex..Ez, Hx..Hz")
    a = grid.resolution
    inva = grid.dx
    # the axes MEEP's loops carry: an invariant one (z of a 2-D run) is one point of
    # weight 1 at stored cell 0, with no bounds, tapers, lattice shifts or amplitude scale
    directions = grid.directions
    resolved = [d in directions for d in range(3)]
    where_min = [float(center[d]) - float(size[d]) / 2 for d in range(3)]
    where_max = [float(center[d]) + float(size[d]) / 2 for d in range(3)]
    lengths = tuple(n * grid.dx for n in grid.shape_full)  # the snapped cell (reference Grid.Lx/Ly/Lz)
    for d in directions:
        span = where_max[d] - where_min[d]
        if span > lengths[d] + inva:
            raise ValueError(f"source size {size[d]} exceeds the cell length {lengths[d]} by more than one cell")
        if span > lengths[d]:
            excess = span - lengths[d]
            where_min[d] = where_min[d] - excess * 0.5
            where_max[d] = where_min[d] + lengths[d]
    # amp * a per zero-extent carried direction, except a one-cell periodic one (MEEP's
    # nosize_direction: a zero extent there means the whole direction)
    amp = (float(complex(amplitude).real), float(complex(amplitude).imag))
    for d in directions:
        if where_max[d] - where_min[d] == 0.0 and not grid.nosize_direction(d):
            amp = (amp[0] * a, amp[1] * a)
    iyee = IYEE[comp]
    iyee_c = [1 - iyee[d] for d in range(3)]
    is_ = [0, 0, 0]
    ie = [0, 0, 0]
    tapers = [(1.0, 1.0, 1.0, 1.0)] * 3
    for d in directions:
        yee_c = iyee_c[d] * 0.5 * inva
        is_[d] = vec2diel_floor(where_min[d] + yee_c, a) - iyee_c[d]
        ie[d] = vec2diel_ceil(where_max[d] + yee_c, a) - iyee_c[d]
        tapers[d] = boundary_weights(where_min[d], where_max[d], is_[d], ie[d], a)
    io = [grid.origin_doubled(d) for d in range(3)]
    counts = grid.shape
    # the window top is MEEP's big corner, owned cells up: a folded periodic axis's far
    # ghost slot is never deposited into
    big = [io[d] + 2 * grid.owned_cells(d) for d in range(3)]
    window_low = [io[d] + 2 - iyee[d] for d in range(3)]
    window_high = [big[d] - iyee[d] for d in range(3)]
    if boxes is None:
        boxes = [((io[0], io[1], io[2]), (big[0], big[1], big[2]))]
    wraps = [grid.axis_wraps(d) for d in range(3)]
    # MEEP loops lattice shifts on every axis with a periodic outer face, a folded one
    # included (its second mirror is a lattice image; reference sources.py:925), by the
    # full cell's lattice vector
    periodic = [resolved[d] and (wraps[d] or (grid.is_mirrored(d) and not grid.is_metallic(d)))
                for d in range(3)]
    half_inva = 0.5 * inva
    min_shift = [0, 0, 0]
    max_shift = [0, 0, 0]
    period = [0, 0, 0]
    for d in range(3):
        if not periodic[d]:
            continue
        period[d] = 2 * grid.shape_full[d]
        lattice = abs(period[d] * half_inva)
        min_shift[d] = int(math.floor((where_min[d] - big[d] * half_inva) / lattice))
        max_shift[d] = int(math.ceil((where_max[d] - io[d] * half_inva) / lattice))
    centre = [(where_min[d] + where_max[d]) * 0.5 for d in range(3)]

    pieces: List[Tuple[int, List[Tuple[int, int, int]], List[complex]]] = []
    shift = list(min_shift)
    while True:
        shifted = [period[d] * shift[d] for d in range(3)]
        # a pass one lattice vector away on a Bloch-phased axis carries amp * conj(ph),
        # ph the product of eikna^shift over the axes (MEEP's loop_in_chunks)
        pass_amp = amp
        if grid.has_bloch:
            ph = (1.0, 0.0)
            for d in range(3):
                ph = cmul(ph, cpow_int(grid.eikna(d), shift[d]))
            pass_amp = cmul(amp, (ph[0], -ph[1]))
        ranges = []
        for d in range(3):
            if not resolved[d]:
                ranges.append([None])
                continue
            low = max(is_[d] - shifted[d], window_low[d])
            high = min(ie[d] - shifted[d], window_high[d])
            ranges.append(list(range(low, high + 1, 2)) if low <= high else [])
        points = []
        if all(ranges):
            for px in ranges[0]:
                for py in ranges[1]:
                    for pz in ranges[2]:
                        coords = (px, py, pz)
                        cell = []
                        inert = False
                        rel = []
                        for d in range(3):
                            if not resolved[d]:
                                # an amplitude function is handed 0 on an axis the run
                                # does not carry (MEEP's vec2py)
                                rel.append(0.0)
                                cell.append(0)
                                continue
                            loc = (0.5 * coords[d]) * inva + shifted[d] * half_inva
                            rel.append(loc - centre[d])
                            ladder = (coords[d] - io[d]) // 2
                            if wraps[d]:
                                cell.append(ladder % counts[d])
                            elif ladder >= counts[d]:
                                inert = True
                                cell.append(-1)
                            else:
                                cell.append(ladder)
                        if amp_func is None:
                            value = (1.0, 0.0)
                        else:
                            result = complex(amp_func(rel[0], rel[1], rel[2]))
                            value = (result.real, result.imag)
                        points.append((coords, None if inert else tuple(cell), value))
        for chunk, (lo, hi) in enumerate(boxes if points else ()):
            isc = [0, 0, 0]
            iec = [0, 0, 0]
            weights = []
            empty = False
            for d in range(3):
                if not resolved[d]:
                    weights.append(None)
                    continue
                isc[d] = max(is_[d] - shifted[d], window_low[d], lo[d] + 2 - iyee[d])
                iec[d] = min(ie[d] - shifted[d], hi[d] - iyee[d])
                if isc[d] > iec[d]:
                    empty = True
                    break
                ends = _chunk_weights(isc[d] + shifted[d], iec[d] + shifted[d], is_[d], ie[d], tapers[d])
                weights.append(ends + ((iec[d] - isc[d]) // 2 + 1,))
            if empty:
                continue
            cells: List[Tuple[int, int, int]] = []
            amps: List[complex] = []
            for coords, cell, value in points:
                if any(not isc[d] <= coords[d] <= iec[d] for d in directions):
                    continue
                factors = []
                for d in range(3):
                    if weights[d] is None:
                        factors.append(1.0)
                        continue
                    ws0, ws1, we0, we1, n = weights[d]
                    factors.append(loop_weight((coords[d] - isc[d]) // 2, n, ws0, ws1, we0, we1))
                weight = factors[2] * (factors[1] * (1.0 * factors[0]))
                if cell is None:
                    continue
                scaled = (weight * pass_amp[0], weight * pass_amp[1])
                product = _cmul(scaled, value)
                cells.append(cell)
                amps.append(complex(product[0], product[1]))
            if cells:
                pieces.append((chunk, cells, amps))
        for d in range(3):
            if shift[d] + 1 <= max_shift[d]:
                shift[d] += 1
                break
            shift[d] = min_shift[d]
        else:
            break
    return pieces


def deposition_table(grid: Grid, component: str, center: Sequence[float], size: Sequence[float],
                     amplitude: complex = 1.0,
                     amp_func: Optional[Callable[[float, float, float], complex]] = None,
                     ) -> Tuple[List[Tuple[int, int, int]], List[complex]]:
    """Every cell a source deposits into (D for an electric one, B for a magnetic one),
    once, with its pieces' amplitudes summed in placement order (one chunk spanning the
    window; reference ``sources.py:1144`` ``_summed_table``)."""
    accumulated: Dict[Tuple[int, int, int], complex] = {}
    for _chunk, cells, amps in deposition_pieces(grid, component, center, size, amplitude, amp_func):
        for cell, value in zip(cells, amps):
            previous = accumulated.get(cell)
            accumulated[cell] = value if previous is None else complex(previous.real + value.real,
                                                                       previous.imag + value.imag)
    cells = list(accumulated)
    return cells, [accumulated[c] for c in cells]


def bind_src_vols(sources: Sequence["Source"], grid: Grid, faces) -> None:
    """Give every source the entries it deposits in MEEP's ``src_vol`` lists (reference
    ``sources.py:1585`` ``bind_src_vols``): one piece per (lattice shift, chunk); a piece
    whose chunk, component, waveform and cells equal an earlier entry's is summed into it
    and deposits once; pieces that share a cell without sharing their cells -- the two
    ends of a request across a periodic seam -- stay two entries, and the cell is
    deposited twice. Each source's ``cells`` / ``amps`` become its entries, in creation
    order.
    """
    boxes = chunk_boxes(grid, faces)
    entries = {}
    owned: Dict[int, List[list]] = {}
    for index, source in enumerate(sources):
        key_time = _waveform_key(source.waveform) or ("object", id(source.waveform))
        for chunk, cells, amps in deposition_pieces(grid, source.component, source.center, source.size,
                                                    source.amplitude, source.amp_func, boxes):
            key = (chunk, source.component, key_time, tuple(cells))
            entry = entries.get(key)
            if entry is None:
                entry = [cells, list(amps)]
                entries[key] = entry
                owned.setdefault(index, []).append(entry)
                continue
            entry[1] = [complex(x.real + y.real, x.imag + y.imag) for x, y in zip(entry[1], amps)]
    for index, source in enumerate(sources):
        mine = owned.get(index, [])
        source.cells = [cell for cells, _ in mine for cell in cells]
        source.amps = [amp for _, amps in mine for amp in amps]


def require_stored_half(grid: Grid, center: Sequence[float]) -> None:
    """A source centre must lie in the half a folded axis stores (reference
    ``sources.py:333``): MEEP deposits with ``use_symmetry=false``, so a source in the
    discarded half reaches no stored cell and the run is silently empty."""
    tol = grid.dx / 10
    for axis in range(3):
        if not grid.is_mirrored(axis) or center[axis] >= -tol:
            continue
        name = AXIS_NAMES[axis]
        raise ValueError(
            f"With {name.upper()} symmetry the stored half is {name} >= 0, and this source is at "
            f"{name}={center[axis]:g}, in the half the fold discards; nothing would be deposited. "
            f"Declare it at {name}={-center[axis]:g} instead: under this plane that is the same "
            f"physical configuration, and its image is supplied by the fold.")


def mirror_parity_offenders(grid: Grid, component: str, center: Sequence[float],
                            size: Sequence[float], has_amp_func: bool) -> list:
    """The planes a source centred on them cannot carry the parity of (reference
    ``sources.py:500``): a component odd about a plane, on it, with no extent across it
    or a uniform profile over it, would deposit a current the fold images with the
    opposite sign. One ``(axis, phase, why)`` per offending plane."""
    from .grid import mirror_parity
    tol = grid.dx / 10
    offenders = []
    for axis in range(3):
        phase = grid.mirror_phase(axis)
        if phase is None or mirror_parity(component, axis, phase) > 0 or abs(center[axis]) > tol:
            continue
        name = AXIS_NAMES[axis]
        if size[axis] <= tol:
            why = (f"it has no extent along {name} (size[{name}]={size[axis]:g}), so the parity "
                   f"condition admits only zero current")
        elif not has_amp_func:
            why = (f"its profile over |{name}| <= {size[axis] / 2:g} is uniform (no amp_func), and a "
                   f"constant is even about every plane")
        else:
            continue
        offenders.append((axis, phase, why))
    return offenders


def mirror_parity_message(component: str, offenders: list) -> str:
    from .grid import mirror_parity
    parts = []
    for axis, phase, why in offenders:
        odd = [n for n in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz") if mirror_parity(n, axis, phase) < 0]
        parts.append(f"the {'even' if phase > 0 else 'odd'} {'XYZ'[axis]} plane (phase {phase:+d}) gives "
                     f"it parity -1 (odd there: {', '.join(odd)}), and {why}")
    return (f"A {component} source centred on the mirror plane cannot carry the parity the fold "
            f"demands: " + "; also ".join(parts) + ". Give it an extent across the plane with an "
            f"amp_func odd about it, drive a component the plane leaves even, declare the opposite "
            f"phase, or run the full domain.")


@dataclass
class Source:
    """One current source: a waveform, a component and a deposition table. An electric
    source deposits into D in the E half at t + dt/2; a magnetic one (Hx, Hy, Hz) into B
    right after step_B, at t (reference ``driver.py:3527-3535``)."""

    grid: Grid
    component: str
    center: Tuple[float, float, float]
    size: Tuple[float, float, float]
    waveform: object
    amplitude: complex = 1.0
    amp_func: Optional[Callable[[float, float, float], complex]] = None
    cells: List[Tuple[int, int, int]] = field(default_factory=list, init=False)
    amps: List[complex] = field(default_factory=list, init=False)

    def __post_init__(self):
        self.component = _COMPONENT_ALIASES.get(self.component, self.component)
        if self.component not in ELECTRIC + MAGNETIC:
            raise Unsupported(f"source component {self.component!r} is not stepped by this engine")
        if self.grid.has_symmetry:
            require_stored_half(self.grid, self.center)
            offenders = mirror_parity_offenders(self.grid, self.component, self.center, self.size,
                                                self.amp_func is not None)
            if offenders:
                raise ValueError(mirror_parity_message(self.component, offenders))
        self.cells, self.amps = deposition_table(self.grid, self.component, self.center,
                                                 self.size, self.amplitude, self.amp_func)

    @property
    def magnetic(self) -> bool:
        return self.component in MAGNETIC

    @property
    def comp_index(self) -> int:
        """0..2 for Dx..Dz, 3..5 for Bx..Bz: the component the deposit writes."""
        return (ELECTRIC + MAGNETIC).index(self.component)

    @property
    def time_offset(self) -> float:
        """The current's time within step n, in steps: n + 1/2 (electric), n (magnetic)."""
        return 0.0 if self.magnetic else 0.5

    def current(self, t: float) -> Tuple[float, float]:
        return current(self.waveform, t, self.grid.dt)


# Current sequences from step 0, per waveform and time step: every simulation of a served
# stream with the same source spectrum and resolution shares one.
_CURRENT_CACHE: Dict[tuple, np.ndarray] = {}
_CURRENT_CACHE_STEPS = 1 << 20


def _waveform_key(waveform) -> Optional[tuple]:
    if isinstance(waveform, GaussianWaveform):
        return ("gaussian", waveform.frequency, waveform.fwidth, waveform.start_time, waveform.cutoff)
    if isinstance(waveform, ContinuousWaveform):
        return ("continuous", waveform.frequency, waveform.start_time, waveform.end_time,
                waveform.width, waveform.slowness)
    return None  # a caller's function may not be pure: never cached


def _currents(waveform, dt: float, first: int, steps: int, offset: float = 0.5) -> np.ndarray:
    out = np.empty((steps, 2), dtype=np.float64)
    for row in range(steps):
        n = first + row
        t = n * dt + 0.5 * dt if offset == 0.5 else n * dt
        out[row] = current(waveform, t, dt)
    return out


def current_sequence(waveform, dt: float, first: int, steps: int, offset: float = 0.5) -> np.ndarray:
    """Currents ``(re, im)`` of steps ``first .. first+steps-1``, evaluated at ``n*dt + dt/2``
    (``offset`` 0.5: MEEP's ``calc_sources(time() + dt/2)`` before the D half) or at
    ``n*dt`` (``offset`` 0: a magnetic source after step_B), shape ``(steps, 2)``."""
    if offset not in (0.0, 0.5):
        raise ValueError("a current is evaluated at n*dt or n*dt + dt/2")
    key = _waveform_key(waveform)
    if key is None or first + steps > _CURRENT_CACHE_STEPS:
        return _currents(waveform, dt, first, steps, offset)
    key = key + (dt, offset)
    table = _CURRENT_CACHE.get(key)
    have = 0 if table is None else len(table)
    if have < first + steps:
        grown = _currents(waveform, dt, have, first + steps - have, offset)
        table = grown if table is None else np.concatenate([table, grown])
        _CURRENT_CACHE[key] = table
    return table[first:first + steps]


def deposit_words(sources: Sequence[Source], first_step: int, steps: int, dt: float,
                  scales: Optional[np.ndarray] = None, part: str = "real") -> np.ndarray:
    """Float64 subtrahends ``A[step][point]`` for steps ``first_step .. first_step+steps-1``.

    ``A = ((amp_re*c_re) - (amp_im*c_im))*dt`` with each product and the difference
    rounded on its own (separate array operations), ``+0`` where the current is bitwise
    ``(+0, +0)``. Points are laid out source by source in table order, the order the
    device deposits them. ``scales`` (one float64 per point) multiplies each word last:
    a lossy target component's ``condinv`` at the point (reference ``sources.py:1357``
    ``_deposit``, MEEP's ``A = current * dt * cndinv[i]``). ``part="imag"`` gives the
    words a complex run subtracts from its imaginary fields,
    ``((amp_re*c_im) + (amp_im*c_re))*dt``.
    """
    if part not in ("real", "imag"):
        raise ValueError("part is 'real' or 'imag'")
    count = sum(len(s.cells) for s in sources)
    out = np.zeros((steps, count), dtype=np.float64)
    column = 0
    for source in sources:
        seq = current_sequence(source.waveform, source.grid.dt, first_step, steps, source.time_offset)
        c_re, c_im = seq[:, 0], seq[:, 1]
        plus_zero = ((c_re == 0.0) & ~np.signbit(c_re)) & ((c_im == 0.0) & ~np.signbit(c_im))
        for amp in source.amps:
            if part == "real":
                value = ((amp.real * c_re) - (amp.imag * c_im)) * dt
            else:
                value = ((amp.real * c_im) + (amp.imag * c_re)) * dt
            value[plus_zero] = 0.0
            out[:, column] = value
            column += 1
    if scales is not None:
        out *= np.asarray(scales, dtype=np.float64)[None, :]
    return out


def deposit_scales(sources: Sequence[Source], condinv: Dict[int, np.ndarray]) -> Optional[np.ndarray]:
    """Per deposit point, the float64 ``condinv`` word of its target component at its
    cell (``condinv``: component index 0..2 (D) or 3..5 (B) -> float32 volume of the
    lossy components), or None when no point lands on a lossy component."""
    if not any(source.comp_index in condinv for source in sources):
        return None
    scales = []
    for source in sources:
        volume = condinv.get(source.comp_index)
        for (i, j, k) in source.cells:
            scales.append(1.0 if volume is None else float(volume[i, j, k]))
    return np.asarray(scales, dtype=np.float64)


def deposit_words_scalar(sources: Sequence[Source], first_step: int, steps: int, dt: float) -> np.ndarray:
    """The per-step, per-point form of :func:`deposit_words` (kept to check the array form)."""
    count = sum(len(s.cells) for s in sources)
    out = np.zeros((steps, count), dtype=np.float64)
    for row in range(steps):
        n = first_step + row
        column = 0
        for source in sources:
            t = n * dt + 0.5 * dt if not source.magnetic else n * dt
            c = source.current(t)
            plus_zero = (c[0] == 0.0 and math.copysign(1.0, c[0]) > 0
                         and c[1] == 0.0 and math.copysign(1.0, c[1]) > 0)
            for amp in source.amps:
                out[row, column] = 0.0 if plus_zero else (amp.real * c[0] - amp.imag * c[1]) * dt
                column += 1
    return out


def make_waveform(spec: dict):
    """Waveform from the reference's ``add_source`` protocol dict (driver.py:2567)."""
    kind = spec.get("source_type", "continuous")
    if spec.get("is_integrated", False):
        raise Unsupported("integrated sources are not stepped by this engine")
    if kind == "gaussian":
        kwargs = {k: spec[k] for k in ("start_time", "cutoff") if k in spec}
        return GaussianWaveform(float(spec["frequency"]), float(spec["fwidth"]), **kwargs)
    if kind == "continuous":
        kwargs = {k: spec[k] for k in ("start_time", "end_time", "width", "slowness") if k in spec}
        return ContinuousWaveform(float(spec["frequency"]), **kwargs)
    if kind == "custom":
        if "frequency" in spec:
            raise ValueError("a custom source takes src_func and no frequency")
        kwargs = {k: spec[k] for k in ("start_time", "end_time") if k in spec}
        return CustomWaveform(spec["src_func"], **kwargs)
    raise ValueError(f"unknown source_type {kind!r}")
