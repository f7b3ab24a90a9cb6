"""Lift a MEEP simulation onto this engine and step it: ``lift_simulation``, ``run_on_gpu``
and the ``GpuRunResult`` they return.

Mirrors the reference's MEEP entry points (``meep_gpu/from_meep.py``: ``lift_simulation``
:5297, ``run_on_gpu`` :9532, ``GpuRunResult`` :454 with ``get_flux_spectrum`` :522,
``get_flux_data`` :575, ``get_array`` :956, ``get_field`` :982) for the simulations this
engine steps: 3-D Cartesian cells, metallic or (Bloch-)periodic boundaries, mirror
symmetries, isotropic media with Lorentzian/Drude susceptibilities and D/B
conductivity, ``mp.PML`` and ``mp.Absorber`` layers, Gaussian and continuous
``mp.Source`` objects, and ``sim.add_flux`` / ``sim.add_dft_fields`` monitors. Anything
else is refused by name (:class:`MeepSimulationNotLiftable`) before anything is built.

The simulation is read only through MEEP's public Python names: ``cell_size``,
``resolution``, ``Courant``, ``k_point``, ``symmetries``, ``geometry``,
``default_material``, ``boundary_layers``, ``sources``, ``dft_objects``,
``eps_averaging``, ``init_sim()``, ``fields.is_real``, ``fields.last_source_time()``,
``fields.get_chi1inv(c, d, loc, frequency)`` and ``get_epsilon_grid(xtics, ytics, ztics)``.
MEEP itself is imported lazily (only these functions need it); the component and
direction constants are taken from the imported module by name.

The permittivity is read per E component at that component's own Yee points:
``1 / fields.get_chi1inv(c, c, loc, 0)`` (MEEP's stored, subpixel-smoothed words; one
call per point) when ``sim.eps_averaging`` is on, and one ``get_epsilon_grid`` call per
component (point sampling, which is what MEEP stores without smoothing) when it is off.
Susceptibility sigma and conductivity are sampled at the same points from the media of
the geometry (axis-aligned ``Block``, ``Sphere`` and ``Cylinder``; a later object wins,
MEEP's rule), the default material filling the rest.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .conductivity import AbsorberLayer
from .dispersion import Susceptibility
from .driver import FdtdDriver
from .grid import IYEE, Mirror, Unsupported

E_NAMES = ("Ex", "Ey", "Ez")
H_NAMES = ("Hx", "Hy", "Hz")
D_NAMES = ("Dx", "Dy", "Dz")
B_NAMES = ("Bx", "By", "Bz")
SHAPES = ("Block", "Sphere", "Cylinder")
SUSCEPTIBILITY_KINDS = {"LorentzianSusceptibility": "lorentzian", "DrudeSusceptibility": "drude"}
MIGRATABLE_MONITORS = ("DftFlux", "DftFields")


class MeepSimulationNotLiftable(Unsupported):
    """The simulation uses something this engine does not step; nothing was built."""

    def __init__(self, reasons: Sequence[str]):
        self.reasons = tuple(reasons)
        super().__init__("this MEEP simulation cannot be lifted: " + "; ".join(self.reasons))


def _import_meep():
    try:
        import meep  # noqa: PLC0415 - only the lift needs MEEP
    except ImportError as exc:
        raise ImportError("meep_gpu_gb300.from_meep needs CPU MEEP importable to read an mp.Simulation; "
                          "FdtdDriver and everything under it do not") from exc
    return meep


def _vector3(value: Any) -> Tuple[float, float, float]:
    if value is None:
        return (0.0, 0.0, 0.0)
    if hasattr(value, "x"):
        return (float(value.x), float(value.y), float(value.z))
    values = tuple(float(v) for v in value)
    return values + (0.0,) * (3 - len(values))


def _component_name(mp, component) -> str:
    for name in E_NAMES + H_NAMES:
        if getattr(mp, name, None) == component:
            return name
    raise MeepSimulationNotLiftable([f"source component {component!r} is not one of {E_NAMES + H_NAMES}"])


def _direction_axis(mp, direction) -> Optional[int]:
    """mp.X/Y/Z -> 0/1/2; mp.ALL (or mp.AUTOMATIC) -> None."""
    for axis, name in enumerate("XYZ"):
        if getattr(mp, name, None) == direction:
            return axis
    return None


def _side_names(mp, side) -> Tuple[str, ...]:
    if side == getattr(mp, "Low", 0) and side != getattr(mp, "ALL", -1):
        return ("low",)
    if side == getattr(mp, "High", 1) and side != getattr(mp, "ALL", -1):
        return ("high",)
    return ("low", "high")


# --- compatibility ---------------------------------------------------------------------
def lifted_dimensions(sim) -> Optional[int]:
    """MEEP's dimensions of ``sim``: its ``dimensions``, or 2 / 1 inferred from a zero
    cell extent on z / on x and y (MEEP's ``Simulation._infer_dimensions``); None for a
    combination this engine does not step. MEEP ignores an invariant axis's extent, so
    the lift passes 0 there."""
    dims = int(getattr(sim, "dimensions", 3) or 3)
    cell = _vector3(sim.cell_size)
    if dims == 3 and cell[2] == 0.0 and cell[0] > 0.0 and cell[1] > 0.0:
        dims = 2
    elif dims == 3 and cell[0] == 0.0 and cell[1] == 0.0 and cell[2] > 0.0:
        dims = 1
    resolved = {3: (0, 1, 2), 2: (0, 1), 1: (2,)}.get(dims)
    if resolved is None or any(cell[a] <= 0.0 for a in resolved):
        return None
    return dims


def _lifted_cell(sim, dims: int) -> Tuple[float, float, float]:
    cell = list(_vector3(sim.cell_size))
    for axis in {3: (), 2: (2,), 1: (0, 1)}[dims]:
        cell[axis] = 0.0
    return tuple(cell)  # type: ignore[return-value]


def _lifted_boundaries(sim, dims: int, kind: str) -> Dict[str, str]:
    """The boundary of every axis the run resolves; a one-cell axis is periodic whatever
    the k_point (MEEP's unit directions, fields.cpp)."""
    cell = _vector3(sim.cell_size)
    out = {}
    for axis in {3: (0, 1, 2), 2: (0, 1), 1: (2,)}[dims]:
        one_cell = int(cell[axis] * float(sim.resolution) + 0.5) == 1
        out["xyz"[axis]] = "periodic" if one_cell else kind
    return out


def _materials(sim) -> List[Any]:
    materials = [getattr(sim, "default_material", None)]
    materials += [getattr(obj, "material", None) for obj in (getattr(sim, "geometry", None) or ())]
    return [m for m in materials if m is not None]


def gpu_compatibility(mp, sim) -> List[str]:
    """Every reason this engine refuses ``sim`` (empty: it can be lifted); reference
    ``gpu_compatibility`` (from_meep.py) for the configurations stepped here."""
    reasons: List[str] = []
    if getattr(sim, "is_cylindrical", False):
        reasons.append("cylindrical cells are not stepped")
    dims = lifted_dimensions(sim)
    if dims is None:
        reasons.append(f"dimensions={getattr(sim, 'dimensions', 3)!r} on a cell of size "
                       f"{_vector3(sim.cell_size)}: 3-D, 2-D (z invariant) and 1-D (along z) cells are stepped")
    if getattr(sim, "special_kz", False):
        reasons.append("special_kz (an out-of-plane beta) is not stepped")
    if getattr(sim, "material_function", None) is not None or getattr(sim, "epsilon_input_file", ""):
        reasons.append("a material_function or epsilon_input_file cell is not lifted (use FdtdDriver directly)")
    for obj in getattr(sim, "geometry", None) or ():
        kind = type(obj).__name__
        material = getattr(obj, "material", None)
        if _is_structured_medium(material) and kind not in SHAPES:
            reasons.append(f"a {kind} carrying a susceptibility or conductivity (its sigma is sampled from "
                           f"{list(SHAPES)} only)")
        for attr in ("e1", "e2", "e3"):
            axis = getattr(obj, attr, None)
            if axis is not None and kind == "Block":
                v = _vector3(axis)
                if sum(1 for c in v if c != 0.0) != 1:
                    reasons.append("a rotated Block (e1/e2/e3 off the axes)")
                    break
        if kind == "Cylinder" and _direction_axis(mp, getattr(obj, "axis", None)) is None:
            axis = _vector3(getattr(obj, "axis", (0, 0, 1)))
            if sum(1 for c in axis if c != 0.0) != 1:
                reasons.append("a Cylinder off the coordinate axes")
    for material in _materials(sim):
        for term in getattr(material, "E_susceptibilities", None) or ():
            kind = type(term).__name__
            if kind not in SUSCEPTIBILITY_KINDS:
                reasons.append(f"a {kind} (only Lorentzian and Drude terms are stepped)")
            offdiag = _vector3(getattr(term, "sigma_offdiag", None))
            if any(offdiag):
                reasons.append("an anisotropic susceptibility (sigma_offdiag)")
        if getattr(material, "H_susceptibilities", None):
            reasons.append("magnetic susceptibilities are not stepped")
        if any(_vector3(getattr(material, "epsilon_offdiag", None))):
            reasons.append("off-diagonal epsilon is not stepped")
        if any(v != 1.0 for v in _vector3(getattr(material, "mu_diag", (1.0, 1.0, 1.0)))):
            reasons.append("mu != 1 is not stepped")
        for attr in ("E_chi2_diag", "E_chi3_diag", "H_chi2_diag", "H_chi3_diag"):
            if any(_vector3(getattr(material, attr, None))):
                reasons.append("chi2/chi3 nonlinearity is not stepped")
    for layer in getattr(sim, "boundary_layers", None) or ():
        kind = type(layer).__name__
        if kind not in ("PML", "Absorber"):
            reasons.append(f"a {kind} boundary layer")
            continue
        if getattr(layer, "pml_profile", None) is not None and not _default_profile(layer.pml_profile):
            reasons.append(f"a custom {kind} profile")
        if kind == "PML" and float(getattr(layer, "mean_stretch", 1.0)) != 1.0:
            reasons.append("a PML with mean_stretch != 1")
    for source in getattr(sim, "sources", None) or ():
        kind = type(source).__name__
        if kind != "Source":
            reasons.append(f"a {kind} (only mp.Source is lifted)")
            continue
        src_kind = type(source.src).__name__
        if src_kind not in ("GaussianSource", "ContinuousSource"):
            reasons.append(f"a {src_kind} waveform")
        if getattr(source.src, "is_integrated", False):
            reasons.append("an integrated source")
        try:
            _component_name(mp, source.component)
        except MeepSimulationNotLiftable as exc:
            reasons.extend(exc.reasons)
    for monitor in getattr(sim, "dft_objects", None) or ():
        kind = type(monitor).__name__
        if kind not in MIGRATABLE_MONITORS:
            reasons.append(f"a {kind} monitor (migrated: {list(MIGRATABLE_MONITORS)})")
        elif kind == "DftFlux" and len(getattr(monitor, "regions", ())) != 1:
            reasons.append("a flux object over more than one FluxRegion (add one flux per region)")
    return reasons


def _default_profile(profile) -> bool:
    try:
        return abs(float(profile(0.5)) - 0.25) < 1e-15 and abs(float(profile(1.0)) - 1.0) < 1e-15
    except Exception:  # noqa: BLE001 - an unreadable profile is a custom one
        return False


def _is_structured_medium(material) -> bool:
    if material is None:
        return False
    return bool(getattr(material, "E_susceptibilities", None)) or _conductivity_of(material, "D") != (0, 0, 0) \
        or _conductivity_of(material, "B") != (0, 0, 0)


def _conductivity_of(material, side: str) -> Tuple[float, float, float]:
    value = getattr(material, f"{side}_conductivity_diag", None)
    if value is None:
        scalar = getattr(material, f"{side}_conductivity", 0.0) or 0.0
        return (float(scalar),) * 3
    return _vector3(value)


# --- geometry sampling -----------------------------------------------------------------
def yee_points(grid, component: str) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """User coordinates of every stored point of ``component`` along each axis: doubled
    offset ``origin + 2 i + shift`` times ``dx / 2``."""
    shifts = IYEE[component]
    tics = []
    for axis in range(3):
        n = grid.shape[axis]
        if grid.is_invariant(axis):
            # MEEP hands 0 on an axis the run does not carry (vec2py)
            tics.append(np.zeros(1))
            continue
        doubled = grid.origin_doubled(axis) + 2 * np.arange(n) + shifts[axis]
        tics.append(doubled * (grid.dx / 2.0))
    return tuple(tics)  # type: ignore[return-value]


def _inside(mp, obj, x, y, z) -> np.ndarray:
    """Points of the broadcast (x, y, z) inside one axis-aligned geometric object."""
    kind = type(obj).__name__
    center = _vector3(getattr(obj, "center", None))
    if kind == "Block":
        size = _vector3(obj.size)
        # the block's own axes: each e_i names one coordinate axis
        extents = [0.0, 0.0, 0.0]
        for attr, length in zip(("e1", "e2", "e3"), size):
            e = _vector3(getattr(obj, attr, None)) if getattr(obj, attr, None) is not None else None
            axis = {"e1": 0, "e2": 1, "e3": 2}[attr] if e is None else int(np.argmax(np.abs(e)))
            extents[axis] = length
        inside = np.ones(np.broadcast(x, y, z).shape, dtype=bool)
        for coord, c, length in zip((x, y, z), center, extents):
            inside &= np.abs(coord - c) <= length / 2.0
        return inside
    if kind == "Sphere":
        r = float(obj.radius)
        return (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2 <= r * r
    if kind == "Cylinder":
        axis = _direction_axis(mp, getattr(obj, "axis", None))
        if axis is None:
            axis = int(np.argmax(np.abs(_vector3(getattr(obj, "axis", (0, 0, 1))))))
        coords = (x, y, z)
        radial = [a for a in range(3) if a != axis]
        r2 = (coords[radial[0]] - center[radial[0]]) ** 2 + (coords[radial[1]] - center[radial[1]]) ** 2
        height = float(getattr(obj, "height", math.inf))
        along = np.abs(coords[axis] - center[axis]) <= height / 2.0
        return (r2 <= float(obj.radius) ** 2) & along
    raise MeepSimulationNotLiftable([f"a {kind} whose material varies the dispersion or conductivity"])


def _owner_map(mp, sim, grid, component: str) -> Tuple[np.ndarray, List[Any]]:
    """Index into ``media`` of the medium at each stored point of ``component`` (0: the
    default material; later objects over earlier ones)."""
    x, y, z = (t.reshape(s) for t, s in zip(yee_points(grid, component),
                                           ((-1, 1, 1), (1, -1, 1), (1, 1, -1))))
    media = [getattr(sim, "default_material", None)]
    owner = np.zeros(grid.shape, dtype=np.int32)
    for obj in getattr(sim, "geometry", None) or ():
        material = getattr(obj, "material", None)
        media.append(material)
        if material is None or type(obj).__name__ not in SHAPES:
            continue
        owner[np.broadcast_to(_inside(mp, obj, x, y, z), grid.shape)] = len(media) - 1
    return owner, media


def _read_epsilon(mp, sim, driver, route: str, progress_cb) -> None:
    grid = driver.grid
    volumes = []
    for q, name in enumerate(E_NAMES):
        xs, ys, zs = yee_points(grid, name)
        if route == "grid":
            eps = np.asarray(sim.get_epsilon_grid(xs, ys, zs), dtype=np.float64).reshape(grid.shape)
        else:
            comp, direction = getattr(mp, name), getattr(mp, "XYZ"[q])
            read = sim.fields.get_chi1inv
            eps = np.empty(grid.shape, dtype=np.float64)
            for i, xv in enumerate(xs):
                for j, yv in enumerate(ys):
                    for k, zv in enumerate(zs):
                        chi1inv = complex(read(comp, direction, mp.Vector3(xv, yv, zv), 0)).real
                        eps[i, j, k] = 1.0 / chi1inv
                if progress_cb is not None:
                    progress_cb(q * len(xs) + i + 1, 3 * len(xs))
        volumes.append(eps)
    if all(np.array_equal(volumes[0], v) for v in volumes[1:]):
        driver.set_epsilon(volumes[0])
    else:
        driver.set_epsilon_components(*volumes)


def _lift_dispersion(mp, sim, driver) -> None:
    """One driver susceptibility per distinct pole (kind, frequency, gamma), its sigma per
    E component sampled from the media at that component's Yee points."""
    grid = driver.grid
    poles: Dict[Tuple[str, float, float], Dict[str, np.ndarray]] = {}
    owners = {name: _owner_map(mp, sim, grid, name) for name in E_NAMES}
    for q, name in enumerate(E_NAMES):
        owner, media = owners[name]
        for index, medium in enumerate(media):
            for term in (getattr(medium, "E_susceptibilities", None) or ()) if medium is not None else ():
                kind = SUSCEPTIBILITY_KINDS[type(term).__name__]
                key = (kind, float(term.frequency), float(term.gamma))
                sigma_diag = getattr(term, "sigma_diag", None)
                sigma = _vector3(sigma_diag)[q] if sigma_diag is not None else float(term.sigma)
                volume = poles.setdefault(key, {c: np.zeros(grid.shape, np.float64) for c in E_NAMES})[name]
                volume[owner == index] += sigma
    for (kind, frequency, gamma), sigma in poles.items():
        driver.add_susceptibility(Susceptibility(frequency=frequency, gamma=gamma, kind=kind),
                                  {c: v.astype(np.float32) for c, v in sigma.items()})


def _lift_conductivity(mp, sim, driver) -> None:
    grid = driver.grid
    for side, names in (("D", D_NAMES), ("B", B_NAMES)):
        volumes = {}
        for q, name in enumerate(names):
            owner, media = _owner_map(mp, sim, grid, name)
            values = np.array([_conductivity_of(m, side)[q] if m is not None else 0.0 for m in media])
            volume = values[owner]
            volumes[name] = volume.astype(np.float32) if np.any(volume != 0.0) else None
        if any(v is not None for v in volumes.values()):
            (driver.set_conductivity if side == "D" else driver.set_b_conductivity)(volumes)


def _lift_layers(mp, sim, driver) -> None:
    pml: Dict[str, Dict[str, float]] = {}
    absorbers: List[AbsorberLayer] = []
    order = None
    r_asymptotic = None
    for layer in getattr(sim, "boundary_layers", None) or ():
        thickness = float(layer.thickness)
        axis = _direction_axis(mp, getattr(layer, "direction", getattr(mp, "ALL", -1)))
        # a layer on an invariant axis is dropped, as MEEP drops it (it has no face)
        axes = [a for a in (range(3) if axis is None else (axis,)) if not driver.grid.is_invariant(a)]
        sides = _side_names(mp, getattr(layer, "side", getattr(mp, "ALL", -1)))
        kind = type(layer).__name__
        for a in axes:
            for side in sides:
                if kind == "PML":
                    pml.setdefault("xyz"[a], {})[side] = thickness * driver.grid.resolution
                else:
                    absorbers.append(AbsorberLayer(thickness, a, side,
                                                   float(getattr(layer, "R_asymptotic", 1e-15))))
        if kind == "PML":
            r = float(getattr(layer, "R_asymptotic", 1e-15))
            if r_asymptotic is not None and r != r_asymptotic:
                raise MeepSimulationNotLiftable(["PML layers with different R_asymptotic"])
            r_asymptotic = r
            order = 2
    if pml:
        faces = {axis: dict(sides) for axis, sides in pml.items()}
        if r_asymptotic is not None and r_asymptotic != 1e-15:
            raise MeepSimulationNotLiftable([f"a PML with R_asymptotic={r_asymptotic} (the engine grades 1e-15)"])
        driver.setup_pml(faces, order=order or 2)
    if absorbers:
        driver.set_absorber(absorbers)


def _lift_absent_components(mp, sim, driver) -> None:
    """The components MEEP allocated no array for (``fields::have_component``, read once
    the sources are in; reference ``driver.py:2344``): a reduced-dimension run's other
    polarization. A fields object without that query leaves every component stepped."""
    have = getattr(sim.fields, "have_component", None)
    if not callable(have) or driver.grid.dimensions == 3:
        return
    absent = [name for name in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz", "Bx", "By", "Bz")
              if hasattr(mp, name) and not have(getattr(mp, name))]
    if absent:
        driver.set_absent_components(absent)


def _lift_source(mp, source) -> Dict[str, Any]:
    src = source.src
    spec: Dict[str, Any] = {
        "component": _component_name(mp, source.component),
        "center": _vector3(source.center),
        "size": _vector3(getattr(source, "size", None)),
        "amplitude": complex(getattr(source, "amplitude", 1.0)),
        "frequency": float(src.frequency),
        "start_time": float(getattr(src, "start_time", 0.0)),
    }
    if getattr(source, "amp_func", None) is not None:
        spec["amp_func"] = source.amp_func
    if type(src).__name__ == "GaussianSource":
        spec.update(source_type="gaussian", fwidth=float(src.fwidth), cutoff=float(getattr(src, "cutoff", 5.0)))
    else:
        spec.update(source_type="continuous", end_time=float(getattr(src, "end_time", 1e20)),
                    width=float(getattr(src, "width", 0.0)), slowness=float(getattr(src, "slowness", 3.0)))
    if spec["amplitude"].imag == 0.0:
        spec["amplitude"] = spec["amplitude"].real
    return spec


def _frequencies(monitor) -> List[float]:
    freq = getattr(monitor, "freq", None)
    if freq is None:
        freq = getattr(monitor, "frequencies", None)
    return [float(f) for f in freq]


class MigratedMonitors:
    """The monitors the lift rebuilt, keyed by the IDENTITY of the MEEP objects (reference
    ``MigratedMonitors``): an object is resolved only if it is the one the lift read."""

    def __init__(self, pairs: Sequence[Tuple[Any, Any]] = ()):
        self._pairs = list(pairs)

    def resolve(self, meep_monitor) -> Optional[Any]:
        for original, migrated in self._pairs:
            if original is meep_monitor:
                return migrated
        return None

    def items(self):
        return list(self._pairs)

    def __len__(self) -> int:
        return len(self._pairs)

    def __iter__(self):
        return iter([migrated for _, migrated in self._pairs])


def migrate_monitors(mp, sim, driver) -> MigratedMonitors:
    """Each ``sim.add_flux`` / ``sim.add_dft_fields`` object as this driver's monitor."""
    pairs = []
    for monitor in getattr(sim, "dft_objects", None) or ():
        kind = type(monitor).__name__
        decimation = int(getattr(monitor, "decimation_factor", 0) or 0)
        freqs = _frequencies(monitor)
        if kind == "DftFlux":
            region = monitor.regions[0]
            direction = _direction_axis(mp, getattr(region, "direction", None))
            migrated = driver.add_flux_monitor(freqs, center=_vector3(region.center), size=_vector3(region.size),
                                               direction=direction, weight=complex(getattr(region, "weight", 1.0)).real,
                                               decimation_factor=decimation)
        else:
            components = tuple(_component_name(mp, c) for c in monitor.components)
            where = getattr(monitor, "where", None)
            center = _vector3(getattr(where, "center", getattr(monitor, "center", None)))
            size = _vector3(getattr(where, "size", getattr(monitor, "size", None)))
            migrated = driver.add_dft_monitor(freqs, components=components, center=center, size=size,
                                              decimation_factor=decimation)
        pairs.append((monitor, migrated))
    return MigratedMonitors(pairs)


def lift_simulation(sim, *, prefer_gpu: bool = True, gpu_id: int = 0, epsilon_route: str = "auto",
                    progress_cb: Optional[Callable[[int, int], None]] = None) -> FdtdDriver:
    """Build an :class:`FdtdDriver` that reproduces ``sim``, ready to step (reference
    ``lift_simulation``, from_meep.py:5297).

    Calls ``sim.init_sim()`` (MEEP's grid, rasterization and smoothing), then reads the
    cell, clock, symmetries, boundaries, permittivity (``epsilon_route``: ``"chi1inv"``
    reads MEEP's stored words point by point, ``"grid"`` samples the geometry with
    ``get_epsilon_grid``; ``"auto"`` takes ``"chi1inv"`` when ``sim.eps_averaging`` is
    on), dispersion, conductivity, layers, sources and monitors. Nothing is stepped.
    """
    if not prefer_gpu:
        raise Unsupported("this engine has no CPU stepping path: prefer_gpu=False is the reference's "
                          "NumPy driver, not this one")
    if epsilon_route not in ("auto", "chi1inv", "grid"):
        raise ValueError(f"epsilon_route must be 'auto', 'chi1inv' or 'grid', got {epsilon_route!r}")
    mp = _import_meep()
    reasons = gpu_compatibility(mp, sim)
    if reasons:
        raise MeepSimulationNotLiftable(reasons)
    started = time.perf_counter()
    sim.init_sim()
    k_point = getattr(sim, "k_point", False)
    dims = lifted_dimensions(sim)
    driver = FdtdDriver(
        cell_size=_lifted_cell(sim, dims), resolution=float(sim.resolution), courant=float(sim.Courant),
        force_complex_fields=not bool(sim.fields.is_real),
        symmetry=tuple(Mirror("XYZ"[_direction_axis(mp, s.direction)], int(complex(s.phase).real))
                       for s in getattr(sim, "symmetries", None) or ()),
        k_point=_vector3(k_point) if k_point else (0.0, 0.0, 0.0),
        boundaries=_lifted_boundaries(sim, dims, "periodic" if k_point else "metallic"),
        dimensions=dims, gpu_id=gpu_id)
    try:
        route = epsilon_route
        if route == "auto":
            route = "chi1inv" if getattr(sim, "eps_averaging", True) else "grid"
        _read_epsilon(mp, sim, driver, route, progress_cb)
        _lift_dispersion(mp, sim, driver)
        _lift_conductivity(mp, sim, driver)
        _lift_layers(mp, sim, driver)
        for source in getattr(sim, "sources", None) or ():
            driver.add_source(_lift_source(mp, source))
        _lift_absent_components(mp, sim, driver)
        driver.migrated_monitors = migrate_monitors(mp, sim, driver)
    except Exception:
        driver.close()
        raise
    driver.lift_record = {"meep_version": getattr(mp, "__version__", None), "engine_precision": "single",
                          "epsilon_route": route, "lift_seconds": time.perf_counter() - started}
    return driver


@dataclass(frozen=True)
class GpuRunResult:
    """The outcome of :func:`run_on_gpu` (reference ``GpuRunResult``, from_meep.py:454):
    the stepped driver, the steps this call took, the simulation time reached and the
    wall time of the step loop. The driver stays open; :meth:`close` releases it."""

    driver: FdtdDriver
    steps: int
    meep_time: float
    wall_time_s: float

    @property
    def monitors(self) -> MigratedMonitors:
        return getattr(self.driver, "migrated_monitors", None) or MigratedMonitors()

    @property
    def lift_record(self):
        return getattr(self.driver, "lift_record", None)

    def monitor_for(self, meep_monitor):
        found = self.monitors.resolve(meep_monitor)
        if found is None:
            raise KeyError(f"{type(meep_monitor).__name__} was not migrated onto this run (only "
                           f"{list(MIGRATABLE_MONITORS)} attached to the simulation before the lift are)")
        return found

    def get_flux_spectrum(self, meep_flux) -> np.ndarray:
        """``mp.get_fluxes(flux)`` for a migrated ``sim.add_flux`` object."""
        return self.monitor_for(meep_flux).get_flux_spectrum()

    def get_flux_data(self, meep_flux):
        """``sim.get_flux_data(flux)``: the transforms, for ``run_on_gpu(...,
        minus_flux_data=[(flux2, data)])`` on a later run (two-run normalisation)."""
        return self.monitor_for(meep_flux).get_dft_data()

    def get_dft_array(self, meep_dft, component: str, frequency_index: int) -> np.ndarray:
        """``sim.get_dft_array(dft, component, index)`` over the migrated region."""
        return self.monitor_for(meep_dft).raw(component)[frequency_index]

    def get_array(self, component: str, center: Any = None, size: Any = None) -> np.ndarray:
        """One component as MEEP's ``sim.get_array(component=...)`` over the whole cell
        returns it: the cell-centred values, plus on every unfolded periodic axis MEEP's
        duplicate plane at index 0 (the top plane's lattice image; on a Bloch-phased axis
        times ``conj(eikna)``)."""
        if center is not None or size is not None:
            raise Unsupported("get_array over a sub-volume is not provided; read the whole cell")
        driver = self.driver
        grid = driver.grid
        values = driver.get_field(component, cell_centered=True)
        for axis in range(3):
            if grid.is_metallic(axis) or grid.is_mirrored(axis):
                continue
            top = np.take(values, [values.shape[axis] - 1], axis=axis)
            phase = grid.bloch_phase(axis)
            if phase is not None:
                top = (top * np.complex64(np.conj(phase))).astype(values.dtype)
            values = np.concatenate([top, values], axis=axis)
        return values

    def get_field(self, component: str, cell_centered: bool = True) -> np.ndarray:
        """One component in the driver's own layout (no duplicate plane)."""
        return self.driver.get_field(component, cell_centered=cell_centered)

    def close(self) -> None:
        self.driver.close()


def _load_flux_data(driver, pairs, minus: bool) -> None:
    monitors = getattr(driver, "migrated_monitors", None) or MigratedMonitors()
    for meep_flux, data in pairs:
        target = monitors.resolve(meep_flux)
        if target is None:
            raise KeyError(f"{type(meep_flux).__name__} passed to run_on_gpu is not a monitor of this simulation")
        (target.load_minus_dft_data if minus else target.load_dft_data)(data)


def run_on_gpu(sim, until: Optional[float] = None, until_after_sources: Optional[float] = None, *,
               prefer_gpu: bool = True, gpu_id: int = 0,
               prepare: Optional[Callable[[FdtdDriver], None]] = None,
               flux_data: Sequence[Tuple[Any, Any]] = (), minus_flux_data: Sequence[Tuple[Any, Any]] = (),
               step_functions: Sequence[Callable[..., Any]] = (),
               progress_cb: Optional[Callable[[int, int], None]] = None,
               lift_progress_cb: Optional[Callable[[int, int], None]] = None,
               cancel_check: Optional[Callable[[], bool]] = None, progress_interval: int = 100,
               epsilon_route: str = "auto") -> GpuRunResult:
    """Lift ``sim`` and step it: MEEP's ``sim.run(until=...)`` or
    ``sim.run(until_after_sources=...)`` with the loop on the GPU (reference
    ``run_on_gpu``, from_meep.py:9532). ``until_after_sources`` is measured from MEEP's
    own ``sim.fields.last_source_time()``. ``flux_data`` / ``minus_flux_data`` are
    ``[(meep_flux, data), ...]`` loaded into the migrated monitors before the first
    step (MEEP's ``load_flux_data`` / ``load_minus_flux_data``)."""
    given = [name for name, value in (("until", until), ("until_after_sources", until_after_sources))
             if value is not None]
    if len(given) != 1:
        raise ValueError(f"run_on_gpu takes exactly one of until or until_after_sources, got {given or 'none'}")
    for keyword, value in (("until", until), ("until_after_sources", until_after_sources)):
        if value is not None and (callable(value) or isinstance(value, (list, tuple))):
            raise TypeError(f"{keyword} takes a simulation time; MEEP stop conditions (callables) are not "
                            "run by this engine: lift the simulation and call FdtdDriver.run")
    if step_functions:
        raise Unsupported("MEEP step functions are not run by this engine")
    driver = lift_simulation(sim, prefer_gpu=prefer_gpu, gpu_id=gpu_id, epsilon_route=epsilon_route,
                             progress_cb=lift_progress_cb)
    try:
        if prepare is not None:
            prepare(driver)
        _load_flux_data(driver, flux_data, minus=False)
        _load_flux_data(driver, minus_flux_data, minus=True)
        if until is not None:
            end_time = float(until)
        else:
            end_time = float(sim.fields.last_source_time()) + float(until_after_sources)
            if not math.isfinite(end_time) or end_time > 1e19:
                raise ValueError(f"until_after_sources={until_after_sources!r} never ends: a source emits "
                                 "forever (give it an end_time, or use until=)")
        before = driver.step_count
        driver.run(until=end_time, progress_cb=progress_cb, cancel_check=cancel_check,
                   progress_interval=progress_interval)
    except Exception:
        driver.close()
        raise
    return GpuRunResult(driver=driver, steps=driver.step_count - before, meep_time=driver.time,
                        wall_time_s=driver.last_run_seconds)
