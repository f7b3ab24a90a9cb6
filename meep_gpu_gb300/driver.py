"""``FdtdDriver``: the reference's driver API, stepped on one GB300 by ``libmeepgb.so``.

Mirrors ``meep_gpu/driver.py``'s ``FdtdDriver`` (constructor :810, ``set_epsilon``
:1170, ``add_susceptibility`` :1531, ``setup_pml`` :2155, ``add_source`` :2567,
``add_dft_monitor`` :2783, ``add_flux_monitor`` :3001, ``step`` :3419, ``run`` :3667,
``get_field`` :4056, ``set_conductivity`` :1649, ``set_b_conductivity`` :1752,
``set_absorber`` :1863) for the configurations this engine steps: 3-D, real float32 or
complex64 fields, metallic, periodic or Bloch-periodic boundaries, mirror planes (``Mirror``)
folding metallic axes, isotropic or
diagonal chi1inv, Lorentz/Drude poles, D and B conductivity (material and
``mp.Absorber``), electric sources and DFT/flux monitors.
Anything else is refused by name when it is asked for, never approximated.

The configuration freezes at the first step (as the reference's fast-path plan
does, driver.py:3509): the engine allocates the device state and every later step
is two kernel launches (plus a monitor launch on decimated steps). There is no CPU
stepping path: without a GPU, or without the built library, stepping raises.
"""

from __future__ import annotations

import math
import numbers
import time as time_module
from typing import Any, Callable, Dict, List, Mapping, Optional, Sequence, Tuple

import numpy as np

from . import conductivity as cond
from .conductivity import AbsorberLayer
from .dft import (DFTMonitor, FluxMonitor, absorbing_cells, automatic_decimation, folded_site,
                  normalize_frequencies)
from .dispersion import Susceptibility
from .grid import AXIS_NAMES, IYEE, Grid, Unsupported
from .pml import PML
from .sources import Source, bind_src_vols, make_waveform

FIELD_COMPONENTS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz", "Bx", "By", "Bz")
STEP_TOLERANCE = 1e-9
# How often run() samples the field energy of a dispersive run, and how far above the peak
# reached while the sources still emit it may climb afterwards (reference driver.py:319-320).
STABILITY_CHECK_INTERVAL = 20
STABILITY_GROWTH_LIMIT = 1e3


class FdtdDivergence(RuntimeError):
    """The run diverged: a non-finite field was written, or a dispersive run's field
    energy ran away after its sources stopped."""


class DivergenceGuard:
    """The field-energy watch of a dispersive run (reference ``_DivergenceGuard``,
    driver.py:747-792).

    A dispersive run can diverge smoothly, staying finite for thousands of steps. In a
    passive medium under periodic or absorbing boundaries the field energy is
    non-increasing once the last source has stopped, so every ``interval`` steps the
    energy ``sum |E|^2 eps + |B|^2`` is read: a non-finite value raises, while the
    sources emit the peak is tracked, and afterwards a value above ``growth_limit``
    times that peak raises :class:`FdtdDivergence`.

    ``energy`` is the scalar's source (default: the driver's device reduction).
    """

    def __init__(self, driver: "FdtdDriver", interval: int = STABILITY_CHECK_INTERVAL,
                 growth_limit: float = STABILITY_GROWTH_LIMIT,
                 energy: Optional[Callable[[], float]] = None):
        self._driver = driver
        self.interval = max(1, int(interval))
        self._growth_limit = float(growth_limit)
        self._source_end = driver.last_source_time()
        self._energy = energy if energy is not None else driver.field_energy
        self.peak = 0.0
        self.samples = 0

    def update(self) -> None:
        """Sample when the step count is a multiple of the interval; raise on divergence."""
        driver = self._driver
        if driver.step_count % self.interval:
            return
        energy = float(self._energy())
        self.samples += 1
        if not math.isfinite(energy):
            raise FdtdDivergence(f"field energy is not finite ({energy}) after {driver.step_count} steps of "
                                 f"a dispersive run")
        if driver.time <= self._source_end:
            self.peak = max(self.peak, energy)
            return
        if self.peak > 0.0 and energy > self._growth_limit * self.peak:
            raise FdtdDivergence(
                f"field energy grew to {energy:.3e} after {driver.step_count} steps, {energy / self.peak:.3e} "
                f"times the peak {self.peak:.3e} reached while the sources emitted (they stopped at "
                f"t={self._source_end:g}, it is now t={driver.time:g}); a passive medium cannot gain energy "
                f"after its drive stops, so the run is diverging")
        self.peak = max(self.peak, energy)


class FdtdCancelled(RuntimeError):
    """``cancel_check`` asked the run to stop."""


class _null_context:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def _as_xyz(name: str, value: Any) -> Tuple[float, float, float]:
    values = tuple(float(v) for v in value)
    if len(values) != 3:
        raise ValueError(f"{name} needs three components, got {value!r}")
    return values  # type: ignore[return-value]


class FdtdDriver:
    """One FDTD simulation: build it on the host, step it on the GPU."""

    def __init__(self, cell_size: Sequence[float], resolution: float, courant: float = 0.5,
                 force_complex_fields: bool = True, symmetry: Sequence[Any] = (),
                 k_point: Sequence[float] = (0.0, 0.0, 0.0), boundaries: Any = None,
                 dimensions: int = 3, cylindrical: bool = False, m: int = 0,
                 accurate_fields_near_cylorigin: bool = False, beta: float = 0.0,
                 bfast_scaled_k: Sequence[float] = (0.0, 0.0, 0.0), prefer_gpu: bool = True,
                 gpu_id: int = 0, launch_shape: Optional[Tuple[int, int, int]] = None,
                 kernels: Optional[Tuple[int, int, int, int]] = None,
                 dft_accumulation: Optional[str] = None):
        if dimensions not in (1, 2, 3) or cylindrical:
            raise Unsupported("3-D, 2-D (z invariant) and 1-D (along z) Cartesian runs are stepped by "
                              "this engine; cylindrical ones are not")
        if beta != 0.0 or any(float(k) != 0.0 for k in bfast_scaled_k):
            raise Unsupported("out-of-plane beta and BFAST are not stepped by this engine")
        del m, accurate_fields_near_cylorigin, prefer_gpu
        self.grid = Grid(cell_size, resolution, courant, boundaries, k_point, symmetry, dimensions=dimensions)
        # complex64 fields (the reference's default): at k = 0 the real and imaginary
        # parts step as two real runs (engine.ComplexEngine)
        self.complex_fields = bool(force_complex_fields)
        if self.grid.has_bloch and not self.complex_fields:
            raise ValueError("Bloch boundaries need complex fields: build the driver with "
                             "force_complex_fields=True or use k_point = (0, 0, 0)")
        self.gpu_id = int(gpu_id)
        self.launch_shape = launch_shape
        # (family, block_z, block_y, x_chunk): 1 the TMA tile kernels, 0 the generic ones;
        # None lets the autotuner time both on this grid and keep the faster.
        self.kernels = kernels
        # "tensor": buffered samples contracted on the tensor cores (default); "direct":
        # every sample added into the accumulators as it is taken.
        self.dft_accumulation = dft_accumulation
        self.pml: Optional[PML] = None
        self._eps: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None
        self._inv_eps: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None
        self._poles: List[Tuple[Susceptibility, List[Optional[np.ndarray]]]] = []
        self._sources: List[Source] = []
        # conductivity: the material's own sigma per side (component -> float32 volume or
        # None), the absorber faces and their float64 ramp, and the installed sum
        self._material_d_conductivity: Optional[Dict[str, Optional[np.ndarray]]] = None
        self._material_b_conductivity: Optional[Dict[str, Optional[np.ndarray]]] = None
        self._material_includes_absorber = False
        self._absorber_layers: Tuple[AbsorberLayer, ...] = ()
        self._absorber_sigma: Dict[str, np.ndarray] = {}
        self._conductivity: Dict[str, Optional[np.ndarray]] = {}
        # components MEEP allocated no array for (a 2-D run's other polarization)
        self._absent: Tuple[str, ...] = ()
        self._flux_monitors: List[FluxMonitor] = []
        self._dft_monitors: List[DFTMonitor] = []
        self._automatic: List[Any] = []
        self._pending_regions: List[Tuple[DFTMonitor, Any, Any]] = []
        self.step_count = 0
        self.engine = None
        self.last_run_seconds = 0.0

    # --- configuration --------------------------------------------------------------
    def _require_unfrozen(self, what: str) -> None:
        if self.engine is not None:
            raise RuntimeError(f"{what} after the first step: the configuration is frozen")

    def _volume(self, value: Any, label: str) -> np.ndarray:
        shape = self.grid.shape
        if np.isscalar(value):
            return np.full(shape, float(value), dtype=np.float64)
        array = np.asarray(value)
        if array.shape == tuple(n + 1 for n in shape):
            array = array[:-1, :-1, :-1]
        if array.shape != shape:
            raise ValueError(f"{label} shape {array.shape} does not match the grid {shape}")
        return array

    def _epsilon_and_inverse(self, value: Any, label: str) -> Tuple[np.ndarray, np.ndarray]:
        """Float32 epsilon and float32(1 / float64(epsilon)) (MEEP's chi1inv, formed in
        double), checked finite and positive; slab by slab, so the float64 temporaries
        stay in cache. Both are private copies."""
        array = self._volume(value, label)
        flat = np.ascontiguousarray(array).reshape(-1)
        epsilon = np.empty(flat.size, dtype=np.float32)
        inverse = np.empty(flat.size, dtype=np.float32)
        step = 1 << 18
        for start in range(0, flat.size, step):
            wide = flat[start:start + step].astype(np.float64)
            if not np.isfinite(wide).all() or (wide <= 0).any():
                raise ValueError(f"{label} must be finite and positive everywhere")
            epsilon[start:start + step] = wide
            np.divide(1.0, wide, out=wide)
            inverse[start:start + step] = wide
        return epsilon.reshape(self.grid.shape), inverse.reshape(self.grid.shape)

    def set_epsilon(self, eps: Any) -> None:
        """Isotropic permittivity: a scalar or a volume at the integer Yee positions."""
        self._require_unfrozen("set_epsilon")
        epsilon, inverse = self._epsilon_and_inverse(eps, "epsilon")
        self._eps = (epsilon, epsilon, epsilon)
        self._inv_eps = (inverse, inverse, inverse)

    def set_epsilon_components(self, epsilon: Any, eps_y: Any = None, eps_z: Any = None,
                               chi1inv_offdiagonal: Any = None) -> None:
        """Diagonal permittivity, one volume per E component (MEEP's chi1inv[c][c]):
        the reference's form, a mapping with exactly ``Ex``, ``Ey`` and ``Ez`` (reference
        ``driver.py:1220``), or the three volumes in order. Off-diagonal chi1inv rows are
        refused unless every one is identically zero."""
        self._require_unfrozen("set_epsilon_components")
        if chi1inv_offdiagonal:
            for row in dict(chi1inv_offdiagonal).values():
                for volume in dict(row).values():
                    if np.any(np.asarray(volume) != 0):
                        raise Unsupported("off-diagonal chi1inv is not stepped by this engine")
        if isinstance(epsilon, Mapping):
            if set(epsilon) != {"Ex", "Ey", "Ez"} or eps_y is not None or eps_z is not None:
                raise ValueError("set_epsilon_components takes a mapping of exactly Ex, Ey and Ez")
            values = (epsilon["Ex"], epsilon["Ey"], epsilon["Ez"])
        else:
            if eps_y is None or eps_z is None:
                raise ValueError("set_epsilon_components takes a mapping or three volumes")
            values = (epsilon, eps_y, eps_z)
        eps = []
        inv = []
        for label, value in zip(("eps_x", "eps_y", "eps_z"), values):
            epsilon, inverse = self._epsilon_and_inverse(value, label)
            eps.append(epsilon)
            inv.append(inverse)
        self._eps = tuple(eps)  # type: ignore[assignment]
        self._inv_eps = tuple(inv)  # type: ignore[assignment]

    def setup_pml(self, thickness_cells: Any, order: int = 2) -> PML:
        self._require_unfrozen("setup_pml")
        pml = PML(self.grid, thickness_cells, order=order)
        if self.has_conductivity:
            for source in self._sources:
                self._require_source_clear_of_conductive_pml(source.center, source.size, pml.faces)
        self.pml = pml
        return self.pml

    # --- conductivity -----------------------------------------------------------------
    @property
    def has_conductivity(self) -> bool:
        return any(v is not None for v in self._conductivity.values())

    def set_conductivity(self, d_conductivity: Any, absorber_included: bool = False) -> None:
        """MEEP's ``D_conductivity`` (driver.py:1649): a scalar, a grid-shaped or
        (n+1)-padded volume, or a ``{'Dx': .., 'Dy': .., 'Dz': ..}`` mapping of those;
        zero or None removes it. ``absorber_included`` says the volumes already carry the
        absorber ramp, which is then not added a second time on the D side."""
        self._require_unfrozen("set_conductivity")
        per_component = self._conductivity_components(d_conductivity, cond.D_COMPONENTS, "D")
        if any(v is not None for v in per_component.values()):
            self._require_existing_sources_clear()
        self._material_d_conductivity = (per_component if any(v is not None for v in per_component.values())
                                         else None)
        self._material_includes_absorber = bool(absorber_included)
        self._install_conductivity()

    def set_b_conductivity(self, b_conductivity: Any) -> None:
        """MEEP's ``B_conductivity`` (driver.py:1752), the magnetic twin of
        :meth:`set_conductivity`, with the B keys."""
        self._require_unfrozen("set_b_conductivity")
        per_component = self._conductivity_components(b_conductivity, cond.B_COMPONENTS, "B")
        self._material_b_conductivity = (per_component if any(v is not None for v in per_component.values())
                                         else None)
        self._install_conductivity()

    def set_absorber(self, layers: Any) -> None:
        """``mp.Absorber`` faces (driver.py:1863): a sequence of :class:`AbsorberLayer`,
        installed as a graded D and B conductivity added to the material's own; an empty
        sequence removes it. The faces keep their boundary condition."""
        self._require_unfrozen("set_absorber")
        resolved = tuple(layers or ())
        for layer in resolved:
            if not isinstance(layer, AbsorberLayer):
                raise TypeError(f"set_absorber takes AbsorberLayer instances, got {type(layer).__name__}")
        self._absorber_layers = resolved
        self._absorber_sigma = cond.absorber_conductivity(self.grid, resolved)
        self._install_conductivity()

    @property
    def absorber_layers(self) -> Tuple[AbsorberLayer, ...]:
        return self._absorber_layers

    def conductivity_volumes(self) -> Dict[str, Optional[np.ndarray]]:
        """The installed float32 sigma volume of each D and B component (None: lossless)."""
        return {name: self._conductivity.get(name) for name in cond.CONDUCTIVITY_COMPONENTS}

    def _conductivity_components(self, value: Any, components: Tuple[str, ...], side: str):
        if isinstance(value, Mapping):
            unknown = sorted(set(value) - set(components))
            if unknown:
                raise ValueError(f"{side} conductivity mapping carries {unknown}; the keys are the {side} "
                                 f"components {list(components)}")
            return {c: cond.coerce(value.get(c), self.grid.shape, side) for c in components}
        shared = cond.coerce(value, self.grid.shape, side)
        return {c: shared for c in components}

    def _install_conductivity(self) -> None:
        """Material sigma plus the absorber ramp per side (driver.py:1915)."""
        ramp = self._absorber_sigma
        electric_ramp = {} if (self._material_includes_absorber and self._material_d_conductivity) else ramp
        installed = {}
        installed.update(cond.compose(cond.D_COMPONENTS, self._material_d_conductivity, electric_ramp))
        installed.update(cond.compose(cond.B_COMPONENTS, self._material_b_conductivity, ramp))
        self._conductivity = installed

    def _require_existing_sources_clear(self) -> None:
        if self.pml is None:
            return
        for source in self._sources:
            self._require_source_clear_of_conductive_pml(source.center, source.size, self.pml.faces)

    def _require_source_clear_of_conductive_pml(self, center, size, faces) -> None:
        """A source stays two cells inside every absorbing face when the installed
        conductivity reaches into a PML (driver.py:2520)."""
        if not cond.reaches_a_pml(self.grid, faces, self._conductivity):
            return
        cond.require_source_clear(self.grid, faces, center, size)

    def add_susceptibility(self, susceptibility: Susceptibility, sigma: Any) -> None:
        """One Lorentz/Drude term of ``eps_inf + sum_n sigma_n chi_n`` (scalar, volume or per component)."""
        self._require_unfrozen("add_susceptibility")
        if not isinstance(susceptibility, Susceptibility):
            raise TypeError("add_susceptibility takes a meep_gpu_gb300.Susceptibility")
        if isinstance(sigma, Mapping):
            unknown = set(sigma) - {"Ex", "Ey", "Ez"}
            if unknown:
                raise Unsupported(f"sigma components {sorted(unknown)} are not stepped")
            raw = [sigma.get(c) for c in ("Ex", "Ey", "Ez")]
        else:
            raw = [sigma, sigma, sigma]
        volumes: List[Optional[np.ndarray]] = []
        for value in raw:
            if value is None:
                volumes.append(None)
                continue
            volume = np.ascontiguousarray(self._volume(value, "sigma").astype(np.float32))
            if not np.all(np.isfinite(volume)) or np.any(volume < 0):
                # reference dispersion.py:623: a negative sigma is gain
                raise ValueError("sigma must be finite and >= 0 in every cell: a negative sigma is gain, which "
                                 "grows the field while every magnitude still looks reasonable")
            volumes.append(volume if np.any(volume != 0) else None)
        radius = susceptibility.stability_radius(self.grid.dt)
        if radius > 1.0 + 1e-12:
            raise ValueError(f"susceptibility {susceptibility} is unstable at dt={self.grid.dt} "
                             f"(root modulus {radius:.6f})")
        self._poles.append((susceptibility, volumes))

    # MEEP allocates a component with every component "like" it (fields.cpp:458-474): in a
    # 2-D cell its own polarization, in 1-D the pair it couples to, in 3-D every component.
    _POLARIZATIONS = {2: (("Ez", "Dz", "Hx", "Hy", "Bx", "By"), ("Ex", "Ey", "Dx", "Dy", "Hz", "Bz")),
                      1: (("Ex", "Dx", "Hy", "By"), ("Ey", "Dy", "Hx", "Bx"))}

    def _allocated_with(self, component: str) -> Tuple[str, ...]:
        if self.grid.dimensions == 3:
            return FIELD_COMPONENTS
        for family in self._POLARIZATIONS[self.grid.dimensions]:
            if component in family:
                return family
        return (component,)

    def set_absent_components(self, names: Any) -> None:
        """Record the components MEEP allocated no array for (reference ``driver.py:2344``,
        ``fields.py:1088``): a 2-D run's other polarization, whose E MEEP never steps and
        reads as +0. Every component is stepped here; with no source on them and nothing
        coupling them in they hold zeros, +0 through the curls and the PML forms (their
        coefficients are positive) and through the positive inverse permittivity. The one
        form that can leave a -0 is a mirror fold's odd-parity ghost, so on a folded run
        the absent E words are reset to +0 after every step. Refused: a component a source
        drives, and any change after the first step. An empty ``names`` steps everything."""
        self._require_unfrozen("set_absent_components")
        names = tuple(names)
        unknown = sorted(set(names) - set(FIELD_COMPONENTS))
        if unknown:
            raise ValueError(f"set_absent_components: {unknown} are not field components "
                             f"(the twelve are {FIELD_COMPONENTS})")
        driven = sorted({source.component for source in self._sources} & set(names))
        if driven:
            raise ValueError(f"set_absent_components: {driven} carry a source, and MEEP allocates "
                             "every component a source requires")
        self._absent = tuple(name for name in FIELD_COMPONENTS if name in names)

    @property
    def absent_components(self) -> Tuple[str, ...]:
        return self._absent

    def _clear_absent(self) -> None:
        """Reset the absent E components to +0 (folded runs only: see
        :meth:`set_absent_components`)."""
        import torch

        engine = self.engine
        parts = (engine.re, engine.im) if hasattr(engine, "re") else (engine,)
        for part in parts:
            with torch.cuda.stream(part.stream) if part.stream is not None else _null_context():
                for name in self._absent:
                    if name[0] == "E":
                        part.fields[name].zero_()

    def add_source(self, source_data: Mapping[str, Any]) -> Source:
        """A source from the reference's boundary-protocol dict (driver.py:2567)."""
        self._require_unfrozen("add_source")
        spec = dict(source_data)
        unknown = set(spec) - {"component", "center", "size", "amplitude", "amp_func",
                               "is_integrated", "source_type", "frequency", "fwidth",
                               "start_time", "end_time", "cutoff", "width", "slowness",
                               "src_func"}
        if unknown:
            raise ValueError(f"unknown source keys {sorted(unknown)}")
        waveform = make_waveform(spec)
        source = Source(self.grid, spec.get("component", "Ez"),
                        _as_xyz("center", spec.get("center", (0.0, 0.0, 0.0))),
                        _as_xyz("size", spec.get("size", (0.0, 0.0, 0.0))),
                        waveform, complex(spec.get("amplitude", 1.0)), spec.get("amp_func"))
        if complex(spec.get("amplitude", 1.0)).imag != 0.0 and not self.complex_fields:
            raise Unsupported("a complex source amplitude needs complex fields")
        if self.pml is not None and self.has_conductivity:
            self._require_source_clear_of_conductive_pml(source.center, source.size, self.pml.faces)
        # MEEP's require_component: a sourced component, and every one allocated with it,
        # is present
        if source.component in self._absent:
            allocated = self._allocated_with(source.component)
            self._absent = tuple(name for name in self._absent if name not in allocated)
        self._sources.append(source)
        return source

    def _require_flat_on_invariant_axes(self, size, what: str) -> None:
        """A monitor region has no extent on an invariant axis (reference ``driver.py:3270``):
        the measure takes one dx per extended axis, so an extent there would scale the
        result by dx."""
        offenders = [AXIS_NAMES[a] for a in range(3) if self.grid.is_invariant(a) and float(size[a]) != 0.0]
        if offenders:
            raise ValueError(f"{what} size {tuple(size)} claims an extent along the invariant axes {offenders} "
                             f"of a {self.grid.dimensions}-D run; give those axes 0")

    def _decimation(self, request: int, frequencies) -> int:
        request = int(request)
        if request < 0:
            raise ValueError(f"decimation_factor must be >= 0, got {request}")
        if request == 0:
            return automatic_decimation(self.grid.dt, frequencies, self._sources)
        return request

    def add_flux_monitor(self, frequencies: Any = None, center: Optional[Sequence[float]] = None,
                         size: Optional[Sequence[float]] = None, direction: Optional[int] = None, *,
                         frequency: Any = None, fcen: Optional[float] = None, df: Optional[float] = None,
                         nfreq: Optional[int] = None, decimation_factor: int = 1,
                         weight: float = 1.0) -> FluxMonitor:
        self._require_unfrozen("add_flux_monitor")
        freqs = normalize_frequencies(frequencies, frequency, fcen, df, nfreq)
        if center is None or size is None:
            raise ValueError("a flux monitor needs a center and a size")
        plane_size = _as_xyz("size", size)
        self._require_flat_on_invariant_axes(plane_size, "flux plane")
        if self.grid.dimensions != 3:
            # an invariant axis is flat by construction and never the normal (no power
            # crosses it): the normal is the first flat axis the run resolves (reference
            # driver.py:3037-3058)
            if direction is None:
                flat = [a for a in self.grid.directions if plane_size[a] < self.grid.dx]
                if not flat:
                    raise ValueError(f"flux plane size {plane_size} has no flat axis among the axes this "
                                     "run resolves; give a size below one cell on the normal axis")
                direction = flat[0]
            elif self.grid.is_invariant(int(direction)):
                raise ValueError(f"a flux plane normal to the invariant {AXIS_NAMES[int(direction)]} axis "
                                 "measures a power that is identically zero")
        monitor = FluxMonitor(self.grid, freqs, _as_xyz("center", center), plane_size,
                              direction, weight, self._decimation(decimation_factor, freqs))
        if int(decimation_factor) == 0:
            self._automatic.append(monitor)
        self._flux_monitors.append(monitor)
        return monitor

    def add_dft_monitor(self, frequencies: Any = None, components: Sequence[str] = ("Ex", "Ey", "Ez"),
                        center: Optional[Sequence[float]] = None, size: Optional[Sequence[float]] = None,
                        *, frequency: Any = None, fcen: Optional[float] = None, df: Optional[float] = None,
                        nfreq: Optional[int] = None, decimation_factor: int = 1) -> DFTMonitor:
        self._require_unfrozen("add_dft_monitor")
        if size is not None:
            self._require_flat_on_invariant_axes(_as_xyz("size", size), "DFT region")
        freqs = normalize_frequencies(frequencies, frequency, fcen, df, nfreq)
        monitor = DFTMonitor(self.grid, freqs, tuple(components), self._decimation(decimation_factor, freqs))
        if int(decimation_factor) == 0:
            self._automatic.append(monitor)
        self._pending_regions.append((monitor, center, size))
        self._dft_monitors.append(monitor)
        return monitor

    # --- freeze ---------------------------------------------------------------------
    def _resolve_regions(self) -> None:
        for monitor, center, size in self._pending_regions:
            if center is not None and size is not None:
                monitor.set_region_from_volume(_as_xyz("center", center), _as_xyz("size", size))
                continue
            region = []
            for axis in range(3):
                n = self.grid.shape[axis]
                low, high = self.pml.faces[axis] if self.pml is not None else (0, 0)
                region += [absorbing_cells(low) if low > 0 else 0,
                           n - (absorbing_cells(high) if high > 0 else 0)]
            monitor.set_region(region)
        self._pending_regions = []

    def prepare(self) -> None:
        """Resolve what the first step fixes (automatic decimation, default monitor
        regions, vacuum epsilon) without touching the GPU."""
        for monitor in self._automatic:
            monitor._configure_decimation(automatic_decimation(self.grid.dt, monitor.frequencies,
                                                               self._sources))
        self._automatic = []
        self._resolve_regions()
        if self._inv_eps is None:
            self.set_epsilon(1.0)
        # the sources' deposit entries in MEEP's src_vol lists on this run's chunks
        faces = self.pml.faces if (self.pml is not None and self.pml.is_active) else None
        bind_src_vols(self._sources, self.grid, faces)

    def _freeze(self) -> None:
        self.freeze()

    def freeze(self, stream=None, autotune: bool = True, dft_accumulation: Optional[str] = None):
        """Fix the configuration and make the device state (once); returns the engine.

        ``stream`` is the CUDA stream the engine steps and reads on (default: the current
        stream at each call); ``autotune=False`` keeps the default kernel choice, for
        simulations stepped by a batch rather than by this driver.
        """
        if self.engine is not None:
            return self.engine
        import torch

        from .engine import ComplexEngine, Engine
        if self.grid.total_cells >= 1 << 31:
            raise Unsupported(f"a grid of {self.grid.total_cells} cells (2^31 or more) is not stepped by "
                              "this engine (32-bit cell offsets)")
        self.prepare()
        device = torch.device("cuda", self.gpu_id)
        engine_cls = ComplexEngine if self.complex_fields else Engine
        self.engine = engine_cls(self.grid, self.pml, self._inv_eps, self._poles, self._sources,
                             list(self._flux_monitors) + list(self._dft_monitors), device=device,
                             stream=stream, launch_shape=self.launch_shape, kernels=self.kernels,
                             autotune=autotune,
                             dft_accumulation=dft_accumulation or self.dft_accumulation,
                             conductivity=self._conductivity)
        return self.engine

    @property
    def sources(self):
        return list(self._sources)

    # --- stepping -------------------------------------------------------------------
    @property
    def time(self) -> float:
        return self.step_count * self.grid.dt

    @property
    def dt(self) -> float:
        return self.grid.dt

    @property
    def dx(self) -> float:
        return self.grid.dx

    @property
    def shape(self) -> Tuple[int, int, int]:
        return self.grid.shape

    def step(self) -> None:
        """One FDTD step in MEEP's ``fields::step()`` order (two fused kernels)."""
        self.step_many(1)

    def step_many(self, nsteps: int) -> None:
        if self.engine is None:
            self._freeze()
        if any(name[0] == "E" for name in self._absent) and self.grid.has_symmetry:
            for _ in range(int(nsteps)):
                self.engine.step(self.step_count, 1)
                self._clear_absent()
                self.step_count += 1
            return
        self.engine.step(self.step_count, int(nsteps))
        self.step_count += int(nsteps)

    @property
    def has_polarizations(self) -> bool:
        return any(any(v is not None for v in volumes) for _, volumes in self._poles)

    def field_energy(self) -> float:
        """``sum |E|^2 eps + |B|^2`` over the grid in float64, reduced on the device
        (reference ``_field_energy``, driver.py:3634); 0 before the first step."""
        if self.engine is None:
            return 0.0
        return self.engine.field_energy()

    def last_source_time(self) -> float:
        """The latest time any source emits (reference ``_last_source_time``,
        driver.py:3918): a Gaussian's peak plus cutoff times width, a continuous
        source's end time."""
        latest = 0.0
        for source in self._sources:
            waveform = source.waveform
            if hasattr(waveform, "peak_time"):
                latest = max(latest, waveform.peak_time + waveform.cutoff * waveform.width)
            elif getattr(waveform, "end_time", None) is not None:
                latest = max(latest, float(waveform.end_time))
        return latest

    def sources_end_time(self) -> float:
        """Last time any source is on (Gaussian: peak + cutoff), MEEP's ``last_source_time``."""
        latest = 0.0
        for source in self._sources:
            waveform = source.waveform
            if hasattr(waveform, "peak_time"):
                latest = max(latest, waveform.peak_time + waveform.cutoff_time)
            elif getattr(waveform, "end_time", None) is not None:
                latest = max(latest, float(waveform.end_time))
        return latest

    def run(self, num_steps: Optional[int] = None, until: Optional[float] = None,
            progress_cb: Optional[Callable[[int, int], None]] = None,
            cancel_check: Optional[Callable[[], bool]] = None, progress_interval: int = 100, *,
            until_after_sources: Optional[float] = None, check_finite: bool = True, **unsupported) -> int:
        """Advance ``num_steps`` steps, or until a simulation time (reference driver.py:3667).

        Steps are queued in chunks of ``progress_interval``; between chunks the
        non-finite detector is read (one small device-to-host read) and the cancel
        and progress callbacks run. A dispersive run also stops at every multiple of
        ``STABILITY_CHECK_INTERVAL`` steps for the divergence guard's field energy
        (:class:`DivergenceGuard`). Returns the number of steps taken.
        """
        if unsupported:
            raise Unsupported(f"run options {sorted(unsupported)} are not supported by this engine")
        given = [x is not None for x in (num_steps, until, until_after_sources)]
        if sum(given) != 1:
            raise ValueError("give exactly one of num_steps, until, until_after_sources")
        if until_after_sources is not None:
            until = self.sources_end_time() + float(until_after_sources)
        if until is not None:
            end_time = float(until)
            if not math.isfinite(end_time) or end_time <= self.time:
                raise ValueError(f"until={until!r} is not beyond the current time {self.time}")
            total = int(math.ceil((end_time - self.time) / self.grid.dt - STEP_TOLERANCE))
        else:
            total = int(num_steps)
            if total != num_steps or total < 1:
                raise ValueError(f"num_steps must be a positive whole number, got {num_steps!r}")
        interval = max(1, int(progress_interval))
        guard = DivergenceGuard(self) if (check_finite and self.has_polarizations) else None
        started = time_module.perf_counter()
        completed = 0
        since_report = 0
        while completed < total:
            chunk = min(interval - since_report, total - completed)
            if guard is not None:
                chunk = min(chunk, guard.interval - self.step_count % guard.interval)
            self.step_many(chunk)
            completed += chunk
            since_report += chunk
            if guard is not None:
                guard.update()
            if since_report < interval and completed < total:
                continue
            since_report = 0
            if check_finite and self.engine.nonfinite():
                raise FdtdDivergence(f"a non-finite E was written by step {self.step_count}")
            if cancel_check is not None and cancel_check():
                raise FdtdCancelled(f"FDTD run cancelled after {self.step_count} steps")
            if progress_cb is not None:
                progress_cb(completed, total)
        if self.engine is not None:
            import torch
            torch.cuda.synchronize(self.engine.device)
        self.last_run_seconds = time_module.perf_counter() - started
        return total

    # --- read-out -------------------------------------------------------------------
    def get_field(self, component: str, cell_centered: bool = True) -> np.ndarray:
        """Host copy of one component: the stored Yee words, or their cell-centre values.

        The centred value is MEEP's ``get_array`` sum ``0.25 * (((a + b) + c) + d)``
        over the shift-0 neighbours (``0.5 * (a + b)`` with one such axis), with the
        PEC zero (or the periodic image) past the high face.
        """
        if component not in FIELD_COMPONENTS:
            raise ValueError(f"unknown component {component!r}; supported {FIELD_COMPONENTS}")
        if self.engine is None:
            return np.zeros(self.grid.shape, dtype=np.complex64 if self.complex_fields else np.float32)
        name = {"D": "D", "E": "E", "B": "B", "H": "H"}[component[0]] + component[1]
        raw = self.engine.field(name).detach().cpu().numpy().copy()
        if not cell_centered:
            return raw
        shifts = IYEE[component]
        axes = [a for a in range(3) if shifts[a] == 0]
        padded = raw
        for axis in axes:
            pad = [(0, 0)] * 3
            pad[axis] = (0, 1)
            if self.grid.is_mirrored(axis):
                # one past the stored rows of a folded axis: the metallic wall's zero, or on
                # a periodic fold the image about the second mirror (dft.folded_site)
                site = folded_site(self.grid, axis, 0, self.grid.shape[axis])
                if isinstance(site, tuple):
                    row, flipped = site
                    image = np.take(padded, [row], axis=axis)
                    if flipped:
                        image = image * self.grid.parity(component, axis)
                    padded = np.concatenate([padded, image.astype(padded.dtype)], axis=axis)
                else:
                    padded = np.pad(padded, pad)
            elif self.grid.is_metallic(axis):
                padded = np.pad(padded, pad)
            else:
                padded = np.pad(padded, pad, mode="wrap")
        n = self.grid.shape
        # On a Bloch-phased axis cell 0 of a shift-0 component stores the owned top point:
        # the word at ladder index 0 (the low face) is conj(eikna) times it.
        low_factor = {}
        for axis in axes:
            phase = self.grid.bloch_phase(axis)
            if phase is not None:
                line = np.ones(n[axis], dtype=np.complex64)
                line[0] = np.complex64(np.conj(phase))
                shape = [1, 1, 1]
                shape[axis] = n[axis]
                low_factor[axis] = line.reshape(shape)

        def view(offsets):
            term = padded[tuple(slice(o, o + n[a]) for a, o in enumerate(offsets))]
            for axis, factor in low_factor.items():
                if offsets[axis] == 0:
                    term = term * factor
            return term
        if not axes:
            return raw
        if len(axes) == 1:
            o = [0, 0, 0]
            o[axes[0]] = 1
            return (np.float32(0.5) * (view((0, 0, 0)) + view(o))).astype(raw.dtype)
        a0, a1 = axes
        o1 = [0, 0, 0]; o1[a0] = 1
        o2 = [0, 0, 0]; o2[a1] = 1
        o3 = [0, 0, 0]; o3[a0] = 1; o3[a1] = 1
        total = ((view((0, 0, 0)) + view(o1)) + view(o2)) + view(o3)
        return (np.float32(0.25) * total).astype(raw.dtype)

    def get_flux_spectrum(self, monitor: FluxMonitor) -> np.ndarray:
        return monitor.get_flux_spectrum()

    def close(self) -> None:
        if self.engine is not None:
            self.engine.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
