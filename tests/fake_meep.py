"""A duck-typed stand-in for the parts of MEEP's Python API the lift reads.

MEEP is not installed here or on the GPU machine, so the lift (``meep_gpu_gb300.from_meep``)
is tested against this module, installed as ``sys.modules["meep"]`` by the tests. It
carries MEEP's component, direction and side constants, the class names the lift keys
on (``Medium``, ``LorentzianSusceptibility``, ``Block``, ``Sphere``, ``PML``,
``Absorber``, ``Source``, ``GaussianSource``, ``FluxRegion`` ...) and a ``Simulation``
whose structure queries (``get_epsilon_grid``, ``fields.get_chi1inv``) point-sample its
geometry (later objects over earlier ones, no subpixel smoothing).
"""

from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np

__version__ = "stand-in"

# MEEP's component, direction and side numbering (meep.i / meep.hpp)
Ex, Ey, Er, Ep, Ez, Hx, Hy, Hr, Hp, Hz = range(10)
Dx, Dy, Dr, Dp, Dz, Bx, By, Br, Bp, Bz = range(10, 20)
Dielectric, Permeability = 20, 21
X, Y, Z, R, P = 0, 1, 2, 4, 5
ALL = -1
AUTOMATIC = -1
Low, High = 0, 1


class Vector3:
    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def __iter__(self):
        return iter((self.x, self.y, self.z))


class Medium:
    def __init__(self, epsilon=1.0, E_susceptibilities=(), D_conductivity=0.0, B_conductivity=0.0):
        self.epsilon_diag = Vector3(epsilon, epsilon, epsilon)
        self.E_susceptibilities = list(E_susceptibilities)
        self.D_conductivity = D_conductivity
        self.B_conductivity = B_conductivity


class LorentzianSusceptibility:
    def __init__(self, frequency=0.0, gamma=0.0, sigma=0.0):
        self.frequency, self.gamma, self.sigma = frequency, gamma, sigma


class DrudeSusceptibility(LorentzianSusceptibility):
    pass


class Block:
    def __init__(self, size, center=None, material=None):
        self.size, self.center, self.material = size, center or Vector3(), material


class Sphere:
    def __init__(self, radius, center=None, material=None):
        self.radius, self.center, self.material = radius, center or Vector3(), material


class Cylinder:
    def __init__(self, radius, height=math.inf, axis=None, center=None, material=None):
        self.radius, self.height = radius, height
        self.axis = axis or Vector3(0, 0, 1)
        self.center, self.material = center or Vector3(), material


class PML:
    def __init__(self, thickness, direction=ALL, side=ALL, R_asymptotic=1e-15):
        self.thickness, self.direction, self.side, self.R_asymptotic = thickness, direction, side, R_asymptotic


class Absorber(PML):
    pass


class Mirror:
    def __init__(self, direction, phase=1):
        self.direction, self.phase = direction, phase


class GaussianSource:
    def __init__(self, frequency, fwidth, start_time=0.0, cutoff=5.0, is_integrated=False):
        self.frequency, self.fwidth, self.start_time, self.cutoff = frequency, fwidth, start_time, cutoff
        self.is_integrated = is_integrated

    def last_time(self):
        width = 1.0 / self.fwidth
        return self.start_time + 2 * self.cutoff * width


class ContinuousSource:
    def __init__(self, frequency, start_time=0.0, end_time=1e20, width=0.0, slowness=3.0, is_integrated=False):
        self.frequency, self.start_time, self.end_time = frequency, start_time, end_time
        self.width, self.slowness, self.is_integrated = width, slowness, is_integrated

    def last_time(self):
        return self.end_time


class Source:
    def __init__(self, src, component, center, size=None, amplitude=1.0, amp_func=None):
        self.src, self.component, self.center = src, component, center
        self.size, self.amplitude, self.amp_func = size or Vector3(), amplitude, amp_func


class FluxRegion:
    def __init__(self, center, size, direction=AUTOMATIC, weight=1.0):
        self.center, self.size, self.direction, self.weight = center, size, direction, weight


class DftFlux:
    def __init__(self, freq, regions, decimation_factor):
        self.freq, self.regions, self.decimation_factor = list(freq), list(regions), decimation_factor


class DftFields:
    def __init__(self, components, freq, center, size, decimation_factor):
        self.components, self.freq = list(components), list(freq)
        self.where = SimpleNamespace(center=center, size=size)
        self.decimation_factor = decimation_factor


class DftForce(DftFlux):
    pass


def _inside(obj, x, y, z):
    c = obj.center
    if isinstance(obj, Block):
        s = obj.size
        return (np.abs(x - c.x) <= s.x / 2) & (np.abs(y - c.y) <= s.y / 2) & (np.abs(z - c.z) <= s.z / 2)
    if isinstance(obj, Sphere):
        return (x - c.x) ** 2 + (y - c.y) ** 2 + (z - c.z) ** 2 <= obj.radius ** 2
    if isinstance(obj, Cylinder):
        axis = int(np.argmax(np.abs([obj.axis.x, obj.axis.y, obj.axis.z])))
        coords, centre = (x, y, z), (c.x, c.y, c.z)
        a, b = [i for i in range(3) if i != axis]
        r2 = (coords[a] - centre[a]) ** 2 + (coords[b] - centre[b]) ** 2
        return (r2 <= obj.radius ** 2) & (np.abs(coords[axis] - centre[axis]) <= obj.height / 2)
    raise TypeError(type(obj).__name__)


class _Fields:
    def __init__(self, sim):
        self._sim = sim
        self.is_real = not (sim.force_complex_fields or bool(sim.k_point))

    def last_source_time(self):
        return max([s.src.last_time() for s in self._sim.sources] + [0.0])

    def have_component(self, component):
        """MEEP allocates a component with every one "like" it: in a 2-D cell (zero z
        extent) the polarization of some source, in 3-D everything."""
        cell = self._sim.cell_size
        if cell.z != 0:
            return True
        names = {Ex: "Ex", Ey: "Ey", Ez: "Ez", Hx: "Hx", Hy: "Hy", Hz: "Hz",
                 Dx: "Dx", Dy: "Dy", Dz: "Dz", Bx: "Bx", By: "By", Bz: "Bz"}
        families = (("Ez", "Dz", "Hx", "Hy", "Bx", "By"), ("Ex", "Ey", "Dx", "Dy", "Hz", "Bz"))
        sourced = {names.get(src.component) for src in self._sim.sources}
        return any(names.get(component) in family and sourced & set(family) for family in families)

    def get_chi1inv(self, component, direction, loc, frequency=0.0):
        assert frequency == 0
        eps = self._sim.get_epsilon_grid(np.array([loc.x]), np.array([loc.y]), np.array([loc.z]))
        return 1.0 / float(eps[0, 0, 0])


class Simulation:
    def __init__(self, cell_size, resolution, geometry=(), default_material=None, boundary_layers=(),
                 sources=(), symmetries=(), k_point=False, force_complex_fields=False, Courant=0.5,
                 eps_averaging=False, dimensions=3):
        self.cell_size, self.resolution = cell_size, resolution
        self.geometry = list(geometry)
        self.default_material = default_material or Medium()
        self.boundary_layers, self.sources = list(boundary_layers), list(sources)
        self.symmetries, self.k_point = list(symmetries), k_point
        self.force_complex_fields, self.Courant = force_complex_fields, Courant
        self.eps_averaging, self.dimensions = eps_averaging, dimensions
        self.dft_objects = []
        self.fields = None
        self.initialized = 0

    def init_sim(self):
        self.initialized += 1
        self.fields = _Fields(self)

    def add_flux(self, fcen, df, nfreq, *regions, decimation_factor=0):
        freq = np.linspace(fcen - df / 2, fcen + df / 2, nfreq) if nfreq > 1 else [fcen]
        flux = DftFlux(freq, regions, decimation_factor)
        self.dft_objects.append(flux)
        return flux

    def add_dft_fields(self, components, fcen, df, nfreq, center, size, decimation_factor=0):
        freq = np.linspace(fcen - df / 2, fcen + df / 2, nfreq) if nfreq > 1 else [fcen]
        dft = DftFields(components, freq, center, size, decimation_factor)
        self.dft_objects.append(dft)
        return dft

    def get_epsilon_grid(self, xtics, ytics, ztics, frequency=0):
        x = np.asarray(xtics, dtype=np.float64).reshape(-1, 1, 1)
        y = np.asarray(ytics, dtype=np.float64).reshape(1, -1, 1)
        z = np.asarray(ztics, dtype=np.float64).reshape(1, 1, -1)
        shape = np.broadcast(x, y, z).shape
        eps = np.full(shape, self.default_material.epsilon_diag.x)
        for obj in self.geometry:
            eps[np.broadcast_to(_inside(obj, x, y, z), shape)] = obj.material.epsilon_diag.x
        return eps
