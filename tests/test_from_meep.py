"""The MEEP entry points (``lift_simulation``, ``run_on_gpu``, ``GpuRunResult``) against a
duck-typed stand-in for ``mp.Simulation`` (``tests/fake_meep.py``; MEEP itself is absent
here and on the GPU machine).

On the CPU: the lift reads the cell, clock, structure (both permittivity routes),
dispersion, conductivity, layers, sources and monitors into a driver configured like
the same run built by hand on ``FdtdDriver``, and refuses what the engine does not step
by name. On the GPU: ``run_on_gpu`` steps the lifted run to the hand-built run's words
and spectra, and the two-run normalisation goes through ``minus_flux_data``.
"""

import sys

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from meep_gpu_gb300.from_meep import (GpuRunResult, MeepSimulationNotLiftable, lift_simulation, run_on_gpu,
                                      yee_points)
from meep_gpu_gb300.grid import Unsupported
from tests import fake_meep as mp

CELL = (2.4, 2.0, 2.2)
FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


@pytest.fixture(autouse=True)
def meep_module(monkeypatch):
    monkeypatch.setitem(sys.modules, "meep", mp)
    return mp


def standin(sphere_eps=4.0, lossy=False, periodic=False, **kwargs):
    slab = mp.Medium(epsilon=2.25, E_susceptibilities=[mp.LorentzianSusceptibility(1.1, 0.05, 1.5)])
    sphere = mp.Medium(epsilon=sphere_eps, D_conductivity=0.3 if lossy else 0.0)
    geometry = [mp.Block(mp.Vector3(0.4, 1e20, 1e20), center=mp.Vector3(0.1, 0, 0), material=slab),
                mp.Sphere(0.35, center=mp.Vector3(-0.2, 0.1, 0.0), material=sphere)]
    layers = [mp.PML(0.3)] if not lossy else [mp.PML(0.3, direction=mp.X), mp.Absorber(0.25, direction=mp.Z,
                                                                                    side=mp.High)]
    sources = [mp.Source(mp.GaussianSource(0.8, fwidth=1.0), component=mp.Ez, center=mp.Vector3(-0.6, 0.03, 0)),
               mp.Source(mp.ContinuousSource(0.3, end_time=4.0), component=mp.Hx,
                         center=mp.Vector3(0.05, -0.1, 0.07), size=mp.Vector3(0, 0.3, 0), amplitude=0.5)]
    sim = mp.Simulation(mp.Vector3(*CELL), 10, geometry=geometry, boundary_layers=layers, sources=sources,
                        k_point=mp.Vector3(0, 0, 0) if periodic else False, **kwargs)
    flux = sim.add_flux(0.8, 0.5, 5, mp.FluxRegion(mp.Vector3(0.6, 0, 0), mp.Vector3(0, 1.2, 1.4)))
    dft = sim.add_dft_fields([mp.Ex, mp.Ez], 0.8, 0.2, 2, mp.Vector3(0, 0, 0), mp.Vector3(0.6, 0.5, 0.4),
                             decimation_factor=2)
    return sim, flux, dft


def hand_built(lossy=False, periodic=False, sphere_eps=4.0):
    """The same run configured directly on FdtdDriver, its structure sampled here."""
    d = FdtdDriver(CELL, 10, courant=0.5, force_complex_fields=False,
                   boundaries="periodic" if periodic else "metallic")
    grid = d.grid

    def sample(component, slab_value, sphere_value, background):
        x, y, z = (t.reshape(s) for t, s in zip(yee_points(grid, component), ((-1, 1, 1), (1, -1, 1), (1, 1, -1))))
        out = np.full(grid.shape, background)
        out[np.broadcast_to(np.abs(x - 0.1) <= 0.2, grid.shape)] = slab_value
        sphere = (x + 0.2) ** 2 + (y - 0.1) ** 2 + z ** 2 <= 0.35 ** 2
        out[np.broadcast_to(sphere, grid.shape)] = sphere_value
        return out

    d.set_epsilon_components(*(sample(c, 2.25, sphere_eps, 1.0) for c in ("Ex", "Ey", "Ez")))
    d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05),
                         {c: sample(c, 1.5, 0.0, 0.0).astype(np.float32) for c in ("Ex", "Ey", "Ez")})
    if lossy:
        d.set_conductivity({c: sample(c, 0.0, 0.3, 0.0).astype(np.float32) for c in ("Dx", "Dy", "Dz")})
        d.setup_pml({"x": 3.0})
        from meep_gpu_gb300 import AbsorberLayer
        d.set_absorber([AbsorberLayer(0.25, 2, "high")])
    else:
        d.setup_pml({a: {"low": 3.0, "high": 3.0} for a in "xyz"})
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.6, 0.03, 0.0), "size": (0, 0, 0),
                  "frequency": 0.8, "fwidth": 1.0})
    d.add_source({"source_type": "continuous", "component": "Hx", "center": (0.05, -0.1, 0.07),
                  "size": (0, 0.3, 0), "frequency": 0.3, "end_time": 4.0, "amplitude": 0.5})
    flux = d.add_flux_monitor(list(np.linspace(0.55, 1.05, 5)), center=(0.6, 0, 0), size=(0, 1.2, 1.4),
                              decimation_factor=0)
    dft = d.add_dft_monitor(list(np.linspace(0.7, 0.9, 2)), components=("Ex", "Ez"), center=(0, 0, 0),
                            size=(0.6, 0.5, 0.4), decimation_factor=2)
    return d, flux, dft


@pytest.mark.parametrize("lossy", [False, True])
def test_lift_configures_the_hand_built_run(lossy):
    sim, _, _ = standin(lossy=lossy)
    lifted = lift_simulation(sim)
    built, _, _ = hand_built(lossy=lossy)
    assert sim.initialized == 1
    assert lifted.grid.shape == built.grid.shape and lifted.dt == built.dt
    assert lifted.complex_fields is False
    for a, b in zip(lifted._eps, built._eps):
        assert np.array_equal(a, b)
    assert len(lifted._poles) == len(built._poles) == 1
    (pole_a, sig_a), (pole_b, sig_b) = lifted._poles[0], built._poles[0]
    assert pole_a == pole_b
    for a, b in zip(sig_a, sig_b):
        assert np.array_equal(a, b)
    assert lifted.pml.faces == built.pml.faces
    for name, volume in built.conductivity_volumes().items():
        got = lifted.conductivity_volumes()[name]
        assert (got is None and volume is None) or np.array_equal(got, volume), name
    assert [s.component for s in lifted.sources] == [s.component for s in built.sources]
    assert lifted.last_source_time() == built.last_source_time()
    lifted.prepare()
    built.prepare()
    for a, b in zip(lifted.sources, built.sources):
        assert len(a.cells) > 0
        assert np.array_equal(np.asarray(a.cells), np.asarray(b.cells))
        assert np.array_equal(np.asarray(a.amps), np.asarray(b.amps))
    fa, fb = lifted._flux_monitors[0], built._flux_monitors[0]
    assert np.array_equal(fa.frequencies, fb.frequencies) and fa.region == fb.region
    assert fa.decimation_factor == fb.decimation_factor
    da, db = lifted._dft_monitors[0], built._dft_monitors[0]
    assert da.region == db.region and da.components == db.components and da.decimation_factor == 2


def test_both_permittivity_routes_read_the_same_words():
    small = dict(sphere_eps=6.0)
    a, _, _ = standin(**small)
    b, _, _ = standin(eps_averaging=True, **small)
    planes = []
    grid_route = lift_simulation(a)
    chi1inv_route = lift_simulation(b, progress_cb=lambda done, total: planes.append((done, total)))
    assert chi1inv_route.lift_record["epsilon_route"] == "chi1inv"
    assert grid_route.lift_record["epsilon_route"] == "grid"
    for x, y in zip(grid_route._inv_eps, chi1inv_route._inv_eps):
        assert np.array_equal(x, y)
    assert planes[-1][0] == planes[-1][1] == 3 * grid_route.grid.shape[0]


def test_periodic_and_complex_and_symmetric_cells():
    sim, _, _ = standin(periodic=True)
    driver = lift_simulation(sim)
    assert all(not driver.grid.is_metallic(a) for a in range(3))
    sim, _, _ = standin(force_complex_fields=True)
    assert lift_simulation(sim).complex_fields
    sim = mp.Simulation(mp.Vector3(*CELL), 10, symmetries=[mp.Mirror(mp.Y, phase=1)],
                        sources=[mp.Source(mp.GaussianSource(0.8, 1.0), mp.Ez, mp.Vector3(-0.6, 0, 0))])
    driver = lift_simulation(sim)
    assert driver.grid.is_mirrored(1) and not driver.grid.is_mirrored(0)


def test_lift_refuses_what_the_engine_does_not_step_by_name():
    cases = []
    sim, _, _ = standin()
    sim.is_cylindrical = True
    cases.append((sim, "cylindrical"))
    sim, _, _ = standin()
    sim.cell_size = mp.Vector3(2.4, 0, 0)  # a zero extent on y with x resolved
    cases.append((sim, "dimensions"))
    sim, _, _ = standin()
    sim.dft_objects.append(mp.DftForce([0.5], [mp.FluxRegion(mp.Vector3(), mp.Vector3(0, 1, 1))], 0))
    cases.append((sim, "DftForce"))
    sim, _, _ = standin()
    sim.sources[0].src.is_integrated = True
    cases.append((sim, "integrated"))
    sim, _, _ = standin()
    sim.geometry[1].material.mu_diag = mp.Vector3(2, 2, 2)
    cases.append((sim, "mu"))
    sim, _, _ = standin()
    sim.add_flux(0.5, 0.1, 3, mp.FluxRegion(mp.Vector3(), mp.Vector3(0, 1, 1)),
                 mp.FluxRegion(mp.Vector3(0.1, 0, 0), mp.Vector3(0, 1, 1)))
    cases.append((sim, "more than one FluxRegion"))
    for sim, words in cases:
        with pytest.raises(MeepSimulationNotLiftable, match=words):
            lift_simulation(sim)
        assert sim.initialized == 0, "refused before MEEP built anything"
    sim, _, _ = standin()
    with pytest.raises(Unsupported, match="CPU"):
        lift_simulation(sim, prefer_gpu=False)


def test_run_on_gpu_refuses_bad_stop_conditions_before_lifting():
    sim, _, _ = standin()
    with pytest.raises(ValueError, match="exactly one"):
        run_on_gpu(sim)
    with pytest.raises(ValueError, match="exactly one"):
        run_on_gpu(sim, until=3, until_after_sources=2)
    with pytest.raises(TypeError, match="simulation time"):
        run_on_gpu(sim, until=lambda s: True)
    assert sim.initialized == 0


def test_migrated_monitors_resolve_by_identity():
    sim, flux, dft = standin()
    driver = lift_simulation(sim)
    result = GpuRunResult(driver=driver, steps=0, meep_time=0.0, wall_time_s=0.0)
    assert result.monitor_for(flux) is driver._flux_monitors[0]
    assert result.monitor_for(dft) is driver._dft_monitors[0]
    twin, _, _ = standin()
    with pytest.raises(KeyError, match="not migrated"):
        result.monitor_for(twin.dft_objects[0])
    assert len(result.monitors) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("lossy", [False, True])
def test_run_on_gpu_steps_the_hand_built_run(gpu, lossy):
    sim, flux, dft = standin(lossy=lossy)
    result = run_on_gpu(sim, until_after_sources=3.0)
    built, bflux, bdft = hand_built(lossy=lossy)
    end = sim.fields.last_source_time() + 3.0
    built.run(until=end)
    assert result.steps == built.step_count and result.meep_time == built.time
    for c in FIELDS:
        assert np.array_equal(result.get_field(c, cell_centered=False), built.get_field(c, cell_centered=False)), c
    assert np.array_equal(result.get_flux_spectrum(flux), bflux.get_flux_spectrum())
    assert np.array_equal(result.get_dft_array(dft, "Ez", 1), bdft.raw("Ez")[1])
    array = result.get_array("Ez")
    assert array.shape == built.grid.shape  # metallic axes: no duplicate plane
    assert np.array_equal(array, built.get_field("Ez"))
    result.close()
    built.close()


@pytest.mark.gpu
def test_get_array_carries_meeps_duplicate_plane_on_periodic_axes(gpu):
    sim, _, _ = standin(periodic=True)
    result = run_on_gpu(sim, until=2.0)
    array = result.get_array("Hy")
    centred = result.get_field("Hy")
    assert array.shape == tuple(n + 1 for n in centred.shape)
    assert np.array_equal(array[1:, 1:, 1:], centred)
    assert np.array_equal(array[0, 1:, 1:], centred[-1])
    result.close()


@pytest.mark.gpu
def test_two_run_normalisation_through_minus_flux_data(gpu):
    vacuum, flux1, _ = standin(sphere_eps=1.0)
    first = run_on_gpu(vacuum, until=6.0)
    data = first.get_flux_data(flux1)
    first.close()
    structure, flux2, _ = standin()
    second = run_on_gpu(structure, until=6.0, minus_flux_data=[(flux2, data)])
    # the same on FdtdDriver directly
    d1, f1, _ = hand_built(sphere_eps=1.0)
    d1.run(until=6.0)
    d2, f2, _ = hand_built()
    f2.load_minus_dft_data(f1.get_dft_data())
    d2.run(until=6.0)
    assert np.array_equal(second.get_flux_spectrum(flux2), f2.get_flux_spectrum())
    second.close()
    d1.close()
    d2.close()


def test_a_2d_simulation_lifts_to_the_hand_built_2d_run():
    """A cell with no z extent is MEEP's 2-D run: one periodic cell on the invariant z, a
    PML on the two resolved axes only, the other polarization recorded as absent, and a
    flux line; the lifted run's float32 oracle words equal the hand-built run's."""
    from oracle.oracle import Oracle, problem_from_driver

    disk = mp.Medium(epsilon=4.0)
    sim = mp.Simulation(mp.Vector3(2.0, 1.6, 0), 10, geometry=[mp.Cylinder(0.3, material=disk)],
                        boundary_layers=[mp.PML(0.3)],
                        sources=[mp.Source(mp.GaussianSource(0.8, fwidth=1.0), component=mp.Ez,
                                           center=mp.Vector3(-0.5, 0.03, 0))])
    sim.add_flux(0.8, 0.5, 4, mp.FluxRegion(mp.Vector3(0.5, 0, 0), mp.Vector3(0, 1.0, 0)))
    lifted = lift_simulation(sim)
    assert lifted.grid.dimensions == 2 and lifted.grid.shape == (20, 16, 1)
    assert lifted.pml.faces[2] == (0.0, 0.0)
    assert set(lifted.absent_components) == {"Ex", "Ey", "Dx", "Dy", "Hz", "Bz"}
    d = FdtdDriver((2.0, 1.6, 0.0), 10, force_complex_fields=False, dimensions=2,
                   boundaries={"x": "metallic", "y": "metallic"})
    xs, ys, _ = yee_points(d.grid, "Ez")
    eps = np.where((xs[:, None, None] ** 2 + ys[None, :, None] ** 2) <= 0.3 ** 2, 4.0, 1.0)
    d.set_epsilon(np.broadcast_to(eps, d.grid.shape))
    d.setup_pml({"x": 3.0, "y": 3.0})
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.5, 0.03, 0.0), "size": (0, 0, 0),
                  "frequency": 0.8, "fwidth": 1.0})
    d.add_flux_monitor(list(np.linspace(0.55, 1.05, 4)), center=(0.5, 0, 0), size=(0, 1.0, 0),
                       decimation_factor=0)
    runs = []
    for driver in (lifted, d):
        oracle = Oracle(problem_from_driver(driver), "f32")
        oracle.run(40)
        runs.append(oracle)
    for c in FIELDS:
        assert np.array_equal(runs[0].field(c), runs[1].field(c)), c
    assert np.array_equal(runs[0].flux_spectrum(0), runs[1].flux_spectrum(0))
