"""Small seeded cases shared by the golden-vector script and the tests.

Each case is built through whichever driver class is passed in (the reference's
``meep_gpu.FdtdDriver`` when recording, ``meep_gpu_gb300.FdtdDriver`` when testing), with
the same calls, so both sides configure the same simulation.
"""

from __future__ import annotations

import numpy as np

CASES = {
    "sphere_pml": dict(n=(14, 12, 16), pml=3, steps=60),
    "lorentz_slab": dict(n=(16, 12, 14), pml=3, steps=60, lorentz=True),
    "nopml_metallic": dict(n=(12, 14, 13), pml=0, steps=50),
    "periodic": dict(n=(12, 13, 14), pml=0, steps=50, boundaries="periodic"),
    "periodic_pml": dict(n=(14, 12, 13), pml=3, steps=50, boundaries="periodic"),
    "mixed": dict(n=(13, 15, 12), pml={"x": 3, "y": {"low": 2, "high": 4}, "z": 2.5}, steps=45,
                  mixed=True),
    # z extents that are multiples of 4 (the shared-memory tile path), with partial tiles
    # in y and z, a z extent spanning two tiles, and periodic faces in every axis.
    "tile_periodic_pml": dict(n=(12, 14, 20), pml=3, steps=50, boundaries="periodic"),
    "tile_lorentz": dict(n=(16, 10, 24), pml=3, steps=50, lorentz=True),
    "tile_periodic": dict(n=(10, 12, 16), pml=0, steps=40, boundaries="periodic"),
    "tile_mixed": dict(n=(11, 18, 68), pml={"x": 2, "y": {"low": 3, "high": 2}, "z": 4}, steps=40,
                       mixed=True),
    # D and B conductivity under a PML: a D-lossy band |x| < 0.25 that runs through the y
    # and z layers (the x-layer chunks keep no D conductivity; the others take all four
    # conductive forms), a B-lossy block reaching one corner, the source two cells inside
    # the layers.
    "cond_pml": dict(n=(14, 12, 16), pml=3, steps=60, conductivity="band"),
    # A lossy run without PML: a graded absorber on all six faces plus a uniform D
    # conductivity (the two add).
    "absorber": dict(n=(13, 12, 14), pml=0, steps=60, conductivity="absorber"),
    # Periodic axes, PML on x only, a one-sided absorber on each z face (different
    # thicknesses), per-component D conductivity and a Lorentz pole.
    "absorber_pml_periodic": dict(n=(14, 12, 16), pml={"x": 3}, steps=50, boundaries="periodic",
                                  conductivity="mixed", lorentz=True),
    # Magnetic sources (a Gaussian Hx point and a CW Hz sheet) beside the Ez one, under a
    # PML; and again in a lossy run without PML (absorber, D and B conductivity), where
    # the magnetic deposit carries B's condinv.
    "magnetic": dict(n=(14, 12, 16), pml=3, steps=60, magnetic=True),
    "magnetic_lossy": dict(n=(13, 14, 12), pml=0, steps=60, magnetic=True, conductivity="absorber_b"),
    # Complex fields (the reference's default) at k = 0: the mixed case's sources (a
    # complex-amplitude one added), poles and monitors, periodic y; and with a lossy
    # PML run and magnetic sources.
    "complex_mixed": dict(n=(13, 15, 12), pml={"x": 3, "z": 2}, steps=45, mixed=True, complex=True,
                          boundaries=("metallic", "periodic", "metallic")),
    "complex_cond": dict(n=(14, 12, 16), pml=3, steps=50, conductivity="band", magnetic=True,
                         complex=True),
    # Complex fields on the sphere case (a complex source amplitude): the case the serving
    # batch's complex slots are checked on (at most two monitors).
    "complex_sphere": dict(n=(14, 12, 16), pml=3, steps=60, complex=True, complex_amplitude=True),
    # The sphere case on a Bloch lattice (periodic x and y, k = (0.3, -0.2, 0), a z PML):
    # the case the serving batch's Bloch slots are checked on (one monitor).
    "bloch_sphere": dict(n=(14, 12, 16), pml={"z": 3}, steps=60, complex=True, boundaries=("periodic", "periodic", "metallic"),
                         k_point=(0.3, -0.2, 0.0)),
    # The Bloch sphere case with magnetic sources (a Gaussian Hx point, a CW Hz sheet):
    # the magnetic deposit of the batch's phased (index-0) CTAs.
    "bloch_magnetic": dict(n=(14, 12, 16), pml={"z": 3}, steps=60, complex=True,
                           boundaries=("periodic", "periodic", "metallic"), k_point=(0.3, -0.2, 0.0),
                           magnetic=True),
    # Bloch-periodic fields (complex, k != 0): phased x and y with an interior point
    # source, a DFT volume and a flux plane spanning the whole y-z cross-section; and
    # a phased x axis under a z PML with a line source wrapping the phased axis, odd
    # and even counts.
    "bloch": dict(n=(12, 13, 14), pml=0, steps=50, complex=True, boundaries="periodic",
                  k_point=(0.3, -0.2, 0.0), bloch_monitors=True),
    "bloch_pml": dict(n=(15, 12, 16), pml={"z": 3}, steps=50, complex=True, boundaries="periodic",
                      k_point=(0.45, 0.0, 0.0), bloch_line=True, bloch_monitors=True),
    # Mirror symmetry (folded metallic axes): an even X and an odd Y plane under a PML
    # (the scalar thickness skips the planes' faces) with a Lorentz slab across the x
    # plane; an odd Z plane on an odd count with an absorber (its low face lands on no
    # stored cell), D and B conductivity; complex fields with an even Z plane beside a
    # periodic y axis. Sources in the stored half (one on the x plane, one sheet across
    # it), a flux plane and a DFT volume spanning both halves of every plane.
    "mirror_pml": dict(n=(14, 12, 16), pml=3, steps=60, symmetry=(("X", 1), ("Y", -1)),
                       mirror_sources=True, lorentz=True),
    "mirror_odd_lossy": dict(n=(13, 12, 15), pml=0, steps=60, symmetry=(("Z", -1),),
                             conductivity="absorber_b", mirror_sources=True),
    "mirror_complex": dict(n=(12, 14, 14), pml={"x": 3, "z": {"high": 2}}, steps=50,
                           symmetry=(("Z", 1),), complex=True, mirror_sources=True,
                           boundaries=("metallic", "periodic", "metallic")),
    # Folds of periodic axes (one more stored cell: MEEP's big_corner plane and the far
    # ghost slot past the second mirror): an even count and an odd one, without an
    # absorber, with a Lorentz slab; and a PML on a folded periodic axis's high face.
    "mirror_periodic": dict(n=(14, 13, 12), pml={"z": 3}, steps=60, symmetry=(("X", 1), ("Y", -1)),
                            boundaries="periodic", mirror_sources=True, lorentz=True),
    "mirror_periodic_pml": dict(n=(16, 12, 13), pml={"z": {"high": 3}, "x": 2}, steps=50,
                                symmetry=(("Z", -1),), boundaries=("metallic", "periodic", "periodic"),
                                mirror_sources=True),
    # A conductivity under a PML on a folded periodic axis (its chunks cut MEEP's window,
    # the far ghost slot taking the top one).
    "mirror_periodic_lossy": dict(n=(14, 16, 12), pml={"y": {"high": 3}, "x": 2}, steps=50,
                                  symmetry=(("Y", 1),), boundaries=("metallic", "periodic", "metallic"),
                                  mirror_sources=True, conductivity="band"),
    # A 2-D run (z invariant: one periodic cell): a dielectric cylinder, a Lorentz block,
    # both polarizations driven (an Ez and an Hz Gaussian point), PML on x and y, flux
    # lines normal to x and y and a DFT area.
    "two_d": dict(n=(16, 14, 0), pml=3, steps=60, dims=2),
    # A 1-D run along z (x and y invariant): an absorber-free PML line, an Ex Gaussian
    # point, a Drude pole, a z-normal flux point and a DFT segment.
    "one_d": dict(n=(0, 0, 40), pml=4, steps=80, dims=1),
}

# The 80^3 sphere-under-PML workload (resolution 10, 10-cell PML, eps 4 sphere of radius
# 2, Ez Gaussian at x = -2, one 50-frequency x-normal flux plane at x = 2.5).
SPHERE80 = dict(n=(80, 80, 80), pml=10, steps=200, sphere80=True)
# The same workload over its full 2000 steps.
SPHERE80_FULL = dict(SPHERE80, steps=2000)


def _build_reduced(driver_cls, susceptibility_cls, case: dict, reference: bool):
    """A 2-D (z invariant) or 1-D (along z) case: MEEP's spelling, a zero extent on each
    invariant axis."""
    res = 10
    dims = case["dims"]
    lengths = tuple(v / res for v in case["n"])
    boundaries = {"x": "metallic", "y": "metallic"} if dims == 2 else {"z": "metallic"}
    d = driver_cls(cell_size=lengths, resolution=res, courant=0.5, force_complex_fields=False,
                   boundaries=boundaries, dimensions=dims, **({"prefer_gpu": False} if reference else {}))
    d.setup_pml({"x": case["pml"], "y": case["pml"]} if dims == 2 else {"z": case["pml"]})
    x, y, z = d.grid.meshgrid()
    flux, dft = [], []
    if dims == 2:
        d.set_epsilon(np.where(x ** 2 + y ** 2 < 0.3 ** 2, 4.0, 1.0).astype(np.float32))
        block = (np.abs(x - 0.3) < 0.15) & (np.abs(y) < 0.3)
        d.add_susceptibility(susceptibility_cls(frequency=0.9, gamma=0.1),
                             np.where(block, 0.8, 0.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.4, 0.03, 0.0),
                      "size": (0, 0, 0), "frequency": 0.6, "fwidth": 0.5})
        d.add_source({"source_type": "gaussian", "component": "Hz", "center": (-0.35, -0.1, 0.0),
                      "size": (0, 0, 0), "frequency": 0.5, "fwidth": 0.4, "amplitude": 0.7})
        flux.append(d.add_flux_monitor(fcen=0.6, df=0.3, nfreq=4, center=(0.45, 0.0, 0.0),
                                       size=(0, 0.8, 0), decimation_factor=1))
        flux.append(d.add_flux_monitor(frequencies=[0.4, 0.55], center=(0.0, 0.35, 0.0),
                                       size=(0.9, 0, 0), decimation_factor=2))
        dft.append(d.add_dft_monitor(frequencies=[0.5, 0.7], components=("Ez", "Hx", "Hz"),
                                     center=(0.1, 0.0, 0.0), size=(0.6, 0.5, 0), decimation_factor=1))
    else:
        d.set_epsilon(np.where(np.abs(z) < 0.5, 2.5, 1.0).astype(np.float32))
        d.add_susceptibility(susceptibility_cls(frequency=0.6, gamma=0.2, kind="drude"),
                             np.where(np.abs(z) < 0.5, 0.4, 0.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ex", "center": (0.0, 0.0, -1.0),
                      "size": (0, 0, 0), "frequency": 0.7, "fwidth": 0.6})
        flux.append(d.add_flux_monitor(fcen=0.7, df=0.4, nfreq=5, center=(0.0, 0.0, 1.0),
                                       size=(0, 0, 0), decimation_factor=1))
        dft.append(d.add_dft_monitor(frequencies=[0.6, 0.8], components=("Ex", "Hy"),
                                     center=(0.0, 0.0, 0.2), size=(0, 0, 0.6), decimation_factor=1))
    return d, flux, dft


def build_case(driver_cls, susceptibility_cls, case: dict, reference: bool = False):
    """Configure one case; returns (driver, flux monitors, DFT monitors)."""
    if case.get("dims"):
        return _build_reduced(driver_cls, susceptibility_cls, case, reference)
    res = 10
    n = case["n"]
    lengths = tuple(v / res for v in n)
    boundaries = case.get("boundaries", "metallic")
    symmetry = ()
    if case.get("symmetry"):
        if reference:
            from meep_gpu.grid import Mirror
        else:
            from meep_gpu_gb300 import Mirror
        symmetry = tuple(Mirror(axis, phase) for axis, phase in case["symmetry"])
    d = driver_cls(cell_size=lengths, resolution=res, courant=0.5,
                   force_complex_fields=bool(case.get("complex", False)),
                   k_point=case.get("k_point", (0.0, 0.0, 0.0)), symmetry=symmetry,
                   boundaries=boundaries, **({"prefer_gpu": False} if reference else {}))
    if case["pml"]:
        d.setup_pml(case["pml"])
    x, y, z = d.grid.meshgrid()
    flux, dft = [], []
    if case.get("sphere80"):
        d.set_epsilon(np.where(x ** 2 + y ** 2 + z ** 2 < 2.0 ** 2, 4.0, 1.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.0, 0, 0),
                      "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
        flux.append(d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=50, center=(2.5, 0, 0),
                                       size=(0, 6, 6), decimation_factor=0))
        return d, flux, dft
    if case.get("lorentz"):
        inside = np.abs(x) < 0.2
        d.set_epsilon(np.where(inside, 2.25, 1.0).astype(np.float32))
        d.add_susceptibility(susceptibility_cls(frequency=1.1, gamma=0.05),
                             np.where(inside, 1.5, 0.0).astype(np.float32))
        fcen, fwidth = 0.8, 1.0
    else:
        d.set_epsilon(np.where(x ** 2 + y ** 2 + z ** 2 < 0.35 ** 2, 4.0, 1.0).astype(np.float32))
        fcen, fwidth = 0.15, 0.1
    lossy = case.get("conductivity")
    if lossy:
        _set_conductivity(d, case, x, y, z, lengths, reference)
    source_x = -0.15 if lossy else -lengths[0] / 4
    if case.get("mirror_sources"):
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (0.25, 0.13, 0.17),
                      "size": (0, 0, 0), "frequency": fcen, "fwidth": fwidth})
        d.add_source({"source_type": "gaussian", "component": "Ey", "center": (0.0, 0.21, 0.1),
                      "size": (0, 0, 0), "frequency": 0.5, "fwidth": 0.4,
                      "amplitude": (0.5 + 0.3j) if case.get("complex") else 0.5})
        d.add_source({"source_type": "continuous", "component": "Hx", "center": (0.1, 0.2, 0.3),
                      "size": (0.3, 0, 0.2), "frequency": 0.3, "amplitude": 0.5})
        flux.append(d.add_flux_monitor(fcen=fcen, df=fwidth / 2, nfreq=3, center=(0, 0, 0.25),
                                       size=(1.0, 0.9, 0), decimation_factor=1))
        dft.append(d.add_dft_monitor(frequencies=[fcen, 0.4], components=("Ex", "Ez", "Hy", "Hx"),
                                     center=(0.0, 0.0, 0.0), size=(0.6, 0.5, 0.4),
                                     decimation_factor=2))
    else:
        d.add_source({"source_type": "gaussian", "component": "Ez",
                      "center": (source_x, 0.03, 0.0), "size": (0, 0, 0),
                      "frequency": fcen, "fwidth": fwidth,
                      "amplitude": (0.6 - 0.8j) if case.get("complex_amplitude") else 1.0})
    if case.get("bloch_line"):
        d.add_source({"source_type": "gaussian", "component": "Ey", "center": (0.0, -0.1, 0.1),
                      "size": (lengths[0], 0, 0), "frequency": fcen, "fwidth": fwidth,
                      "amplitude": 0.7})
    if case.get("bloch_monitors"):
        flux.append(d.add_flux_monitor(fcen=fcen, df=fwidth / 2, nfreq=3, center=(0, 0, 0.25),
                                       size=(lengths[0], lengths[1], 0), decimation_factor=1))
        dft.append(d.add_dft_monitor(frequencies=[fcen, 1.5 * fcen], components=("Ex", "Ez", "Hy"),
                                     center=(0.0, 0.0, 0.0), size=(lengths[0], lengths[1], 0.4),
                                     decimation_factor=2))
    if case.get("magnetic"):
        d.add_source({"source_type": "gaussian", "component": "Hx", "center": (0.1, -0.05, 0.07),
                      "size": (0, 0, 0), "frequency": fcen, "fwidth": fwidth})
        d.add_source({"source_type": "continuous", "component": "Hz", "center": (-0.05, 0.1, -0.1),
                      "size": (0.3, 0, 0.2), "frequency": 0.3, "amplitude": 0.5})
    if case.get("mixed"):
        block = (np.abs(x - 0.2) < 0.15) & (np.abs(y) < 0.3)
        d.add_susceptibility(susceptibility_cls(frequency=0.9, gamma=0.1),
                             np.where(block, 0.8, 0.0).astype(np.float32))
        d.add_susceptibility(susceptibility_cls(frequency=0.5, gamma=0.2, kind="drude"),
                             np.where(block, 0.3, 0.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ex", "center": (0.1, 0.0, 0.05),
                      "size": (0, 0.4, 0), "frequency": 0.5, "fwidth": 0.4})
        d.add_source({"source_type": "continuous", "component": "Ey", "center": (-0.2, 0.21, -0.1),
                      "size": (0, 0, 0), "frequency": 0.3, "amplitude": 0.5})
        if case.get("complex"):
            d.add_source({"source_type": "gaussian", "component": "Ez", "center": (0.15, -0.1, 0.0),
                          "size": (0, 0, 0.3), "frequency": 0.4, "fwidth": 0.3, "amplitude": 0.6 - 0.8j})
        flux.append(d.add_flux_monitor(fcen=0.3, df=0.2, nfreq=3, center=(0, 0.4, 0),
                                       size=(0.8, 0, 0.7), decimation_factor=0))
        flux.append(d.add_flux_monitor(frequencies=[0.2, 0.35], center=(0.05, -0.05, 0.25),
                                       size=(0.9, 0.8, 0), decimation_factor=2))
        dft.append(d.add_dft_monitor(frequencies=[0.25, 0.4], components=("Ex", "Ey", "Hz", "Hx"),
                                     center=(0.0, 0.1, 0.0), size=(0.6, 0.5, 0.4),
                                     decimation_factor=1))
    flux.append(d.add_flux_monitor(fcen=fcen, df=fwidth / 2, nfreq=4, center=(lengths[0] / 4, 0, 0),
                                   size=(0, lengths[1] - 0.5, lengths[2] - 0.5), decimation_factor=0))
    return d, flux, dft


def _set_conductivity(d, case: dict, x, y, z, lengths, reference: bool) -> None:
    """The lossy cases' conductivity (through the same calls on either driver)."""
    if reference:
        from meep_gpu.absorber import AbsorberLayer
    else:
        from meep_gpu_gb300 import AbsorberLayer
    kind = case["conductivity"]
    if kind == "band":
        d.set_conductivity(np.where(np.abs(x) < 0.25, 0.4, 0.0).astype(np.float32))
        d.set_b_conductivity({"Bx": np.where((x > 0.2) & (y > 0.0), 0.3, 0.0).astype(np.float32),
                              "Bz": np.where((x > 0.2) & (y > 0.0), 0.2, 0.0).astype(np.float32)})
    elif kind == "absorber":
        d.set_conductivity(0.05)
        d.set_absorber([AbsorberLayer(0.3, axis, side) for axis in range(3) for side in ("low", "high")])
    elif kind == "absorber_b":
        d.set_conductivity(0.05)
        d.set_b_conductivity(0.1)
        d.set_absorber([AbsorberLayer(0.3, axis, side) for axis in range(3) for side in ("low", "high")])
    elif kind == "mixed":
        d.set_conductivity({"Dx": np.where(np.abs(z) < 0.3, 0.25, 0.0).astype(np.float32),
                            "Dz": np.where(y > 0.1, 0.15, 0.0).astype(np.float32)})
        d.set_absorber([AbsorberLayer(0.25, 2, "low"), AbsorberLayer(0.35, 2, "high")])
    else:
        raise ValueError(f"unknown conductivity case {kind!r}")


# The two-run flux normalisation: run 1 in vacuum saves its flux-plane transforms, run 2
# (a dielectric sphere between the source and the plane) starts from minus them.
FLUX_NORM = dict(n=(14, 12, 16), pml=3, steps=120)


def build_flux_norm(driver_cls, structure: bool, reference: bool = False):
    """One run of the normalisation pair; returns (driver, flux monitor)."""
    res = 10
    lengths = tuple(v / res for v in FLUX_NORM["n"])
    d = driver_cls(cell_size=lengths, resolution=res, courant=0.5, force_complex_fields=False,
                   boundaries="metallic", **({"prefer_gpu": False} if reference else {}))
    d.setup_pml(FLUX_NORM["pml"])
    x, y, z = d.grid.meshgrid()
    if structure:
        d.set_epsilon(np.where((x - 0.1) ** 2 + y ** 2 + z ** 2 < 0.2 ** 2, 4.0, 1.0).astype(np.float32))
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.2, 0.03, 0.0),
                  "size": (0, 0, 0), "frequency": 0.5, "fwidth": 0.4})
    flux = d.add_flux_monitor(fcen=0.5, df=0.3, nfreq=4, center=(0.35, 0, 0), size=(0, 0.7, 1.1),
                              decimation_factor=0)
    return d, flux
