"""Synthetic workloads with the shapes of the benchmarked configurations.

Each builder configures an ``FdtdDriver`` (or any class with the same API) and
returns ``(driver, flux_monitors, dft_monitors)``. Geometry is point-sampled on the
grid's cell centres, as the configurations specify; there is no dataset.

* ``sphere80``: 80^3 cells at resolution 10 (8-unit cube), 10-cell PML, eps-4 sphere of
  radius 2, Ez Gaussian (fcen 0.15, df 0.1) at x = -2, one x-normal flux plane at
  x = 2.5 of size 6 x 6 with 50 frequencies; 2000 steps.
* ``sphere192_8dft``: the same physical case at resolution 24 (192^3 = 7,077,888 cells),
  with eight DFT objects: flux planes one cell inside the PML on all six faces and two
  32^3 field-DFT volumes (Ex, Ey, Ez) centred at (+-1.6, 0, 0), 100 frequencies each;
  5000 steps.
* ``lorentz192``: 192^3 at resolution 20 (9.6-unit cube), slab |x| < 0.5 with
  eps_inf 2.25 and one Lorentz pole (f0 1.1, gamma 0.05, sigma 1.5), 10-cell PML,
  Ez Gaussian (fcen 0.8, df 1.0) at x = -2.4, transmission/reflection planes at x = +-2
  of size 7.6 x 7.6 with 200 frequencies; 10,000 steps.
* ``sphere128``: a 128^3 sphere case with one flux plane.
* ``sphere192``: the 192^3 sphere case with one 50-frequency flux plane (working set
  ~0.4 GB, above the L2 size): the case detailed kernel profiles are taken on.
* ``bloch192``: the 192^3 sphere case (resolution 24) with complex fields on a lattice
  periodic in x and y with Bloch vector k = (0.25, 0.1, 0), the 10-cell PML on z only,
  a z-normal 50-frequency flux plane at z = 2.5 across the whole period; 5000 steps.
* ``bloch48``: the ``bloch192`` case at resolution 6 (48^3, 5-cell PML on z); the case
  the Bloch path's float64 error is quoted on (600 steps).
* ``complex80``: the ``sphere80`` case with complex fields (k = 0) and a complex source
  amplitude (0.6 - 0.8i); the case the complex path's float64 error is quoted on (600
  steps).
* ``sphere192_nopml``: the same without the PML (a bare metallic box): every CTA steps
  the plain update, the case the PML's own cost is measured against.
* ``absorber192``: the ``sphere192`` case with ``mp.Absorber(1.0)`` on all six faces (a
  graded D and B conductivity, 24 cells deep) in place of the PML, and a D conductivity
  0.05 inside the sphere; 5000 steps.
* ``lossy_pml192``: the ``sphere192`` case (10-cell PML) with a D conductivity 0.05 in
  the sphere and a B conductivity 0.02 in the |x| < 3 slab, which runs through the y and
  z layers (every conductive PML form is live); 5000 steps.
* ``lossy40``: 40^3 at resolution 10: PML (6 cells) on x and y, an absorber on each z
  face (0.6 and 0.5), an eps-3 sphere of radius 0.8, a D conductivity 0.35 in |y| < 0.7
  (through the x layers), a B conductivity (0.2 on Bx for x > 0.5, 0.05 on Bz), a
  Lorentz slab, an extended Ez source on a lossy component and a 20-frequency flux
  plane; the case the lossy path's float64 error is quoted on (300 steps).
* ``mirror192``: the ``sphere192_8dft`` case (its eight DFT objects included) folded by
  an even Y and an odd Z mirror (``mp.Mirror``): 192 x 97 x 97 stored cells, the
  discarded halves' flux planes and volume parts read from their mirror images; 5000
  steps.
* ``mirror80``: the ``sphere80`` case folded the same way (80 x 41 x 41); the case the
  folded path's float64 error is quoted on (600 steps).
* ``adjoint96`` (:func:`adjoint96`): 96^3 at resolution 10, 10-cell PML, a 16 x 64 x 64
  design box centred in the cell with eps ~ U[1, 12] (seed 0), Ez Gaussian (fcen 0.15,
  df 0.05) at x = -L/4, a 10-frequency x-normal flux plane 4 cells past the box;
  4000 steps, checkpoints every 200.
"""

from __future__ import annotations

import numpy as np

WORKLOADS = ("sphere80", "sphere192_8dft", "lorentz192", "sphere128", "sphere192", "absorber192",
             "lossy_pml192", "lossy40", "mirror192", "mirror80", "sphere192_nopml", "bloch192",
             "complex80", "bloch48", "tm2d_4096")
STEPS = {"sphere80": 2000, "sphere192_8dft": 5000, "lorentz192": 10000, "sphere128": 1000,
         "sphere192": 5000, "absorber192": 5000, "lossy_pml192": 5000, "lossy40": 300,
         "mirror192": 5000, "mirror80": 600, "sphere192_nopml": 5000, "bloch192": 5000,
         "complex80": 600, "bloch48": 600, "tm2d_4096": 4000}


def _axes(grid):
    """The cell-centre coordinates as broadcastable (n, 1, 1), (1, n, 1), (1, 1, n)
    float32 arrays: the same words as the dense meshgrid, without its three volumes."""
    return grid.x[:, None, None], grid.y[None, :, None], grid.z[None, None, :]


def build(name: str, driver_cls=None, susceptibility_cls=None, **driver_kwargs):
    if driver_cls is None:
        from .driver import FdtdDriver as driver_cls  # noqa: N813
    if susceptibility_cls is None:
        from .dispersion import Susceptibility as susceptibility_cls  # noqa: N813
    if name in ("sphere80", "sphere192_8dft", "sphere128", "sphere192", "mirror192", "mirror80",
                "sphere192_nopml"):
        res = {"sphere80": 10, "sphere192_8dft": 24, "sphere128": 16, "sphere192": 24,
               "mirror192": 24, "mirror80": 10, "sphere192_nopml": 24}[name]
        length = 8.0
        if name.startswith("mirror"):
            from .grid import Mirror
            # the Ez source on both planes is even about them: Ez is even under an even Y
            # mirror and, lying along z, under an odd Z one
            driver_kwargs = dict(driver_kwargs, symmetry=(Mirror("Y", 1), Mirror("Z", -1)))
            name = "sphere192_8dft" if name == "mirror192" else "sphere80"
        open_box = name == "sphere192_nopml"
        if open_box:
            name = "sphere192"
        d = driver_cls(cell_size=(length, length, length), resolution=res, courant=0.5,
                       force_complex_fields=False, boundaries="metallic", **driver_kwargs)
        if not open_box:
            d.setup_pml(10)
        x, y, z = _axes(d.grid)
        d.set_epsilon(np.where(x ** 2 + y ** 2 + z ** 2 < 2.0 ** 2, np.float32(4.0), np.float32(1.0)))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.0, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
        flux, dft = [], []
        if name != "sphere192_8dft":
            flux.append(d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=50, center=(2.5, 0, 0),
                                           size=(0, 6, 6), decimation_factor=0))
            return d, flux, dft
        inset = 4.0 - 11 * d.grid.dx           # one cell inside the 10-cell PML
        span = 2 * inset
        for axis in range(3):
            for sign in (-1.0, 1.0):
                center = [0.0, 0.0, 0.0]
                center[axis] = sign * inset
                size = [span, span, span]
                size[axis] = 0.0
                flux.append(d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=100, center=tuple(center),
                                               size=tuple(size), decimation_factor=0))
        side = 32 * d.grid.dx
        for sign in (-1.0, 1.0):
            dft.append(d.add_dft_monitor(fcen=0.15, df=0.1, nfreq=100, components=("Ex", "Ey", "Ez"),
                                         center=(sign * 1.6, 0.0, 0.0), size=(side, side, side),
                                         decimation_factor=0))
        return d, flux, dft
    if name in ("bloch192", "complex80", "bloch48"):
        bloch = name != "complex80"
        res = {"bloch192": 24, "bloch48": 6, "complex80": 10}[name]
        d = driver_cls(cell_size=(8.0, 8.0, 8.0), resolution=res, courant=0.5, force_complex_fields=True,
                       boundaries=("periodic", "periodic", "metallic") if bloch else "metallic",
                       k_point=(0.25, 0.1, 0.0) if bloch else (0.0, 0.0, 0.0), **driver_kwargs)
        d.setup_pml({"z": 5 if name == "bloch48" else 10} if bloch else 10)
        x, y, z = _axes(d.grid)
        d.set_epsilon(np.where(x ** 2 + y ** 2 + z ** 2 < 2.0 ** 2, np.float32(4.0), np.float32(1.0)))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.0, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1,
                      "amplitude": 1.0 if bloch else 0.6 - 0.8j})
        if bloch:
            flux = [d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=50, center=(0, 0, 2.5), size=(8.0, 8.0, 0),
                                       decimation_factor=0)]
        else:
            flux = [d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=50, center=(2.5, 0, 0), size=(0, 6, 6),
                                       decimation_factor=0)]
        return d, flux, []
    if name in ("absorber192", "lossy_pml192"):
        from .conductivity import AbsorberLayer
        d = driver_cls(cell_size=(8.0, 8.0, 8.0), resolution=24, courant=0.5,
                       force_complex_fields=False, boundaries="metallic", **driver_kwargs)
        x, y, z = d.grid.meshgrid()
        sphere = x ** 2 + y ** 2 + z ** 2 < 2.0 ** 2
        d.set_epsilon(np.where(sphere, 4.0, 1.0).astype(np.float32))
        d.set_conductivity(np.where(sphere, 0.05, 0.0).astype(np.float32))
        if name == "absorber192":
            d.set_absorber([AbsorberLayer(1.0, axis, side) for axis in range(3) for side in ("low", "high")])
        else:
            d.setup_pml(10)
            d.set_b_conductivity(np.where(np.abs(x) < 3.0, 0.02, 0.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.0, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.1})
        flux = [d.add_flux_monitor(fcen=0.15, df=0.1, nfreq=50, center=(2.5, 0, 0), size=(0, 5, 5),
                                   decimation_factor=0)]
        return d, flux, []
    if name == "lossy40":
        from .conductivity import AbsorberLayer
        d = driver_cls(cell_size=(4.0, 4.0, 4.0), resolution=10, courant=0.5,
                       force_complex_fields=False, boundaries="metallic", **driver_kwargs)
        d.setup_pml({"x": 6, "y": 6})
        d.set_absorber([AbsorberLayer(0.6, 2, "low"), AbsorberLayer(0.5, 2, "high")])
        x, y, z = d.grid.meshgrid()
        d.set_epsilon(np.where(x * x + y * y + z * z < 0.8 ** 2, 3.0, 1.0))
        d.set_conductivity(np.where(np.abs(y) < 0.7, 0.35, 0.0))
        d.set_b_conductivity({"Bx": np.where(x > 0.5, 0.2, 0.0), "Bz": 0.05})
        d.add_susceptibility(susceptibility_cls(frequency=1.1, gamma=0.05),
                             np.where(np.abs(x + 0.8) < 0.2, 0.5, 0.0))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.6, 0.1, 0.0),
                      "size": (0, 0.6, 0.4), "frequency": 0.4, "fwidth": 0.3})
        flux = [d.add_flux_monitor(fcen=0.4, df=0.3, nfreq=20, center=(0.9, 0, 0), size=(0, 2.0, 2.0),
                                   decimation_factor=2)]
        return d, flux, []
    if name == "tm2d_4096":
        # a 2-D run (z invariant): 4096 x 4096 cells at resolution 20, a 20-cell PML on x
        # and y, an eps-4 disk of radius 40, an Ez Gaussian point and two flux lines
        d = driver_cls(cell_size=(204.8, 204.8, 0.0), resolution=20, courant=0.5, dimensions=2,
                       force_complex_fields=False, boundaries={"x": "metallic", "y": "metallic"},
                       **driver_kwargs)
        d.setup_pml({"x": 20, "y": 20})
        x, y, _ = _axes(d.grid)
        d.set_epsilon(np.where(x ** 2 + y ** 2 < 40.0 ** 2, np.float32(4.0), np.float32(1.0)))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-60.0, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.5, "fwidth": 0.3})
        flux = [d.add_flux_monitor(fcen=0.5, df=0.3, nfreq=50, center=(sign * 60.0, 0, 0),
                                   size=(0, 150.0, 0), decimation_factor=0) for sign in (1.0, -1.0)]
        return d, flux, []
    if name == "lorentz192":
        res = 20
        length = 9.6
        d = driver_cls(cell_size=(length, length, length), resolution=res, courant=0.5,
                       force_complex_fields=False, boundaries="metallic", **driver_kwargs)
        d.setup_pml(10)
        x, y, z = d.grid.meshgrid()
        slab = np.abs(x) < 0.5
        d.set_epsilon(np.where(slab, 2.25, 1.0).astype(np.float32))
        d.add_susceptibility(susceptibility_cls(frequency=1.1, gamma=0.05),
                             np.where(slab, 1.5, 0.0).astype(np.float32))
        d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.4, 0.0, 0.0),
                      "size": (0, 0, 0), "frequency": 0.8, "fwidth": 1.0})
        flux = [d.add_flux_monitor(fcen=0.8, df=1.0, nfreq=200, center=(sign * 2.0, 0, 0),
                                   size=(0, 7.6, 7.6), decimation_factor=0) for sign in (1.0, -1.0)]
        return d, flux, []
    raise ValueError(f"unknown workload {name!r}; choose from {WORKLOADS}")


ADJOINT96_BOX = ((40, 56), (16, 80), (16, 80))
ADJOINT96_STEPS = 4000


def adjoint96(eps_box=None, driver_cls=None, seed: int = 0, **driver_kwargs):
    """The adjoint workload; returns ``(driver, flux, box, eps_box)``."""
    if driver_cls is None:
        from .driver import FdtdDriver as driver_cls  # noqa: N813
    box = ADJOINT96_BOX
    shape = tuple(b - a for a, b in box)
    if eps_box is None:
        eps_box = np.random.default_rng(seed).uniform(1.0, 12.0, shape)
    d = driver_cls(cell_size=(9.6, 9.6, 9.6), resolution=10, courant=0.5, force_complex_fields=False,
                   boundaries="metallic", **driver_kwargs)
    d.setup_pml(10)
    eps = np.ones(d.grid.shape)
    (i0, i1), (j0, j1), (k0, k1) = box
    eps[i0:i1, j0:j1, k0:k1] = eps_box
    d.set_epsilon(eps)
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-2.4, 0.0, 0.0),
                  "size": (0, 0, 0), "frequency": 0.15, "fwidth": 0.05})
    plane_x = (i1 + 4 - 48) / 10.0
    flux = d.add_flux_monitor(fcen=0.15, df=0.05, nfreq=10, center=(plane_x, 0.0, 0.0), size=(0, 6.4, 6.4),
                              decimation_factor=0)
    return d, flux, box, eps_box


def main(argv=None) -> None:
    """Build one workload on the GPU and step it: ``python -m meep_gpu_gb300.workloads NAME
    [--steps K]`` (three steps to make the plan and choose its kernels, then K timed).
    ``adjoint96``: the adjoint gradient over K steps (checkpoints every min(200, K)),
    forward and backward once to make the plans, then once timed."""
    import argparse
    import time

    import torch

    from .driver import FdtdDriver

    parser = argparse.ArgumentParser(description=main.__doc__)
    parser.add_argument("name", choices=tuple(WORKLOADS) + ("adjoint96",))
    parser.add_argument("--steps", type=int, default=10)
    parser.add_argument("--kernels", default=None,
                        help="fixed kernel choice: 4 numbers (family, block_z, block_y, x_chunk) "
                             "or 8 (the H half's, then the E half's); default: autotuned")
    parser.add_argument("--split", type=int, default=0,
                        help="with --kernels: launch each half over this many x ranges")
    args = parser.parse_args(argv)
    if args.name == "adjoint96":
        from .adjoint import FluxAdjoint

        driver, flux, box, eps_box = adjoint96()
        problem = FluxAdjoint(driver, flux, box, args.steps, checkpoint_every=min(200, args.steps))
        eps = torch.from_numpy(eps_box)
        problem.forward(eps)
        problem.backward()
        torch.cuda.synchronize()
        start = time.perf_counter()
        problem.forward(eps)
        middle = time.perf_counter()
        problem.backward()
        torch.cuda.synchronize()
        stop = time.perf_counter()
        print(f"adjoint96: {driver.grid}, {args.steps} steps, forward {1e3 * (middle - start):.2f} ms, "
              f"backward {1e3 * (stop - middle):.2f} ms")
        problem.close()
        driver.close()
        return
    kernels = None
    if args.kernels:
        values = tuple(int(v) for v in args.kernels.split(","))
        kernels = values if len(values) == 4 else (values[:4], values[4:])
        if args.split > 1:
            pair = kernels if len(values) == 8 else (kernels, kernels)
            kernels = (pair[0], pair[1], None, args.split)
    driver, _, _ = build(args.name, FdtdDriver, kernels=kernels)
    driver.step_many(3)
    torch.cuda.synchronize()
    start = time.perf_counter()
    driver.engine.step(driver.step_count, args.steps)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - start
    engine = driver.engine.re if hasattr(driver.engine, "re") else driver.engine
    print(f"{args.name}: {driver.grid}, kernels {engine.choice}, split {engine.split}, wave {engine.wave}, "
          f"{1e3 * elapsed / max(args.steps, 1):.4f} ms/step over {args.steps} steps")
    driver.close()


if __name__ == "__main__":
    main()
