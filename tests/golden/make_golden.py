"""Record golden vectors from the reference implementation (run in the build container).

Imports the reference's NumPy array path (``meep_gpu.FdtdDriver`` with
``prefer_gpu=False``) from ``$MEEPGB_REFERENCE`` (default: a ``reference`` checkout in
the directory that holds this repository) and writes small fixtures into this directory:

* ``fields_<case>.npz``: every stored float32 field word (E, D, B, H and, for a
  dispersive case, P) after N steps of a small seeded case, plus its flux spectra and
  DFT accumulators;
* ``digest_sphere80.json``: SHA-256 of every field component after 200 steps of the
  80^3 sphere-under-PML workload (the full-size configuration), plus its flux spectrum;
  ``digest_sphere80_2000.json``: the same after the workload's full 2000 steps
  (``python make_golden.py digest2000``);
* ``tables.npz``: PML coefficient vectors, source deposition tables, flux-plane
  regions and weights and automatic decimation factors for a sweep of requests;
* ``conductivity_tables.npz``: ``mp.Absorber`` sigma volumes, conductivity
  coefficients (condfac / condinv) and, under a one-rank PML, the cells whose chunk
  keeps a conductivity, for seeded configurations (``python make_golden.py conductivity``);
* ``flux_normalization.npz``: the two-run normalisation idiom (``python make_golden.py
  flux_norm``): the vacuum run's saved flux-plane transforms and spectrum, and the
  structure run's spectrum started from minus them and alone;
* ``src_vol_tables.npz``: each source's deposit entries in MEEP's ``src_vol`` lists
  (``python make_golden.py src_vols``) for seeded multi-source cells, with the Bloch
  factors ``eikna`` of each.

The fixtures are committed; this script is how they were made. It is not run by the
tests (the reference is not available where the GPU tests run).
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = os.environ.get("MEEPGB_REFERENCE", str(HERE.parent.parent.parent / "reference"))
if not (Path(REFERENCE) / "meep_gpu").is_dir():
    raise SystemExit(f"no reference checkout at {REFERENCE}: set MEEPGB_REFERENCE to the directory "
                     "that holds the meep_gpu package")
sys.path.insert(0, REFERENCE)

from meep_gpu import FdtdDriver  # noqa: E402
from meep_gpu.dispersion import Susceptibility  # noqa: E402

sys.path.insert(0, str(HERE.parent.parent))
from tests.golden.cases import CASES, SPHERE80, SPHERE80_FULL, build_case  # noqa: E402

COMPONENTS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


def reference_driver(case):
    return build_case(FdtdDriver, Susceptibility, case, reference=True)


def record_fields(name: str, case: dict) -> None:
    driver, flux, dft = reference_driver(case)
    driver.run(num_steps=case["steps"])
    out = {}
    for c in COMPONENTS:
        words = np.asarray(driver.get_field(c, cell_centered=False))
        out[c] = words.astype(np.complex64 if np.iscomplexobj(words) else np.float32)
    for index, monitor in enumerate(flux):
        out[f"flux{index}"] = np.asarray(monitor.get_flux_spectrum(), dtype=np.float64)
    for index, monitor in enumerate(dft):
        for c in monitor.components:
            out[f"dft{index}_{c}"] = np.asarray(monitor._dft[c], dtype=np.complex64)
    for m, state in enumerate(driver.fields.polarizations):
        for c, array in state.P.items():
            out[f"P{m}_{c}"] = np.asarray(array, dtype=np.complex64 if np.iscomplexobj(array) else np.float32)
    np.savez_compressed(HERE / f"fields_{name}.npz", **out)
    print(name, "written")


def record_digest(case=SPHERE80, filename="digest_sphere80.json") -> None:
    driver, flux, _ = reference_driver(case)
    driver.run(num_steps=case["steps"])
    digests = {}
    for c in COMPONENTS:
        words = np.ascontiguousarray(driver.get_field(c, cell_centered=False), dtype=np.float32)
        digests[c] = hashlib.sha256(words.tobytes()).hexdigest()
    payload = {"case": "sphere80", "steps": case["steps"], "sha256": digests,
               "flux": [float(v) for v in flux[0].get_flux_spectrum()],
               "decimation": int(flux[0].decimation_factor)}
    (HERE / filename).write_text(json.dumps(payload, indent=1) + "\n")
    print("digest written")


def record_tables() -> None:
    from meep_gpu.grid import Grid
    from meep_gpu.pml import PML
    from meep_gpu.sources import _build_source_points
    from meep_gpu.dft import FluxMonitor

    out = {}
    grid = Grid(cell_size=(2.4, 2.0, 2.8), resolution=10, boundaries="metallic")
    for thickness in (3, 4, 2.5, 5.2):
        pml = PML(grid, thickness)
        for axis in "xyz":
            for half in ("", "_h"):
                for name in ("kms", "sinv", "kps"):
                    key = f"pml_{thickness}_{name}_{axis}{half}"
                    out[key] = np.asarray(getattr(pml, f"{name}_{axis}{half}")).ravel()
    rng = np.random.default_rng(7)
    requests = []
    for t in range(24):
        component = ["Ex", "Ey", "Ez"][t % 3]
        center = tuple(float(v) for v in np.round(rng.uniform(-0.9, 0.9, 3), 3))
        size = [0.0, 0.0, 0.0]
        if t % 4 == 1:
            size[1] = float(np.round(rng.uniform(0.05, 0.9), 3))
        if t % 4 == 2:
            size[0] = float(np.round(rng.uniform(0.05, 0.9), 3))
            size[2] = float(np.round(rng.uniform(0.05, 0.9), 3))
        if t % 6 == 5:
            center = (round(-0.6 + 0.1 * (t % 3), 10), 0.0, 0.05 * t)
        cells, amps = _build_source_points(grid, component, center, tuple(size), 1.0, None)
        out[f"src{t}_cells"] = np.asarray(cells, dtype=np.int64).reshape(-1, 3)
        out[f"src{t}_amps"] = np.asarray(amps, dtype=np.complex128)
        requests.append({"component": component, "center": center, "size": size})
    planes = []
    for t in range(12):
        direction = t % 3
        center = [float(v) for v in np.round(rng.uniform(-0.7, 0.7, 3), 3)]
        size = [float(np.round(rng.uniform(0.2, 1.4), 3)) for _ in range(3)]
        size[direction] = 0.0
        if t % 4 == 0:
            center[direction] = round(0.1 * (t - 5), 10)
        monitor = FluxMonitor(grid, frequencies=(0.1, 0.2), center=tuple(center), size=tuple(size),
                              periodic=(False, False, False))
        out[f"plane{t}_region"] = np.asarray(monitor._region, dtype=np.int64)
        out[f"plane{t}_weights"] = np.asarray(monitor._weights, dtype=np.float32)
        out[f"plane{t}_measure"] = np.float64(monitor._measure)
        planes.append({"center": center, "size": size, "direction": direction})
    np.savez_compressed(HERE / "tables.npz", **out)
    (HERE / "tables.json").write_text(json.dumps({"grid": {"cell_size": [2.4, 2.0, 2.8], "resolution": 10,
                                                            "boundaries": "metallic"},
                                                   "pml_thicknesses": [3, 4, 2.5, 5.2],
                                                   "sources": requests, "planes": planes}, indent=1) + "\n")
    print("tables written")


# Conductivity host tables: absorber ramps, condfac / condinv, and the chunks that keep a
# conductivity under a one-rank PML, each for a few seeded configurations.
ABSORBER_GRIDS = [
    {"cell": [1.4, 1.2, 1.6], "resolution": 10, "boundaries": "metallic",
     "layers": [[0.3, axis, side] for axis in range(3) for side in ("low", "high")]},
    {"cell": [1.3, 1.1, 1.5], "resolution": 13, "boundaries": "periodic",
     "layers": [[0.35, 0, "low"], [0.25, 2, "high"]]},
    {"cell": [2.0, 1.0, 1.0], "resolution": 10, "boundaries": "metallic", "layers": [[0.5, 0, "high"]]},
]
CHUNK_GRIDS = [
    {"cell": [1.4, 1.2, 1.6], "boundaries": "metallic", "pml": 3},
    {"cell": [1.4, 1.3, 1.2], "boundaries": "periodic", "pml": {"x": 3, "y": {"low": 2, "high": 4}, "z": 2.5}},
    {"cell": [1.3, 1.5, 1.2], "boundaries": "metallic", "pml": {"x": 3, "z": 2}},
]
YEE_DB = {"Dx": (1, 0, 0), "Dy": (0, 1, 0), "Dz": (0, 0, 1), "Bx": (0, 1, 1), "By": (1, 0, 1), "Bz": (1, 1, 0)}


def record_conductivity_tables() -> None:
    from meep_gpu.absorber import AbsorberLayer, absorber_conductivity
    from meep_gpu.chunk_map import ChunkLayout
    from meep_gpu.grid import Grid
    from meep_gpu.pml import PML

    out = {}
    for g, spec in enumerate(ABSORBER_GRIDS):
        grid = Grid(cell_size=tuple(spec["cell"]), resolution=spec["resolution"], boundaries=spec["boundaries"])
        volumes = absorber_conductivity(grid, [AbsorberLayer(t, a, side) for t, a, side in spec["layers"]])
        for name, volume in volumes.items():
            out[f"absorber{g}_{name}"] = np.asarray(volume, dtype=np.float64)
    # condfac / condinv of sigma words that round differently in float32 and double
    driver = FdtdDriver(cell_size=(1.0, 1.0, 1.0), resolution=10, force_complex_fields=False,
                        boundaries="metallic", prefer_gpu=False)
    rng = np.random.default_rng(11)
    sigma = rng.choice(np.array([0.5, 0.3, 0.25, 0.1, 1.7, 3.0, 0.0], dtype=np.float32), driver.grid.shape)
    sigma[0, 0, 0] = 0.5
    driver.set_conductivity(sigma)
    out["coef_sigma"] = sigma
    out["coef_condfac"] = np.asarray(driver.fields.condfac_for("Dx"))
    out["coef_condinv"] = np.asarray(driver.fields.condinv_for("Dx"))
    for g, spec in enumerate(CHUNK_GRIDS):
        grid = Grid(cell_size=tuple(spec["cell"]), resolution=10, boundaries=spec["boundaries"])
        layout = ChunkLayout.one_rank(grid, PML(grid, spec["pml"]))
        for t in range(12):
            sig = np.zeros(grid.shape, np.float32)
            lo = [int(rng.integers(0, n)) for n in grid.shape]
            hi = [min(n, a + int(rng.integers(1, 4))) for a, n in zip(lo, grid.shape)]
            sig[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = 0.3
            out[f"chunks{g}_{t}_sigma"] = sig
            for name, iyee in YEE_DB.items():
                out[f"chunks{g}_{t}_{name}"] = np.packbits(layout.conductive_mask(sig, iyee).ravel())
    np.savez_compressed(HERE / "conductivity_tables.npz", **out)
    (HERE / "conductivity_tables.json").write_text(json.dumps(
        {"absorber_grids": ABSORBER_GRIDS, "chunk_grids": CHUNK_GRIDS, "chunk_trials": 12,
         "coef_dt": driver.grid.dt}, indent=1) + "\n")
    print("conductivity tables written")


def record_flux_normalization() -> None:
    from tests.golden.cases import FLUX_NORM, build_flux_norm

    steps = FLUX_NORM["steps"]
    d1, f1 = build_flux_norm(FdtdDriver, structure=False, reference=True)
    d1.run(num_steps=steps)
    data = f1.get_dft_data()
    out = {"flux1": np.asarray(f1.get_flux_spectrum(), dtype=np.float64),
           "frequencies": np.asarray(data.planes[0].frequencies, dtype=np.float64)}
    for side in (data.planes[0].E, data.planes[0].H):
        for name, block in side.items():
            out[f"data_{name}"] = np.asarray(block, dtype=np.complex64)
    d2, f2 = build_flux_norm(FdtdDriver, structure=True, reference=True)
    f2.load_minus_dft_data(data)
    d2.run(num_steps=steps)
    out["flux2_minus"] = np.asarray(f2.get_flux_spectrum(), dtype=np.float64)
    d3, f3 = build_flux_norm(FdtdDriver, structure=True, reference=True)
    d3.run(num_steps=steps)
    out["flux2_plain"] = np.asarray(f3.get_flux_spectrum(), dtype=np.float64)
    np.savez_compressed(HERE / "flux_normalization.npz", **out)
    print("flux normalization written")


from tests.golden.make_golden_configs import SRC_VOL_CONFIGS, src_vol_config  # noqa: E402


def record_src_vols() -> None:
    from meep_gpu.chunk_map import ChunkLayout
    from meep_gpu.sources import bind_src_vols

    out = {}
    for t in range(SRC_VOL_CONFIGS):
        dims, k, pml, specs = src_vol_config(t)
        d = FdtdDriver(cell_size=dims, resolution=10, k_point=k, boundaries="periodic", prefer_gpu=False,
                       force_complex_fields=True)
        if pml is not None:
            d.setup_pml(pml)
        for spec in specs:
            d.add_source(spec)
        bind_src_vols(d._sources, ChunkLayout.one_rank(d.grid, d.pml), d.grid)
        for m, source in enumerate(d._sources):
            cells, amps = [], []
            for table in source._src_vol:
                ix, iy, iz = (np.asarray(a).reshape(-1) for a in (table.ix, table.iy, table.iz))
                cells += [(int(a), int(b), int(c)) for a, b, c in zip(ix, iy, iz)]
                amps += list(np.asarray(table.amps).reshape(-1))
            out[f"c{t}_s{m}_cells"] = np.asarray(cells, dtype=np.int64).reshape(-1, 3)
            out[f"c{t}_s{m}_amps"] = np.asarray(amps, dtype=np.complex128)
        out[f"c{t}_eikna"] = np.asarray([complex(p) if p is not None else 0j for p in d.grid.bloch_phases])
    np.savez_compressed(HERE / "src_vol_tables.npz", **out)
    print("src_vol tables written")


if __name__ == "__main__":
    which = sys.argv[1:] or ["fields", "digest", "tables"]
    if "fields" in which or any(w in CASES for w in which):
        names = [w for w in which if w in CASES] or list(CASES)
        for name in names:
            record_fields(name, CASES[name])
    if "tables" in which:
        record_tables()
    if "digest" in which:
        record_digest()
    if "digest2000" in which:
        record_digest(SPHERE80_FULL, "digest_sphere80_2000.json")
    if "conductivity" in which:
        record_conductivity_tables()
    if "flux_norm" in which:
        record_flux_normalization()
    if "src_vols" in which:
        record_src_vols()
