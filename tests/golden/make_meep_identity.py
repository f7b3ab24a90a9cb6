"""Record MEEP's own words for the MEEP-identity cases as fixtures of this suite.

The reference keeps, for a few 2-D and 3-D runs minted on MEEP itself, the SHA-256 of every
stored float32 word of each of the twelve field components at every compared step
(``parity/meep_gpu/fixtures/meep_identity/keep/<case>/digests.json``), with a capsule
that rebuilds the run (``meep_gpu/capsule.py``). This script reads both through the
reference's own modules (run here, where the reference checkout is), and writes what
a run of this engine needs to face those digests without the reference:

* ``tests/golden/meep_identity.json``: per case the driver's construction (cell,
  resolution, Courant number, boundaries, dimensions) and its construction calls in
  order (``set_epsilon`` / ``set_epsilon_components``, ``setup_pml``, ``add_source``,
  ``add_susceptibility``, ``set_absent_components``; array arguments by name in the
  npz), the compared steps and MEEP's stored digests at each;
* ``tests/golden/meep_identity.npz``: the array arguments (float64 permittivity volumes)
  and, for a folded case, each component's mask of compared cells (every stored cell
  but the mirror ghosts, ``meep_identity.cell_classes``).

The capsule's ``set_chunk_layout`` call installs MEEP's chunk division. It is left out:
the reference itself, built with its default one-rank division and its own Gaussian
currents (not the recorded table), reproduces every stored digest of these cases, which
this script checks before it writes anything (so the fixture pins the engine to MEEP's
words through arithmetic this engine restates).

    python tests/golden/make_meep_identity.py [--reference PATH]
"""

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# c and c_prime: 3-D, odd Y and Z mirror planes, a PML of 7.5 cells, an Hx source;
# ex.absorber-1d: 1-D, a Drude and four Lorentz poles, absorber layers at both z faces.
# Not recorded: the holey-waveguide band case (its digests need MEEP's recorded chunk
# layout and currents even on the reference) and the cylindrical ring.
CASES = ("a", "b", "c", "c_prime", "ex.material-dispersion", "ex.absorber-1d")
KEPT_CALLS = ("set_epsilon", "set_epsilon_components", "setup_pml", "add_source", "add_susceptibility",
              "set_absorber", "set_absent_components")


def _plain(value, arrays, label):
    """JSON form of a decoded capsule argument; arrays go to ``arrays`` under ``label``."""
    if isinstance(value, np.ndarray):
        if value.size and np.all(value == value.flat[0]):
            return {"uniform": float(value.flat[0])}
        arrays[label] = np.asarray(value, dtype=np.float64)
        return {"array": label}
    if isinstance(value, dict):
        return {str(k): _plain(v, arrays, f"{label}.{k}") for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [_plain(v, arrays, f"{label}.{i}") for i, v in enumerate(value)]
    if isinstance(value, complex):
        return {"complex": [value.real, value.imag]}
    if isinstance(value, (np.floating, float)):
        return float(value)
    if isinstance(value, (np.integer, int, bool, str)) or value is None:
        return value
    kind = type(value).__name__
    if kind == "Mirror":
        return {"mirror": [str(value.axis), int(value.phase)]}
    if kind == "AbsorberLayer":
        return {"absorber": {"thickness": float(value.thickness), "axis": int(value.axis),
                             "side": str(value.side), "R_asymptotic": float(value.R_asymptotic)}}
    if kind == "Susceptibility":
        return {"susceptibility": {"frequency": float(value.frequency), "gamma": float(value.gamma),
                                   "kind": str(value.kind)}}
    raise TypeError(f"{label}: no fixture form for {kind}")


def main():
    parser = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    parser.add_argument("--reference", default=os.environ.get("MEEPGB_REFERENCE", str(HERE.parents[2] / "reference")))
    args = parser.parse_args()
    sys.path.insert(0, args.reference)
    from meep_gpu import capsule, meep_identity  # noqa: PLC0415 - the reference checkout
    from meep_gpu.driver import FdtdDriver  # noqa: PLC0415

    root = meep_identity.fixtures_root()
    components = meep_identity.COMPONENTS
    record = {"source": "reference parity/meep_gpu/fixtures/meep_identity/keep (MEEP's own words)",
              "components": list(components), "cases": {}}
    arrays = {}
    for case in CASES:
        directory = root / "keep" / case
        digests = json.loads((directory / "digests.json").read_text())
        stored = capsule.read_capsule(directory / "capsule.capsule")
        decoder = capsule._Decoder(stored)  # noqa: SLF001 - the reference's own reader
        constructor = decoder.decode(stored.document["construction"]["constructor"])
        calls = [(name, decoder.decode(node)) for name, node in stored.document["construction"]["calls"]]
        # the check: the reference on the kept calls alone reproduces MEEP's digests
        driver = FdtdDriver(**dict(constructor, prefer_gpu=False))
        for name, kwargs in calls:
            if name in KEPT_CALLS:
                getattr(driver, name)(**kwargs)
        masks = {c: meep_identity.cell_classes(driver.grid, c)["compared"] for c in components}
        for target in digests["steps"]:
            while driver.step_count < target:
                driver.step()
            for c in components:
                words = meep_identity.compared_words(driver.get_field(c, cell_centered=False), masks[c])
                if meep_identity.digest_words(words) != digests["stored"][str(target)][c]:
                    raise SystemExit(f"{case}: the reference without the recorded layout and currents "
                                     f"differs from MEEP at step {target} {c}; not recorded")
        driver.close()
        label = case.replace(".", "_")
        masked = {}
        for c in components:
            if not bool(masks[c].all()):
                arrays[f"{label}.mask.{c}"] = masks[c]
                masked[c] = f"{label}.mask.{c}"

        record["cases"][case] = {
            "constructor": {k: _plain(v, arrays, f"{label}.constructor.{k}")
                            for k, v in constructor.items() if k not in ("prefer_gpu", "gpu_id")},
            "calls": [[name, _plain(kwargs, arrays, f"{label}.{index}.{name}")]
                      for index, (name, kwargs) in enumerate(calls) if name in KEPT_CALLS],
            "masks": masked,
            "n_steps": digests["n_steps"],
            "steps": digests["steps"],
            "stored": {str(step): digests["stored"][str(step)] for step in digests["steps"]},
        }
        print(f"{case}: {len(digests['steps'])} steps x {len(components)} components checked and recorded")
    (HERE / "meep_identity.json").write_text(json.dumps(record, indent=1, sort_keys=True) + "\n")
    np.savez_compressed(HERE / "meep_identity.npz", **arrays)
    print("wrote", HERE / "meep_identity.json", "and", HERE / "meep_identity.npz")


if __name__ == "__main__":
    main()
