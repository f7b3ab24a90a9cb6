"""Float64 central differences of the 96^3 adjoint workload's flux objective.

Runs the float64 oracle (``oracle/``) on the ``adjoint96`` workload (96^3, 10-cell PML,
16 x 64 x 64 design box, eps ~ U[1, 12] seed 0, 4000 steps): the objective at the seeded
permittivity, central differences (h = 1e-3) at 32 seeded voxels, and one central
difference along a seeded unit direction over the whole box. The inverse permittivity
is the exact float64 1/eps. Writes ``adjoint96_fd.json`` beside this file, which the
GPU test of the adjoint gradient compares against. Takes about an hour on 8 cores.

    python tests/golden/make_adjoint_fd.py [--voxels 32]
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from meep_gpu_gb300 import workloads  # noqa: E402
from oracle.oracle import Oracle, problem_from_driver  # noqa: E402

H = 1e-3


def objective(values: np.ndarray) -> float:
    d, _, box, _ = workloads.adjoint96(eps_box=values)
    problem = problem_from_driver(d)
    full = np.ones(d.grid.shape)
    (i0, i1), (j0, j1), (k0, k1) = box
    full[i0:i1, j0:j1, k0:k1] = values
    problem.inv_eps64 = [1.0 / full] * 3
    oracle = Oracle(problem, "f64")
    oracle.run(workloads.ADJOINT96_STEPS)
    return float(np.sum(oracle.flux_spectrum(0)))


def picks(eps_box: np.ndarray, count: int):
    rng = np.random.default_rng(0)
    voxels = [tuple(int(rng.integers(0, n)) for n in eps_box.shape) for _ in range(count)]
    direction = rng.standard_normal(eps_box.shape)
    return voxels, direction / np.linalg.norm(direction)


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--voxels", type=int, default=32)
    args = parser.parse_args()
    _, _, box, eps_box = workloads.adjoint96()
    voxels, direction = picks(eps_box, args.voxels)
    started = time.time()
    out = {"h": H, "steps": workloads.ADJOINT96_STEPS, "box": [list(b) for b in box], "seed": 0,
           "objective": objective(eps_box), "voxels": []}
    for v in voxels:
        plus, minus = eps_box.copy(), eps_box.copy()
        plus[v] += H
        minus[v] -= H
        out["voxels"].append({"voxel": list(v), "fd": (objective(plus) - objective(minus)) / (2 * H)})
        print(f"{len(out['voxels'])}/{len(voxels)} {time.time() - started:.0f}s", flush=True)
    out["directional_fd"] = (objective(eps_box + H * direction) - objective(eps_box - H * direction)) / (2 * H)
    (HERE / "adjoint96_fd.json").write_text(json.dumps(out, indent=1))
    print(f"done in {time.time() - started:.0f}s", flush=True)


if __name__ == "__main__":
    main()
