"""Seeded configurations the golden-vector script records and the tests rebuild."""

import numpy as np

# src_vol binding: seeded multi-source configurations on Bloch-phased and plain periodic
# cells with PML chunks, seam-crossing sources and a merged duplicate.
SRC_VOL_CONFIGS = 24


def src_vol_config(t: int):
    rng = np.random.default_rng(1000 + t)
    dims = [(1.2, 1.3, 1.5), (1.5, 1.2, 1.3)][t % 2]
    k = [(0.3, -0.2, 0.45), (0.0, 0.0, 0.0), (0.45, 0.0, 0.0)][t % 3]
    pml = [3, {"z": 3}, {"x": 2, "y": {"low": 3, "high": 2}}, None][t % 4]
    specs = []
    for m in range(3):
        comp = ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"][(t + m) % 6]
        center = tuple(float(v) for v in np.round(rng.uniform(-0.3, 0.3, 3), 3))
        size = [0.0, 0.0, 0.0]
        if (t + m) % 3 == 1:
            size[0] = dims[0]
        if (t + m) % 3 == 2:
            size = [dims[0], 0.0, dims[2]]
        specs.append({"source_type": "gaussian", "component": comp, "center": center, "size": tuple(size),
                      "frequency": 0.4, "fwidth": 0.3, "amplitude": 0.7 - 0.2j})
    specs.append(dict(specs[0]))  # merges into the first source's entries
    return dims, k, pml, specs
