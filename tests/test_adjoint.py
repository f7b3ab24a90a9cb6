"""Adjoint gradient of a flux objective: GPU reverse-time kernels against central finite
differences of the float64 oracle.

Two small cases: metallic walls with a 6-cell PML on every face, and PML on x only with
periodic y and z (the adjoint's periodic gathers). The objective is the sum over 5
frequencies of the flux through a plane past a design box whose permittivity is seeded
U[1, 4]. Finite differences: central, h = 1e-3 on eps, each J from the float64 oracle
with the exact inverse 1/eps; the adjoint runs in float32 on the GPU, so the bar is a
relative L2 error of 2e-3 over the sampled voxels (and 1e-4 between the objectives).
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility, Unsupported
from meep_gpu_gb300.adjoint import FluxAdjoint

STEPS = 360
CASES = {
    "metallic_pml": dict(boundaries="metallic", pml=6, box=((12, 18), (12, 20), (13, 19))),
    "periodic_yz": dict(boundaries="periodic", pml={"x": 6}, box=((11, 17), (3, 9), (20, 26))),
}


def build(case, eps_box, **kwargs):
    d = FdtdDriver((3.2, 2.8, 3.0), 10, force_complex_fields=False, boundaries=case["boundaries"], **kwargs)
    d.setup_pml(case["pml"])
    eps = np.ones(d.grid.shape)
    (i0, i1), (j0, j1), (k0, k1) = case["box"]
    eps[i0:i1, j0:j1, k0:k1] = eps_box
    d.set_epsilon(eps)
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.85, 0.05, 0.02),
                  "size": (0, 0, 0), "frequency": 0.55, "fwidth": 0.4})
    d.add_source({"source_type": "gaussian", "component": "Ey", "center": (-0.8, -0.1, 0.1),
                  "size": (0, 0.3, 0), "frequency": 0.5, "fwidth": 0.5, "amplitude": 0.6})
    flux = d.add_flux_monitor(fcen=0.5, df=0.3, nfreq=5, center=(0.85, 0, 0), size=(0, 1.6, 1.4),
                              decimation_factor=2)
    return d, flux, eps


def eps_box_for(case, seed=0):
    (i0, i1), (j0, j1), (k0, k1) = case["box"]
    return np.random.default_rng(seed).uniform(1.0, 4.0, (i1 - i0, j1 - j0, k1 - k0))


def oracle_objective(case, eps_box):
    from oracle.oracle import Oracle, problem_from_driver

    d, _, eps = build(case, eps_box)
    problem = problem_from_driver(d)
    problem.inv_eps64 = [1.0 / eps] * 3  # the exact inverse, not the float32 word
    oracle = Oracle(problem, "f64")
    oracle.run(STEPS)
    return float(np.sum(oracle.flux_spectrum(0)))


def test_adjoint_refuses_poles_and_stepped_drivers():
    case = CASES["metallic_pml"]
    d, flux, _ = build(case, eps_box_for(case))
    d.add_susceptibility(Susceptibility(frequency=1.0, gamma=0.1), 0.1)
    with pytest.raises(Unsupported):
        FluxAdjoint(d, flux, case["box"], STEPS)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_adjoint_gradient_matches_float64_finite_differences(gpu, name):
    import torch

    case = CASES[name]
    eps_box = eps_box_for(case)
    d, flux, _ = build(case, eps_box, kernels=(0, 32, 4, 4))
    problem = FluxAdjoint(d, flux, case["box"], STEPS, checkpoint_every=100)
    value = problem.forward(torch.from_numpy(eps_box))
    grad = problem.backward().cpu().numpy()
    j64 = oracle_objective(case, eps_box)
    assert abs(value - j64) <= 1e-4 * abs(j64), (value, j64)
    rng = np.random.default_rng(1)
    picks = [tuple(int(rng.integers(0, n)) for n in eps_box.shape) for _ in range(6)]
    h = 1e-3
    fd, ad = [], []
    for v in picks:
        plus, minus = eps_box.copy(), eps_box.copy()
        plus[v] += h
        minus[v] -= h
        fd.append((oracle_objective(case, plus) - oracle_objective(case, minus)) / (2 * h))
        ad.append(grad[v])
    fd, ad = np.array(fd), np.array(ad)
    assert np.linalg.norm(ad - fd) <= 2e-3 * np.linalg.norm(fd), (ad, fd)
    problem.close()
    d.close()


@pytest.mark.gpu
def test_autograd_and_checkpoint_interval(gpu):
    import torch

    case = CASES["metallic_pml"]
    eps_box = eps_box_for(case, seed=3)
    grads = []
    for every in (STEPS, 40):
        d, flux, _ = build(case, eps_box)
        problem = FluxAdjoint(d, flux, case["box"], STEPS, checkpoint_every=every)
        eps = torch.tensor(eps_box, dtype=torch.float64, requires_grad=True)
        value = problem.objective(eps)
        value.backward()
        assert eps.grad is not None and eps.grad.shape == eps.shape
        grads.append(eps.grad.numpy().copy())
        problem.close()
        d.close()
    assert np.max(np.abs(grads[0] - grads[1])) <= 1e-5 * np.max(np.abs(grads[0]))


@pytest.mark.gpu
def test_adjoint96_against_float64_fixture(gpu):
    """The 96^3 workload (4000 steps, checkpoints every 200): the GPU gradient against
    float64 central differences (h = 1e-3) at 32 seeded voxels and along one seeded
    direction over the whole 16 x 64 x 64 box (tests/golden/adjoint96_fd.json, made by
    tests/golden/make_adjoint_fd.py)."""
    import json
    from pathlib import Path

    import torch

    from meep_gpu_gb300 import workloads

    record = json.loads((Path(__file__).parent / "golden" / "adjoint96_fd.json").read_text())
    driver, flux, box, eps_box = workloads.adjoint96()
    problem = FluxAdjoint(driver, flux, box, workloads.ADJOINT96_STEPS, checkpoint_every=200)
    value = problem.forward(torch.from_numpy(eps_box))
    grad = problem.backward().cpu().numpy()
    assert abs(value - record["objective"]) <= 1e-5 * abs(record["objective"])
    rng = np.random.default_rng(0)
    picks = [tuple(int(rng.integers(0, n)) for n in eps_box.shape) for _ in record["voxels"]]
    assert picks == [tuple(v["voxel"]) for v in record["voxels"]]
    direction = rng.standard_normal(eps_box.shape)
    direction /= np.linalg.norm(direction)
    fd = np.array([v["fd"] for v in record["voxels"]])
    ad = np.array([grad[v] for v in picks])
    assert np.linalg.norm(ad - fd) <= 2e-3 * np.linalg.norm(fd), (ad, fd)
    along = float(np.sum(grad * direction))
    assert abs(along - record["directional_fd"]) <= 1e-4 * abs(record["directional_fd"])
    problem.close()
    driver.close()
