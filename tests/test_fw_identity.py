"""The identities that let the CUDA step skip the f_w words, checked on the oracle.

The oracle restates the reference's step with every word it stores, f_w of H and of E
included. After any completed step, on each component's own-axis PML membership:

* f_w of H equals B (MEEP's update_H stores B's new word in both), so the H half reads
  B's old word for it;
* f_w of E equals chi1inv (D - sum of P) of the stored D and of the polarization the E
  half subtracted (the oracle's P_prev after the rotation), formed with the same
  operations in the same order, so the E half recomputes it instead of reading it.

Both must hold word for word, on runs with poles, conductivity and mirror folds.
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from oracle.oracle import Oracle, problem_from_driver
from tests.golden.cases import CASES, build_case

PML_CASES = sorted(n for n, c in CASES.items() if c.get("pml") and not c.get("complex") and not c.get("dims"))


def _membership(problem, lattice: int, q: int, shape) -> np.ndarray:
    """The cells of component q on its own-axis membership of `lattice` (0 integer, 1 half)."""
    runs = np.asarray(problem.member[(lattice, q)], dtype=bool)
    view = [1, 1, 1]
    view[q] = shape[q]
    return np.broadcast_to(runs.reshape(view), shape)


def _recomputed_w(oracle, problem, q: int) -> np.ndarray:
    """chi1inv (D - sum of P_prev) in float32, in the oracle's operation order."""
    w = oracle.fields["D" + "xyz"[q]].copy()
    for pole in oracle.polarization:
        if q in pole:
            w = (w - pole[q][1]).astype(np.float32)  # P_prev: what the last E half subtracted
    return (np.asarray(problem.inv_eps32[q], dtype=np.float32) * w).astype(np.float32)


@pytest.mark.parametrize("name", PML_CASES)
def test_fw_words_are_b_and_the_recomputed_w(name):
    case = CASES[name]
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    oracle = Oracle(problem, "f32")
    oracle.run(min(case["steps"], 40))
    shape = tuple(problem.shape)
    checked = 0
    for q, axis in enumerate("xyz"):
        own_h = _membership(problem, 0, q, shape)
        fw_h, b = oracle.fields["fwH" + axis], oracle.fields["B" + axis]
        assert np.array_equal(fw_h[own_h], b[own_h]), f"{name} fwH{axis}"
        own_e = _membership(problem, 1, q, shape)
        w = _recomputed_w(oracle, problem, q)
        fw_e = oracle.fields["fwE" + axis]
        assert np.array_equal(fw_e[own_e], w[own_e]), f"{name} fwE{axis}"
        checked += int(own_h.sum()) + int(own_e.sum())
    assert checked > 0


def test_a_planted_difference_is_caught():
    """The comparison above sees a one-word change of f_w of E."""
    case = CASES[PML_CASES[0]]
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    problem = problem_from_driver(driver)
    oracle = Oracle(problem, "f32")
    oracle.run(10)
    shape = tuple(problem.shape)
    own_e = _membership(problem, 1, 0, shape)
    where = tuple(int(v[0]) for v in np.nonzero(own_e))
    w = _recomputed_w(oracle, problem, 0)
    assert np.array_equal(oracle.fields["fwEx"][own_e], w[own_e])
    oracle.fields["fwEx"][where] = np.nextafter(oracle.fields["fwEx"][where], np.float32(np.inf))
    assert not np.array_equal(oracle.fields["fwEx"][own_e], w[own_e])
