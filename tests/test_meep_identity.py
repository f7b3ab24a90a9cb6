"""MEEP's own words: the MEEP-identity cases.

For six runs minted on MEEP itself — ``a`` (a 200 x 200 2-D cell, vacuum, PML, a
Gaussian Ez point source), ``b`` (the same with a per-component permittivity up to 12),
``c`` and ``c_prime`` (3-D, 39 x 18 x 19 stored cells under odd Y and Z mirror planes, a
PML of 7.5 cells, a dielectric block, a Gaussian Hx point source) and
``ex.material-dispersion`` (one periodic 2-D cell, eps 2.25 and two Lorentz poles) and
``ex.absorber-1d`` (a 1-D run of 400 cells along z, a Drude and four Lorentz poles,
absorber layers at both faces, an Ex source) — the
reference keeps the SHA-256 of every stored float32 word (mirror ghosts excepted) of all
twelve components at 30 or 31 compared steps (``parity/meep_gpu/fixtures/meep_identity/
keep``, replayed by ``meep_gpu/meep_identity.py:680``). ``tests/golden/
make_meep_identity.py`` copied those digests, each run's construction calls and the
folded runs' masks of compared cells into ``tests/golden/meep_identity.*``.

A 2-D run is one periodic cell on the invariant z (``Grid(dimensions=2)``): every z
difference reads the same word twice, MEEP's own lower-dimensional emulation.

* CPU: the float32 oracle, built from this package's host tables (the 2-D source
  deposition, the PML of x and y), reproduces every digest.
* GPU: the engine reproduces every digest with the autotuned kernels and with each
  generic kernel family, and with the x-range split on the 200-cell x axis.
"""

import os

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from meep_gpu_gb300.grid import IYEE, Grid, Unsupported
from oracle.oracle import Oracle, problem_from_driver
from tests import golden_io

CASES = ("a", "b", "c", "c_prime", "ex.material-dispersion", "ex.absorber-1d")


def _mismatches(case, entry, field_at, advance):
    """(step, component) pairs whose digest differs from MEEP's, stepping through the
    compared steps with ``advance(n)`` and reading with ``field_at(component)``."""
    masks = golden_io.identity_masks(case)
    done = 0
    bad = []
    for step in entry["steps"]:
        if step > done:
            advance(step - done)
            done = step
        for c, mask in masks.items():
            if golden_io.compared_digest(field_at(c), mask) != entry["stored"][str(step)][c]:
                bad.append((step, c))
    return bad


def test_fixture_holds_every_component_at_every_compared_step():
    record, _ = golden_io.meep_identity()
    assert set(record["cases"]) == set(CASES)
    for case in CASES:
        entry = record["cases"][case]
        assert entry["steps"][0] == 0 and entry["steps"][-1] == entry["n_steps"] >= 200
        assert len(entry["steps"]) >= 30
        for step in entry["steps"]:
            assert set(entry["stored"][str(step)]) == set(record["components"])
    # the folded runs leave out exactly the mirror ghosts: plane 0 of a folded axis for
    # the components whose Yee shift along it is 0
    for case in ("c", "c_prime"):
        for c, mask in golden_io.identity_masks(case).items():
            expected = np.ones((39, 18, 19), dtype=bool)
            for axis in (1, 2):  # the odd Y and Z planes
                if IYEE[c][axis] == 0:
                    expected[(slice(None),) * axis + (0,)] = False
            assert np.array_equal(mask if mask is not None else np.ones_like(expected), expected), (case, c)


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_meeps_words(case):
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    driver, entry = golden_io.build_identity(case, FdtdDriver, Susceptibility)
    oracle = Oracle(problem_from_driver(driver), "f32")
    assert _mismatches(case, entry, oracle.field, oracle.run) == []


def test_2d_grid_rules():
    grid = Grid((1.0, 2.0, 0.0), 10, boundaries={"x": "metallic", "y": "metallic"}, dimensions=2)
    assert grid.shape == (10, 20, 1) and grid.is_invariant(2) and grid.axis_wraps(2)
    assert grid.nosize_direction(2) and not grid.nosize_direction(0)
    with pytest.raises(ValueError, match="must be 0"):
        Grid((1.0, 2.0, 0.5), 10, dimensions=2)
    with pytest.raises(ValueError, match="invariant"):
        Grid((1.0, 2.0, 0.0), 10, boundaries="metallic", dimensions=2)
    with pytest.raises(ValueError, match="one-cell direction periodic"):
        Grid((0.1, 2.0, 2.0), 10, boundaries={"x": "metallic"})
    line = Grid((0.0, 0.0, 3.0), 10, boundaries={"z": "metallic"}, dimensions=1)
    assert line.shape == (1, 1, 30) and line.is_invariant(0) and line.is_invariant(1)
    with pytest.raises(ValueError, match="must be 0"):
        Grid((1.0, 1.0, 1.0), 10, dimensions=1)
    with pytest.raises(Unsupported, match="cylindrical"):
        FdtdDriver((1.0, 1.0, 1.0), 10, cylindrical=True)
    # a PML on the invariant axis is refused, a scalar thickness included (the reference's
    # rule); the resolved axes take it
    d = FdtdDriver((2.0, 2.0, 0.0), 10, boundaries={"x": "metallic", "y": "metallic"}, dimensions=2,
                   force_complex_fields=False)
    for request in (4, {"z": 2}):
        with pytest.raises(ValueError, match="invariant"):
            d.setup_pml(request)
    assert d.setup_pml({"x": 4, "y": 4}).faces[2] == (0.0, 0.0)


def test_point_source_in_2d_scales_by_the_carried_axes_only():
    """A zero-extent source is a delta function along x and y (amp * a each) and the
    whole of the invariant z; on one-cell periodic axes it is the whole direction too."""
    d = FdtdDriver((2.0, 2.0, 0.0), 10, boundaries={"x": "metallic", "y": "metallic"}, dimensions=2,
                   force_complex_fields=False)
    src = d.add_source({"component": "Ez", "center": (0, 0, 0), "size": (0, 0, 0),
                        "source_type": "gaussian", "frequency": 1.0, "fwidth": 1.0})
    d.prepare()
    total = sum(a.real for a in src.amps)
    assert np.isclose(total, 10.0 * 10.0) and all(cell[2] == 0 for cell in src.cells)
    one = FdtdDriver((0.1, 0.1, 0.0), 10, dimensions=2, force_complex_fields=False)
    src = one.add_source({"component": "Ez", "center": (0, 0, 0), "size": (0, 0, 0),
                          "source_type": "gaussian", "frequency": 1.0, "fwidth": 1.0})
    one.prepare()
    assert [cell for cell in src.cells] == [(0, 0, 0)] and np.isclose(sum(a.real for a in src.amps), 1.0)


def test_absent_components_are_recorded_and_refused_when_driven():
    d = FdtdDriver((2.0, 2.0, 0.0), 10, dimensions=2, force_complex_fields=False)
    d.add_source({"component": "Ez", "center": (0, 0, 0), "size": (0, 0, 0),
                  "source_type": "gaussian", "frequency": 1.0, "fwidth": 1.0})
    with pytest.raises(ValueError, match="carry a source"):
        d.set_absent_components(["Ez"])
    d.set_absent_components(["Ex", "Ey", "Hz"])
    assert d.absent_components == ("Ex", "Ey", "Hz")
    # a later source on the other polarization brings it back, as MEEP's require_component
    d.add_source({"component": "Ex", "center": (0, 0, 0), "size": (0, 0, 0),
                  "source_type": "gaussian", "frequency": 1.0, "fwidth": 1.0})
    assert d.absent_components == ()


MODES = {"autotuned": None, "generic": (0, 32, 4, 4), "prefetch": (2, 32, 4, 4), "l2": (4, 32, 4, 4),
         "split": ((4, 32, 4, 4), (2, 32, 4, 2), None, 3),
         # y on the warp's lanes (CTAs one cell wide in z) and z rows one cell high in y:
         # the shapes the autotuner adds for 2-D and 1-D grids
         "ylanes": ((0, 1, 128, 4), (4, 1, 64, 2)), "zrows": ((2, 128, 1, 2), (4, 64, 1, 4))}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("case", CASES)
def test_engine_reproduces_meeps_words(gpu, case, mode):
    driver, entry = golden_io.build_identity(case, FdtdDriver, Susceptibility)
    if mode == "split" and driver.grid.shape[0] < 6:
        pytest.skip("the x-range split needs an x axis of several ranges")
    if mode in ("prefetch", "zrows") and driver.has_conductivity:
        pytest.skip("a run with a conductivity steps with the generic families 0 and 4 only")
    driver.kernels = MODES[mode]
    bad = _mismatches(case, entry, lambda c: driver.get_field(c, cell_centered=False), driver.step_many)
    if mode == "split":
        assert driver.engine.split == 3
    assert bad == [], f"{case} ({mode}): digests differ from MEEP's at {bad[:6]}"
    assert driver.engine.device_status_word() == 0
    driver.close()


@pytest.mark.gpu
def test_absent_e_components_stay_plus_zero_on_a_folded_2d_run(gpu):
    """MEEP never steps an absent E component, so it reads +0. On a folded run the odd-
    parity ghost of D (here Dy under an odd X plane) is -0 where its image is +0, and
    E = inv * D would carry that -0: the driver resets the absent E words after every
    step. The present components are the same words as without the absent set."""
    from meep_gpu_gb300 import Mirror

    def run(absent):
        d = FdtdDriver((2.0, 2.0, 0.0), 10, dimensions=2, force_complex_fields=False,
                       boundaries={"x": "metallic", "y": "metallic"}, symmetry=(Mirror("X", -1),))
        d.setup_pml({"y": (3, 3)})
        d.add_source({"component": "Ez", "center": (0.5, 0, 0), "size": (0, 0, 0),
                      "source_type": "gaussian", "frequency": 1.0, "fwidth": 1.0})
        if absent:
            d.set_absent_components(["Ex", "Ey", "Dx", "Dy", "Hz", "Bz"])
        d.run(num_steps=40)
        return d

    plain, marked = run(False), run(True)
    for c in ("Ex", "Ey"):
        words = marked.get_field(c, cell_centered=False)
        assert not np.any(words) and not np.any(np.signbit(words)), c
    assert np.any(np.signbit(plain.get_field("Ey", cell_centered=False))), "the -0 this test guards against"
    for c in ("Ez", "Dz", "Hx", "Hy", "Bx", "By"):
        assert np.array_equal(plain.get_field(c, cell_centered=False), marked.get_field(c, cell_centered=False)), c
    plain.close()
    marked.close()
