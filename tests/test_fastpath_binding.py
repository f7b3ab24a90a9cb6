"""The reference-side binding (``meep_gpu_gb300.fastpath_binding``).

CPU, with the reference importable (its checkout beside this repository, or
``$MEEPGB_REFERENCE``; skipped where it is absent, as on the GPU machine): for every golden
case, the descriptor tables read from the reference's OWN frozen objects (``Fields``,
``PML``, ``Grid``, bound sources, ``ChunkLayout``) equal the tables this engine's host
code forms for the driver the binding maps that configuration onto, and for the same
case built directly on ``meep_gpu_gb300.FdtdDriver``.

GPU: the plan's dispatch protocol, driven in the reference driver's consult order over
reference-shaped ``Fields`` arrays that the driver's own passes scribble on between the
consults, leaves those arrays equal to the reference's recorded words.
"""

import os
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility
from meep_gpu_gb300.fastpath_binding import (DRIVER_SLOTS, GB300Plan, build_desc, driver_for, host_tables,
                                             plan_fast_path)
from tests import golden_io
from tests.golden.cases import CASES, build_case

ROOT = Path(__file__).resolve().parent.parent
REFERENCE = Path(os.environ.get("MEEPGB_REFERENCE", str(ROOT.parent / "reference")))
HAVE_REFERENCE = (REFERENCE / "meep_gpu" / "driver.py").is_file()
needs_reference = pytest.mark.skipif(not HAVE_REFERENCE, reason="the reference checkout is not on this machine "
                                                                "(set MEEPGB_REFERENCE to it)")
FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz")


def reference_classes():
    if str(REFERENCE) not in sys.path:
        sys.path.insert(0, str(REFERENCE))
    from meep_gpu import FdtdDriver as ReferenceDriver
    from meep_gpu.dispersion import Susceptibility as ReferenceSusceptibility
    return ReferenceDriver, ReferenceSusceptibility


def frozen_reference(case):
    driver_cls, susceptibility_cls = reference_classes()
    ref, _, _ = build_case(driver_cls, susceptibility_cls, case, reference=True)
    ref.step()  # the configuration freeze: src_vol tables bound, chunk layout resolved
    return ref


@needs_reference
@pytest.mark.parametrize("name", sorted(CASES))
def test_descriptor_from_the_references_objects_equals_the_engines_tables(name):
    case = CASES[name]
    ref = frozen_reference(case)
    tables = build_desc(ref.fields, ref.pml, ref.grid, ref._sources, ref.chunk_layout)
    mapped = driver_for(ref.fields, ref.pml, ref.grid, ref._sources)
    assert tables.compare(host_tables(mapped)) == []
    ours, _, _ = build_case(FdtdDriver, Susceptibility, case)
    assert tables.compare(host_tables(ours)) == []
    assert tables.sources and all(len(cells) for _, cells, _ in tables.sources)


@needs_reference
def test_a_planted_difference_is_reported():
    ref = frozen_reference(CASES["lorentz_slab"])
    tables = build_desc(ref.fields, ref.pml, ref.grid, ref._sources, ref.chunk_layout)
    mapped = host_tables(driver_for(ref.fields, ref.pml, ref.grid, ref._sources))
    kms, sinv, kps = mapped.pml[(1, 2)]
    kms = kms.copy()
    kms[1] = np.nextafter(kms[1], np.float32(2))
    mapped.pml[(1, 2)] = (kms, sinv, kps)
    mapped.inv_eps = (mapped.inv_eps[0] * np.float32(1.0000001),) + mapped.inv_eps[1:]
    diffs = tables.compare(mapped)
    assert "pml kms (1, 2)" in diffs and any(d.startswith("inv_eps Ex") for d in diffs)


def test_plan_answers_false_for_other_fields_and_unknown_slots():
    plan = GB300Plan.__new__(GB300Plan)
    plan.fields, plan.mirror, plan.launches = object(), False, {}
    assert plan.dispatch("step_B", object()) is False
    assert plan.dispatch("not_a_slot", plan.fields) is False
    assert DRIVER_SLOTS == ("step_B", "fill_B", "update_H", "step_D", "fill_D", "update_E", "update_P")


def reference_shaped_fields(driver):
    """Arrays named as the reference's ``Fields`` holds them, plus its polarization states."""
    shape = driver.grid.shape
    dtype = np.complex64 if driver.complex_fields else np.float32
    fields = SimpleNamespace(**{c: np.zeros(shape, dtype) for c in FIELDS})
    states = []
    for _, volumes in driver._poles:
        driven = {c: np.zeros(shape, dtype) for c, v in zip(("Ex", "Ey", "Ez"), volumes) if v is not None}
        states.append(SimpleNamespace(P=driven, P_prev={c: np.zeros(shape, dtype) for c in driven}))
    fields.polarizations = states
    return fields


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere_pml", "lorentz_slab", "magnetic", "mixed"])
def test_dispatch_in_the_references_consult_order_leaves_the_reference_words(gpu, name):
    case = CASES[name]
    gold = golden_io.fields(name)
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    fields = reference_shaped_fields(driver)
    plan = GB300Plan(fields, driver)
    rng = np.random.default_rng(1)
    scribble = [rng.integers(0, n, 16) for n in driver.grid.shape]
    consults = ("step_B", "fill_B", "fill_folded_far_ghosts_B", "update_H", "step_D", "fill_D",
                "fill_folded_far_ghosts_D", "update_E", "update_P")
    for _ in range(case["steps"]):
        for slot in consults:
            assert plan.dispatch(slot, fields) is True
            # the reference driver's own passes between consults write its arrays
            # (magnetic deposit after step_B, electric after step_D, the wall passes)
            if slot == "step_B":
                fields.Bz[tuple(scribble)] += 1.0
            if slot == "step_D":
                fields.Dz[tuple(scribble)] -= 1.0
    for c in FIELDS:
        assert np.array_equal(getattr(fields, c), gold[c]), c
    for m, state in enumerate(fields.polarizations):
        for c, array in state.P.items():
            assert np.array_equal(array, gold[f"P{m}_{c}"]), f"P{m} {c}"
    assert plan.launches["step_B"] == case["steps"] and plan.report()["table"] == "gb300"
    plan.close()


@needs_reference
@pytest.mark.gpu
def test_plan_from_the_references_objects(gpu):  # runs only where the reference and a GPU meet
    ref = frozen_reference(CASES["sphere_pml"])
    plan = plan_fast_path(ref.fields, ref.pml, ref.grid, ref._sources, ref.chunk_layout, first_step=1)
    assert plan is not None and plan.driver.step_count == 1
    plan.close()
