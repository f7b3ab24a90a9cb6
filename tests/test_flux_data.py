"""Saved flux-plane transforms and the two-run normalisation idiom.

A flux monitor's ``get_dft_data`` / ``load_dft_data`` / ``load_minus_dft_data`` /
``scale_dfts`` / ``reset`` follow the reference's ``FluxMonitor`` (``dft.py:3261-3320``):
the saved transforms are host copies, loading replaces the accumulators, and the minus
form starts the second run at -E1, -H1 so its flux is that of the field difference.
Pinned against the reference's own two runs (``tests/golden/flux_normalization.npz``).
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, FluxDftData, FluxPlaneDft
from meep_gpu_gb300.dft import ELECTRIC, MAGNETIC
from oracle.oracle import Oracle, problem_from_driver
from tests.golden.cases import FLUX_NORM, build_flux_norm
from tests.golden_io import GOLDEN

STEPS = FLUX_NORM["steps"]


@pytest.fixture(scope="module")
def gold():
    with np.load(GOLDEN / "flux_normalization.npz") as data:
        return {k: data[k] for k in data.files}


def reference_data(gold) -> FluxDftData:
    return FluxDftData(planes=(FluxPlaneDft(E={n: gold[f"data_{n}"] for n in ELECTRIC},
                                            H={n: gold[f"data_{n}"] for n in MAGNETIC},
                                            frequencies=tuple(gold["frequencies"])),))


def test_loading_is_checked_and_changes_nothing_on_refusal(gold):
    _, flux = build_flux_norm(FdtdDriver, structure=True)
    good = reference_data(gold)
    with pytest.raises(TypeError):
        flux.load_dft_data({"Ex": gold["data_Ex"]})
    with pytest.raises(ValueError, match="flux plane"):
        flux.load_dft_data(FluxDftData(planes=good.planes * 2))
    plane = good.planes[0]
    with pytest.raises(ValueError, match="frequencies"):
        flux.load_dft_data(FluxDftData(planes=(FluxPlaneDft(plane.E, plane.H, plane.frequencies[:3]),)))
    shifted = tuple(f * 1.01 for f in plane.frequencies)
    with pytest.raises(ValueError, match="frequencies"):
        flux.load_dft_data(FluxDftData(planes=(FluxPlaneDft(plane.E, plane.H, shifted),)))
    with pytest.raises(ValueError, match="components"):
        flux.load_dft_data(FluxDftData(planes=(FluxPlaneDft({"Ex": plane.E["Ex"]}, plane.H, plane.frequencies),)))
    small = {n: b[:, :, :4] for n, b in plane.E.items()}
    with pytest.raises(ValueError, match="shape"):
        flux.load_dft_data(FluxDftData(planes=(FluxPlaneDft(small, plane.H, plane.frequencies),)))
    # nothing was loaded by the refusals
    assert all(not np.any(b) for b in flux.get_dft_data().planes[0].E.values())


def test_pending_load_scale_and_reset(gold):
    _, flux = build_flux_norm(FdtdDriver, structure=True)
    flux.load_dft_data(reference_data(gold))
    saved = flux.get_dft_data().planes[0]
    for name in flux.components:
        block = saved.E[name] if name in saved.E else saved.H[name]
        assert np.array_equal(block, gold[f"data_{name}"])
    normal = [n for n in ELECTRIC + MAGNETIC if n not in flux.components]
    assert all(not np.any((saved.E | saved.H)[n]) for n in normal)  # not accumulated: zero
    flux.scale_dfts(-1.0)
    minus = flux.get_dft_data().planes[0]
    assert np.array_equal(minus.E["Ey"], -gold["data_Ey"])
    flux.scale_dfts(0.5j)
    assert np.array_equal(flux.get_dft_data().planes[0].H["Hz"],
                          (-gold["data_Hz"] * np.complex64(0.5j)).astype(np.complex64))
    flux.reset()
    assert not np.any(flux.get_dft_data().planes[0].E["Ez"])


def test_oracle_started_from_minus_the_saved_transforms_gives_the_reference_flux(gold):
    """The semantics on the CPU: the float32 oracle's accumulators started at minus the
    reference's saved transforms reproduce the reference's normalised spectrum."""
    driver, flux = build_flux_norm(FdtdDriver, structure=True)
    oracle = Oracle(problem_from_driver(driver), "f32")
    acc = oracle.accumulators[0]
    for q, name in enumerate(flux.components):
        block = -gold[f"data_{name}"].reshape(len(flux.frequencies), -1)
        acc[q, :, 0] = block.real
        acc[q, :, 1] = block.imag
    oracle.run(STEPS)
    expected = gold["flux2_minus"]
    assert np.max(np.abs(oracle.flux_spectrum(0) - expected)) <= 1e-5 * np.max(np.abs(expected))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tensor", "direct"])
def test_normalisation_idiom_matches_the_reference(gpu, gold, mode):
    d1, f1 = build_flux_norm(FdtdDriver, structure=False)
    d1.dft_accumulation = mode
    d1.run(num_steps=STEPS)
    saved = f1.get_dft_data()
    plane = saved.planes[0]
    for name in f1.components:
        got = (plane.E | plane.H)[name]
        want = gold[f"data_{name}"]
        assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want)), name
    assert np.max(np.abs(f1.get_flux_spectrum() - gold["flux1"])) <= 1e-5 * np.max(np.abs(gold["flux1"]))
    expected = gold["flux2_minus"]
    for data in (saved, reference_data(gold)):  # our own transforms and the reference's
        d2, f2 = build_flux_norm(FdtdDriver, structure=True)
        d2.dft_accumulation = mode
        f2.load_minus_dft_data(data)
        d2.run(num_steps=STEPS)
        assert np.max(np.abs(f2.get_flux_spectrum() - expected)) <= 1e-4 * np.max(np.abs(expected))
        d2.close()
    d1.close()


@pytest.mark.gpu
def test_load_after_freeze_and_round_trip(gpu, gold):
    d, flux = build_flux_norm(FdtdDriver, structure=True)
    d.freeze()
    flux.load_dft_data(reference_data(gold))
    back = flux.get_dft_data().planes[0]
    for name in flux.components:
        assert np.array_equal((back.E | back.H)[name], gold[f"data_{name}"]), name
    d.run(num_steps=10)  # samples buffered, then read: the saved copy is not changed by them
    assert np.array_equal(back.E["Ey"], gold["data_Ey"])
    flux.reset()
    assert not np.any(flux.get_dft_data().planes[0].E["Ey"])
    d.close()
