"""Mirror symmetry: folded metallic axes (MEEP's ``mp.Mirror``).

A mirror plane halves its axis to MEEP's ``n - n//2 + 1`` stored cells from one cell
below the plane (reference ``grid.py:604``, ``vec.cpp`` ``halve``); cell 0 of every
component with Yee shift 0 there is the plane's ghost, written after each half's sources
from stored row 2 with the component's parity (``stepping.py:2004-2045``). The
reference's own folded runs pin the words (golden cases ``mirror_*``, checked by the
oracle and GPU parity suites); here: the grid, PML and source rules, the ghost lists
against the fill, and the physics — a folded run equals the unfolded run with the
parity-signed image sources on the cells both store.
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Mirror, Susceptibility, Unsupported
from meep_gpu_gb300.engine import fold_ghosts
from meep_gpu_gb300.grid import IYEE, Grid, mirror_parity
from oracle.oracle import Oracle, problem_from_driver
from tests.golden.cases import CASES, build_case


def test_periodic_folds_store_the_far_slot():
    grid = Grid((1.4, 1.3, 1.2), 10, boundaries="periodic", symmetry=("X", "Y"))
    assert grid.shape == (9, 9, 12)  # owned + 1: big_corner's plane, then the far ghost slot
    assert (grid.owned_cells(0), grid.owned_cells(1)) == (8, 8)
    # the second mirror at doubled n_full: two rows below the top at an even count, three
    # at an odd one (reference stepping.py:2361)
    assert (grid.far_reflect_row(0), grid.far_reflect_row(1), grid.far_reflect_row(2)) == (7, 6, None)


def test_folded_counts_origin_and_coordinates():
    grid = Grid((2.0, 1.5, 1.8), 10, boundaries="metallic", symmetry=(Mirror("X", -1), "y"))
    assert grid.shape_full == (20, 15, 18)
    assert grid.shape == (11, 9, 18)  # n - n//2 + 1 on both parities
    assert grid.origin_doubled(0) == grid.origin_doubled(1) == -2
    assert grid.origin_doubled(2) == -18
    assert grid.full_origin_doubled(1) == -14  # an odd count starts half a cell higher
    # cell 0 straddles the plane; the last stored cell of an odd count sits at +L/2
    assert np.isclose(grid.x[0], -0.05) and np.isclose(grid.x[1], 0.05)
    assert np.isclose(grid.y[-1], 0.75)
    assert grid.mirror_phase(0) == -1 and grid.mirror_phase(1) == 1 and grid.mirror_phase(2) is None
    assert not grid.axis_wraps(0) and grid.is_metallic(0)


def test_folds_that_are_not_stepped_are_refused():
    with pytest.raises(Unsupported, match="k_point"):
        Grid((2.0, 2.0, 2.0), 10, boundaries=("metallic", "periodic", "periodic"),
             k_point=(0, 0.2, 0), symmetry=("X",))
    with pytest.raises(ValueError, match="two mirror planes"):
        Grid((2.0, 2.0, 2.0), 10, boundaries="metallic", symmetry=("X", Mirror("x", -1)))
    with pytest.raises(ValueError):
        Mirror("W")
    with pytest.raises(ValueError):
        Mirror("X", 2)
    with pytest.raises(Unsupported, match="at least 4"):
        Grid((0.4, 2.0, 2.0), 10, boundaries="metallic", symmetry=("X",))


def test_mirror_parity_is_meeps_phase_shift():
    # reference sources.py:479-480: Mirror(X, +1) makes Ex, Hy, Hz odd and Ey, Ez, Hx even
    odd_even = {c: mirror_parity(c, 0, 1) for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    assert odd_even == {"Ex": -1, "Ey": 1, "Ez": 1, "Hx": 1, "Hy": -1, "Hz": -1}
    assert all(mirror_parity(c, 0, -1) == -v for c, v in odd_even.items())
    for axis in range(3):
        for q, name in enumerate("xyz"):
            assert mirror_parity("D" + name, axis, 1) == mirror_parity("E" + name, axis, 1)
            assert mirror_parity("B" + name, axis, 1) == mirror_parity("H" + name, axis, 1)


def test_pml_skips_the_plane_face_and_refuses_a_named_one():
    d = FdtdDriver((1.6, 1.6, 1.6), 10, force_complex_fields=False, boundaries="metallic",
                   symmetry=("X", Mirror("Z", -1)))
    assert d.setup_pml(3).faces == ((0.0, 3.0), (3.0, 3.0), (0.0, 3.0))
    with pytest.raises(ValueError, match="mirror plane"):
        d.setup_pml({"x": 3})
    assert d.setup_pml({"x": {"high": 2}, "y": 3}).faces == ((0.0, 2.0), (3.0, 3.0), (0.0, 0.0))


def test_sources_must_sit_in_the_stored_half_and_carry_the_parity():
    d = FdtdDriver((1.6, 1.6, 1.6), 10, force_complex_fields=False, boundaries="metallic",
                   symmetry=("X",))
    base = {"source_type": "gaussian", "frequency": 0.5, "fwidth": 0.3}
    with pytest.raises(ValueError, match="discards"):
        d.add_source(dict(base, component="Ez", center=(-0.3, 0, 0), size=(0, 0, 0)))
    with pytest.raises(ValueError, match="parity"):  # Ex is odd about an even X plane
        d.add_source(dict(base, component="Ex", center=(0, 0.1, 0), size=(0, 0, 0)))
    with pytest.raises(ValueError, match="uniform"):
        d.add_source(dict(base, component="Ex", center=(0, 0.1, 0), size=(0.4, 0, 0)))
    d.add_source(dict(base, component="Ex", center=(0, 0.1, 0), size=(0.4, 0, 0),
                      amp_func=lambda x, y, z: x))
    d.add_source(dict(base, component="Ey", center=(0, 0.1, 0), size=(0, 0, 0)))  # even: allowed
    assert len(d.sources) == 2


def _zero_metal(grid, family, volumes):
    for q in range(3):
        for b in range(3):
            if grid.is_metallic(b) and not grid.is_mirrored(b) and IYEE[family + "xyz"[q]][b] == 0:
                wall = [slice(None)] * 3
                wall[b] = 0
                volumes[q][tuple(wall)] = 0
    return volumes


def _fill_like_the_reference(grid, family, volumes):
    """cell 0 = parity * cell 2 per folded axis in x, y, z order, zero_metal, then the far
    slot of a folded periodic axis = parity * its reflect row."""
    out = [v.copy() for v in volumes]
    for q in range(3):
        comp = family + "xyz"[q]
        for a in range(3):
            if grid.is_mirrored(a) and IYEE[comp][a] == 0:
                dst = [slice(None)] * 3
                src = [slice(None)] * 3
                dst[a], src[a] = 0, 2
                out[q][tuple(dst)] = grid.parity(comp, a) * out[q][tuple(src)]
    out = _zero_metal(grid, family, out)
    for q in range(3):
        comp = family + "xyz"[q]
        for a in range(3):
            if grid.far_reflect_row(a) is not None and IYEE[comp][a] == 1:
                dst = [slice(None)] * 3
                src = [slice(None)] * 3
                dst[a], src[a] = -1, grid.far_reflect_row(a)
                out[q][tuple(dst)] = grid.parity(comp, a) * out[q][tuple(src)]
    return out


@pytest.mark.parametrize("boundaries", ["metallic", ("periodic", "metallic", "periodic"), "periodic"])
@pytest.mark.parametrize("symmetry", [("X",), (Mirror("Y", -1),), ("X", Mirror("Z", -1)),
                                      (Mirror("X", -1), "Y", "Z")])
def test_ghost_lists_are_the_fill(symmetry, boundaries):
    grid = Grid((1.2, 1.1, 1.4), 10, boundaries=boundaries, symmetry=symmetry)
    rng = np.random.default_rng(7)
    for family in ("B", "D"):
        # the step kernels have zeroed the walls (zero_metal) before the ghosts are written
        volumes = _zero_metal(grid, family, [rng.standard_normal(grid.shape).astype(np.float32)
                                             for _ in range(3)])
        expected = _fill_like_the_reference(grid, family, volumes)
        tables = fold_ghosts(grid, family)
        got = [v.copy() for v in volumes]
        for g, r, code in zip(tables["ghost"], tables["image"], tables["code"]):
            q = code & 3
            value = volumes[q].reshape(-1)[r]
            if code & 4:
                value = -value
            if code & 8:
                value = np.float32(0)
            got[q].reshape(-1)[g] = value
        for q in range(3):
            assert np.array_equal(got[q], expected[q]), (family, q)
        # every ghost images a stored word of its component that is not itself a ghost
        q = tables["code"].astype(np.int64) & 3
        keyed = lambda offsets: offsets.astype(np.int64) * 4 + q  # noqa: E731
        assert not np.intersect1d(keyed(tables["ghost"]), keyed(tables["image"])).size


def _mirror_pair(folded: bool, boundaries: str = "metallic"):
    """An even X and an odd Y plane under a PML, a dielectric slab and a Lorentz slab
    normal to z (a medium the planes leave invariant: a cell-centred medium that varies
    along a folded axis is not symmetric about the plane on the shift-0 lattice), an Ez
    point source; unfolded, the same run with the source's parity-signed images."""
    symmetry = (Mirror("X", 1), Mirror("Y", -1)) if folded else ()
    d = FdtdDriver((1.2, 1.0, 1.2), 10, force_complex_fields=False, boundaries=boundaries,
                   symmetry=symmetry)
    d.setup_pml(2 if boundaries == "metallic" else {"z": 2})
    x, y, z = d.grid.meshgrid()
    d.set_epsilon(np.where(np.abs(z - 0.1) < 0.2, 3.0, 1.0).astype(np.float32))
    d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05),
                         np.where(z < -0.15, 0.8, 0.0).astype(np.float32))
    base = {"source_type": "gaussian", "component": "Ez", "size": (0, 0, 0), "frequency": 0.8,
            "fwidth": 0.6}
    images = [(1, 1, 1.0)] if folded else [(1, 1, 1.0), (-1, 1, 1.0), (1, -1, -1.0), (-1, -1, -1.0)]
    for sx, sy, amp in images:  # Ez: even about X, odd about the odd Y plane
        d.add_source(dict(base, center=(0.25 * sx, 0.15 * sy, 0.1), amplitude=amp))
    flux = d.add_flux_monitor(fcen=0.8, df=0.4, nfreq=3, center=(0, 0, 0.3), size=(0.8, 0.6, 0),
                              decimation_factor=1)
    return d, flux


@pytest.mark.parametrize("boundaries", ["metallic", "periodic"])
def test_a_folded_run_is_the_unfolded_run_with_image_sources(boundaries):
    """The float64 oracle: the folded run's stored words (ghosts included, and on a
    periodic fold the far ghost slot past the second mirror) equal the unfolded run's at
    the same positions, and its flux through a plane spanning both halves equals the
    unfolded flux (the device sampling's images and signs)."""
    steps = 70
    runs = {}
    for folded in (True, False):
        driver, _ = _mirror_pair(folded, boundaries)
        oracle = Oracle(problem_from_driver(driver), "f64")
        oracle.run(steps)
        runs[folded] = (driver, oracle)
    (fd, fo), (ud, uo) = runs[True], runs[False]
    offset = [(ud.grid.shape[a] - 2) // 2 if fd.grid.is_mirrored(a) else 0 for a in range(3)]
    # a periodic fold's last stored row lies one cell past the unfolded window: its
    # image is the unfolded row 0 (one lattice vector over)
    unfolded = {c: uo.field(c) for c in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx",
                                          "Hy", "Hz")}
    if boundaries == "periodic":
        unfolded = {c: np.concatenate([v, v[:1]], axis=0) for c, v in unfolded.items()}
        unfolded = {c: np.concatenate([v, v[:, :1]], axis=1) for c, v in unfolded.items()}
    view = tuple(slice(offset[a], offset[a] + fd.grid.shape[a]) for a in range(3))
    scale = max(np.max(np.abs(unfolded[c])) for c in ("Ez", "Hx", "Hy"))
    for c in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz"):
        assert np.max(np.abs(fo.field(c) - unfolded[c][view])) <= 1e-12 * scale, c
    unfolded = uo.flux_spectrum(0)
    assert np.max(np.abs(fo.flux_spectrum(0) - unfolded)) <= 1e-10 * np.max(np.abs(unfolded))


def test_serving_and_adjoint_refuse_a_fold():
    from meep_gpu_gb300.adjoint import FluxAdjoint
    driver, flux, _ = build_case(FdtdDriver, Susceptibility, dict(CASES["mirror_pml"], lorentz=False))
    driver._poles.clear()
    with pytest.raises(Unsupported, match="mirror"):
        FluxAdjoint(driver, flux[0], box=((2, 4), (2, 4), (2, 4)), steps=10)


@pytest.mark.gpu
def test_chunked_and_part_by_part_runs_equal_one_run(gpu):
    """The ghosts' kept state carries across calls: runs of 1, 2, 17 and 40 steps, and a
    step launched part by part, give the reference's words."""
    from tests import golden_io
    gold = golden_io.fields("mirror_pml")
    case = CASES["mirror_pml"]
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    for chunk in (1, 2, 17, 39):
        driver.run(num_steps=chunk)
    engine = driver.engine
    import torch
    for part in range(3):
        engine.launch(driver.step_count, part)
    driver.step_count += 1
    torch.cuda.synchronize()
    for c in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Bx", "By", "Bz", "Hx", "Hy", "Hz"):
        assert np.array_equal(driver.get_field(c, cell_centered=False), gold[c]), c
    driver.close()


@pytest.mark.gpu
def test_the_batch_refuses_a_folded_plan(gpu):
    import ctypes

    import torch

    from meep_gpu_gb300 import _lib

    driver, _, _ = build_case(FdtdDriver, Susceptibility, dict(CASES["mirror_pml"], lorentz=False))
    engine = driver.freeze(autotune=False)
    lib = engine.lib
    nbytes = lib.mgb_batch_bytes(2, 64, 64)
    buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    handle = ctypes.c_void_p()
    _lib.check(lib, lib.mgb_batch_create(2, 64, 64, buf.data_ptr(), nbytes, ctypes.byref(handle)))
    engine.ensure_source_words(0, 10)
    assert lib.mgb_batch_set_slot(handle, 0, engine.handle, 10, engine._words.data_ptr()) == -3
    assert "mirror" in _lib.last_error(lib) or "magnetic" in _lib.last_error(lib)
    lib.mgb_batch_destroy(handle)
    driver.close()


def test_cell_centred_read_takes_the_image_past_a_periodic_fold():
    """The centred value on the last stored row of a folded periodic axis averages with
    the word one past it: its image about the second mirror, with the parity."""
    import torch

    d = FdtdDriver((1.4, 1.2, 1.2), 10, force_complex_fields=False, boundaries="periodic",
                   symmetry=(Mirror("X", -1),))
    rng = np.random.default_rng(3)
    words = {c: torch.from_numpy(rng.standard_normal(d.grid.shape).astype(np.float32))
             for c in ("Ex", "Ey", "Hx")}

    class Stub:
        def field(self, name):
            return words[name]

    d.engine = Stub()
    n = d.grid.shape[0]
    row = d.grid.far_reflect_row(0)
    hx = words["Hx"].numpy()
    # Hx has Yee shift 0 on x alone: the word past the top row n-1 sits at doubled
    # -2 + 2n, whose image about the second mirror is the far reflect row (reference
    # stepping.py:2361)
    from meep_gpu_gb300.dft import folded_site
    assert folded_site(d.grid, 0, 0, n) == (row, True)
    centred = d.get_field("Hx")
    sign = d.grid.parity("Hx", 0)
    expected_top = np.float32(0.5) * (hx[n - 1] + np.float32(sign) * hx[row])
    assert np.array_equal(centred[n - 1], expected_top)
    d.engine = None
