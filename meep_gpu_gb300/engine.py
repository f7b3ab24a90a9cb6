"""Device state of one frozen simulation and the calls into ``libmeepgb.so``.

The engine allocates every device array (as torch tensors: torch is the allocator and
the stream provider here, nothing more), fills the ``mgb_sim_desc`` the C ABI takes,
and drives ``mgb_step``. Layout in HBM, all float32 and C-ordered ``(nx, ny, nz)``:

* E, D, H: three full volumes each; one inverse-epsilon volume per distinct array
  (the isotropic case aliases one volume for all three components). Outside each H
  component's own-axis integer PML runs MEEP's H is B's word, so H carries B there;
* PML auxiliaries, read and written only on their membership runs: B on each H
  component's own-axis integer runs and the split-field ``fu`` of B (half lattice) and
  D (integer lattice) on the dsigu runs. Each is allocated as a full volume (HBM is
  plentiful) so a cell's auxiliary word sits at the cell's own offset and needs no index
  arithmetic; the cells outside the runs are never touched and move no bytes. The
  ``f_w`` of H and E volumes are allocated too (the adjoint keeps its multipliers of
  them there) but the forward step moves neither: ``f_w`` of H is B's old word and
  ``f_w`` of E is recomputed from the old D;
* polarization: two rotating buffers per pole and driven component, over the bounding
  box of the cells where any pole's sigma is nonzero (P stays zero elsewhere);
* DFT accumulators ``[ncomp][nfreq][re, im][cells]`` per monitor.
"""

from __future__ import annotations

import ctypes
import math
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .conductivity import coefficients, keeps_mask, piece_line
from .dft import COMPONENTS, FluxMonitor, _Monitor
from .grid import IYEE, Grid
from .pml import (HALF, INTEGER, PML, aux_shape, constitutive_aux_key, curl_aux_key,
                  identity_tables, no_pml_records, slab_index)
from .sources import Source, deposit_scales, deposit_words

FIELD_NAMES = ("E", "D", "H")
# Source words are uploaded in windows of this many steps.
SOURCE_WINDOW = 4096

# Kernel choices the autotuner times: (family, block_z, block_y, x_chunk); family 1 is
# the tile kernels (block shape fixed at 64 x 8, x_chunk used), family 0 the generic ones,
# family 2 the generic ones with the next plane's loads issued ahead, family 3 the tile
# kernels' warp-specialized form (E half only; the H half refuses it), families 4 and 5
# families 0 and 2 with each thread's x chunk prefetched into L2 before it marches.
AUTOTUNE_CANDIDATES = ((0, 32, 4, 4), (0, 32, 8, 4), (0, 32, 4, 8), (0, 64, 2, 8),
                       (0, 16, 8, 4), (0, 16, 16, 4), (0, 16, 8, 2), (0, 16, 8, 8), (0, 32, 2, 4),
                       (1, 64, 8, 4), (1, 64, 8, 8),
                       (2, 32, 4, 4), (2, 32, 4, 8), (2, 32, 8, 4), (2, 64, 2, 4), (2, 16, 8, 4),
                       (2, 32, 4, 2), (2, 32, 2, 4), (3, 64, 8, 4), (3, 64, 8, 8), (3, 64, 8, 16),
                       (4, 32, 4, 4), (4, 16, 8, 4), (4, 32, 4, 8), (4, 32, 8, 4), (4, 32, 4, 2),
                       (4, 32, 8, 2), (4, 32, 8, 8), (4, 64, 4, 4), (4, 16, 16, 4), (4, 32, 2, 4),
                       (5, 32, 4, 4), (5, 16, 8, 4), (5, 32, 4, 8), (5, 32, 2, 8), (5, 32, 4, 2),
                       # short x chunks: more CTAs for grids too small to fill the SMs
                       (0, 16, 16, 2), (4, 16, 16, 2), (0, 16, 16, 1), (0, 16, 8, 1))
_AUTOTUNE_CACHE: Dict[tuple, Tuple[int, int, int, int]] = {}


def autotune_candidates(grid: Grid) -> Tuple[Tuple[int, int, int, int], ...]:
    """The launch shapes timed for a grid. The marches put z on a warp's lanes, so a grid
    one cell deep in z (a 2-D run) also takes CTAs one cell wide in z with y on the lanes,
    and one a single cell wide in y (a 1-D run) CTAs one row high with z on the lanes."""
    extra = []
    if grid.shape[2] == 1:
        extra += [(f, 1, by, xc) for f in (0, 2, 4, 5) for by in (64, 128) for xc in (2, 4, 8)]
    if grid.shape[1] == 1:
        extra += [(f, bz, 1, xc) for f in (0, 2, 4, 5) for bz in (64, 128) for xc in (1, 2, 4)]
    return AUTOTUNE_CANDIDATES + tuple(extra)
# Wavefront choices the autotuner times against the best pair of per-half kernels:
# (march family, block_z, block_y, x_chunk, window), as kernel choice
# (6, family, block_z, block_y, x_chunk, window); family 0 the plain column marches, 2 the
# prefetching ones.
WAVE_CANDIDATES = ((2, 32, 4, 4, 3), (2, 32, 4, 4, 4), (2, 32, 8, 4, 3), (0, 32, 8, 4, 3), (0, 32, 4, 4, 3),
                   (2, 32, 4, 8, 2), (2, 64, 4, 4, 3))
WAVE_FAMILY = 6
# X-range splits (launches per half) the autotuner times against the unsplit halves.
SPLIT_CANDIDATES = (2, 3, 4, 6)
# Steps one wavefront launch may hold (the length of the counter table).
WAVE_MAX_STEPS = 256


def autotune_key(grid: Grid, pml: Optional[PML], npoles: int, ninv: int, lossy: bool = False) -> tuple:
    faces = pml.faces if (pml is not None and pml.is_active) else None
    return (grid.shape, grid.boundaries, faces, npoles, ninv, lossy)


def host_volumes(volumes: Sequence[torch.Tensor]) -> List[np.ndarray]:
    """Host copies of device volumes, one array per distinct volume: components that share
    a device volume share the host array, so an engine built from them (which keeps one
    device volume per distinct host array) aliases the same components. The autotuner's
    scratch engine is built this way: with three copies of an isotropic run's one
    inverse-epsilon volume its E half would read two more words a cell than the run's."""
    host: Dict[int, np.ndarray] = {}
    out = []
    for t in volumes:
        key = t.data_ptr()
        if key not in host:
            host[key] = t.cpu().numpy()
        out.append(host[key])
    return out


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _fill_accumulator(acc: torch.Tensor, q: int, values: Optional[np.ndarray]) -> None:
    """Write complex ``values [nf][cells]`` (None: zeros) into ``acc[q]`` ([nf][re, im][cells])."""
    if values is None:
        acc[q].zero_()
        return
    pair = np.stack([values.real, values.imag], axis=1).astype(np.float32)
    acc[q].copy_(torch.from_numpy(np.ascontiguousarray(pair)))


def fold_ghosts(grid: Grid, family: str) -> Dict[str, np.ndarray]:
    """The mirror-plane ghosts of one family ("B" or "D") as the library's lists
    (reference ``stepping.py:2004-2045`` ``fill_symmetry_bc_B/D``, ``MIRROR_SOURCE_INDEX``
    2, and ``:2092`` ``fill_folded_far_ghosts_B/D``): every cell with index 0 on a folded
    axis where the component has Yee shift 0, imaged from index 2, and on a folded
    periodic axis every cell in the last slot where it has shift 1, imaged from the far
    reflect row; each with the product of the component's parities over those axes (the
    near passes, ``zero_metal`` and the far passes compose to that), zero where it sits
    on a metallic wall of an unfolded axis. ``ghost`` / ``image``: int32 cell offsets;
    ``code``: component | 4 negate | 8 zero. Entries run in cell-offset order (x plane
    first, the components of one cell in turn), so each x plane's ghosts are one run of
    the list: the x-range split folds a range's ghosts with the range."""
    nx, ny, nz = grid.shape
    strides = (ny * nz, nz, 1)
    ghosts, images, codes = [], [], []
    for q in range(3):
        comp = family + "xyz"[q]
        shifts = IYEE[comp]
        # (axis, ghost row, image row) of every plane of this component's ghosts
        planes_of = [(a, 0, 2) for a in range(3) if grid.is_mirrored(a) and shifts[a] == 0]
        planes_of += [(a, grid.shape[a] - 1, grid.far_reflect_row(a)) for a in range(3)
                      if grid.far_reflect_row(a) is not None and shifts[a] == 1]
        if not planes_of:
            continue
        planes = []
        for a, row, _ in planes_of:
            ranges = [np.arange(n, dtype=np.int64) for n in grid.shape]
            ranges[a] = np.full(1, row, dtype=np.int64)
            ii, jj, kk = np.meshgrid(*ranges, indexing="ij")
            planes.append(ii.ravel() * strides[0] + jj.ravel() * strides[1] + kk.ravel())
        offsets = np.unique(np.concatenate(planes))
        coords = [offsets // strides[0], (offsets // strides[1]) % ny, offsets % nz]
        sign = np.ones(offsets.size, dtype=np.int64)
        image = list(coords)
        for a, row, source in planes_of:
            at = coords[a] == row
            image[a] = np.where(at, source, image[a])
            sign = np.where(at, sign * grid.parity(comp, a), sign)
        zero = np.zeros(offsets.size, dtype=bool)
        for b in range(3):
            if grid.is_metallic(b) and not grid.is_mirrored(b) and shifts[b] == 0:
                zero |= coords[b] == 0
        ghosts.append(offsets)
        images.append(image[0] * strides[0] + image[1] * strides[1] + image[2])
        codes.append(q | np.where(sign < 0, 4, 0) | np.where(zero, 8, 0))
    if not ghosts:
        return {"ghost": np.zeros(0, np.int32), "image": np.zeros(0, np.int32), "code": np.zeros(0, np.uint8)}
    ghost = np.concatenate(ghosts)
    order = np.argsort(ghost, kind="stable")
    return {"ghost": ghost[order].astype(np.int32),
            "image": np.concatenate(images)[order].astype(np.int32),
            "code": np.concatenate(codes)[order].astype(np.uint8)}


class Engine:
    """One simulation resident on one GPU."""

    def __init__(self, grid: Grid, pml: Optional[PML], inv_eps: Sequence[np.ndarray],
                 poles: Sequence[Tuple[object, Sequence[Optional[np.ndarray]]]],
                 sources: Sequence[Source], monitors: Sequence[_Monitor],
                 device: Optional[torch.device] = None, stream: Optional[torch.cuda.Stream] = None,
                 launch_shape: Optional[Tuple[int, int, int]] = None, autotune: bool = True,
                 kernels: Optional[Tuple[int, int, int, int]] = None,
                 dft_accumulation: Optional[str] = None,
                 conductivity: Optional[Dict[str, Optional[np.ndarray]]] = None,
                 part: str = "real", own_monitors: bool = True, create: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("meep_gpu_gb300 steps on a CUDA GPU and none is visible")
        self.lib = _lib.load()
        # "real": the fields a real run steps (or a complex run's real parts), driven by
        # real(A); "imag": a complex run's imaginary parts, driven by imag(A)
        self.part = part
        self.own_monitors = own_monitors
        self.grid = grid
        self.pml = pml if (pml is not None and pml.is_active) else None
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.stream = stream
        # electric points first, then magnetic ones: the library's table layout (each
        # kind keeps its own order, the order the reference deposits in)
        self.sources = [s for s in sources if not s.magnetic] + [s for s in sources if s.magnetic]
        self.monitors = list(monitors)
        shape = grid.shape
        dev = self.device
        zeros = lambda s: torch.zeros(s, dtype=torch.float32, device=dev)  # noqa: E731
        self.fields: Dict[str, torch.Tensor] = {}
        for family in FIELD_NAMES:
            for q, axis in enumerate("xyz"):
                self.fields[family + axis] = zeros(shape)
        # inverse epsilon: one device volume per distinct host array
        self.inv_eps: List[torch.Tensor] = []
        seen: Dict[int, torch.Tensor] = {}
        for array in inv_eps:
            key = id(array)
            if key not in seen:
                seen[key] = torch.from_numpy(np.ascontiguousarray(array, dtype=np.float32)).to(dev)
            self.inv_eps.append(seen[key])
        self.desc = _lib.MgbSimDesc()
        d = self.desc
        d.abi_version = _lib.MGB_ABI_VERSION
        d.nx, d.ny, d.nz = shape
        for axis in range(3):
            d.metallic[axis] = 1 if grid.is_metallic(axis) else 0
        d.dtdx = float(np.float32(grid.dt / grid.dx))
        d.invariant = sum(1 << a for a in range(3) if grid.is_invariant(a))
        for q, axis in enumerate("xyz"):
            d.E[q] = self.fields["E" + axis].data_ptr()
            d.D[q] = self.fields["D" + axis].data_ptr()
            d.H[q] = self.fields["H" + axis].data_ptr()
            d.inv_eps[q] = self.inv_eps[q].data_ptr()
        self.aux: Dict[str, torch.Tensor] = {}
        self.aux_cells: Dict[str, int] = {}  # membership cells each auxiliary touches
        self.coefficients: Dict[Tuple[str, int, int], torch.Tensor] = {}
        if self.pml is not None:
            d.pml_active = 1
            for (lattice, axis), table in self.pml.tables.items():
                for name in ("kms", "sinv", "kps"):
                    t = torch.from_numpy(getattr(table, name).copy()).to(dev)
                    self.coefficients[(name, lattice, axis)] = t
                    getattr(d, name)[lattice][axis] = t.data_ptr()
            self.records = self.pml.records
            for q in range(3):
                self._aux(d.B, "B", q, constitutive_aux_key("H", q))
                self._aux(d.fwH, "fwH", q, constitutive_aux_key("H", q))
                self._aux(d.fwE, "fwE", q, constitutive_aux_key("E", q))
                self._aux(d.fuB, "fuB", q, curl_aux_key("B", q))
                self._aux(d.fuD, "fuD", q, curl_aux_key("D", q))
        else:
            d.pml_active = 0
            self.records = no_pml_records(grid)
        self._setup_poles(poles)
        self._setup_conductivity(conductivity)
        self._setup_sources()
        self._setup_folds()
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        d.status = self.status.data_ptr()
        self._setup_monitors()
        self._pole_specs = list(poles)
        self.choice = None
        self.split = 0
        self.wave = None
        self.wave_buffer = None
        self.handle = None
        self._words: Optional[torch.Tensor] = None
        self._words_first = 0
        self._words_steps = 0
        # kernel families the plan may take: the generic ones only when a conductivity or
        # a Bloch phase is stepped (the library refuses the others for such a plan)
        self.allowed_families = ((0, 4) if (self.conductivity or grid.has_bloch)
                                 else (0, 2, 4, 5) if grid.dimensions != 3 else (0, 1, 2, 3, 4, 5))
        self._finish_args = (dft_accumulation, kernels, launch_shape, autotune)
        if create:
            self.finish()

    def finish(self) -> None:
        """Make the library's plan from the descriptor (deferred while a complex run's
        two parts are wired to each other), then its DFT buffers and kernel choice."""
        dft_accumulation, kernels, launch_shape, autotune = self._finish_args
        handle = ctypes.c_void_p()
        _lib.check(self.lib, self.lib.mgb_create(ctypes.byref(self.desc), ctypes.byref(handle)))
        self.handle = handle
        self._setup_dft_buffers(dft_accumulation)
        if kernels is not None:
            self.select(tuple(kernels) if not isinstance(kernels[0], (tuple, list)) else kernels)
        elif launch_shape is not None:
            self.set_launch_shape(*launch_shape)
        elif autotune and os.environ.get("MEEPGB_AUTOTUNE", "1") != "0":
            self.autotune()

    # --- setup --------------------------------------------------------------------------
    def _aux(self, slot, name: str, q: int, key: Tuple[int, int]) -> None:
        lattice, axis = key
        record = self.records[key]
        # A full volume, of which the kernels touch only the membership cells: the
        # auxiliary word of a cell sits at the cell's own offset.
        tensor = torch.zeros(self.grid.shape, dtype=torch.float32, device=self.device)
        self.aux[f"{name}{'xyz'[q]}"] = tensor
        self.aux_cells[f"{name}{'xyz'[q]}"] = (
            int(np.prod(aux_shape(self.grid, record, axis))))
        entry = slot[q]
        entry.data = tensor.data_ptr()
        entry.axis = axis
        entry.a0, entry.a1, entry.b0, entry.b1 = record

    def _setup_poles(self, poles) -> None:
        d = self.desc
        self.pole_tensors: List[dict] = []
        d.npoles = len(poles)
        if not poles:
            return
        if len(poles) > _lib.MGB_MAX_POLES:
            raise _lib.MeepGBError(-3, f"at most {_lib.MGB_MAX_POLES} susceptibility poles are stepped")
        support = np.zeros(self.grid.shape, dtype=bool)
        for _, sigmas in poles:
            for sigma in sigmas:
                if sigma is not None:
                    support |= (sigma != 0)
        box = []
        for axis in range(3):
            other = tuple(a for a in range(3) if a != axis)
            line = support.any(axis=other)
            idx = np.flatnonzero(line)
            if idx.size == 0:
                idx = np.array([0])
            box += [int(idx[0]), int(idx[-1]) + 1]
        self.pbox = tuple(box)
        d.pbox[:] = box
        slices = (slice(box[0], box[1]), slice(box[2], box[3]), slice(box[4], box[5]))
        bshape = (box[1] - box[0], box[3] - box[2], box[5] - box[4])
        for m, (susceptibility, sigmas) in enumerate(poles):
            const = susceptibility.realnum_constants(self.grid.dt)
            pole = d.poles[m]
            pole.two_minus_od = float(const.two_minus_od)
            pole.gamma1 = float(const.gamma1)
            pole.omega0dtsqr = float(const.omega0dtsqr)
            pole.gamma1inv = float(const.gamma1inv)
            kept = {}
            for q in range(3):
                sigma = sigmas[q]
                if sigma is None:
                    pole.sigma[q] = None
                    continue
                s = torch.from_numpy(np.ascontiguousarray(sigma[slices], dtype=np.float32)).to(self.device)
                p0 = torch.zeros(bshape, dtype=torch.float32, device=self.device)
                p1 = torch.zeros(bshape, dtype=torch.float32, device=self.device)
                kept[q] = (s, p0, p1)
                pole.sigma[q] = s.data_ptr()
                pole.p[q][0] = p0.data_ptr()
                pole.p[q][1] = p1.data_ptr()
            self.pole_tensors.append(kept)

    def _setup_conductivity(self, conductivity) -> None:
        """D and B conductivity: condfac / condinv volumes per lossy component and,
        under a PML, its conductive-stage history, the chunk of every stored row and the
        mask of the chunks that keep the component's conductivity."""
        self.conductivity = {k: v for k, v in (conductivity or {}).items() if v is not None}
        self.cond_tensors: Dict[str, torch.Tensor] = {}
        self.cond_history: Dict[str, torch.Tensor] = {}
        self.cond_desc = None
        if not self.conductivity:
            return
        grid, dev = self.grid, self.device
        cd = _lib.MgbConductivity()
        for name, sigma in self.conductivity.items():
            side = 0 if name[0] == "B" else 1
            q = "xyz".index(name[1])
            fac, inv = coefficients(sigma, grid.dt)
            self.cond_tensors[name + ".condfac"] = torch.from_numpy(fac).to(dev)
            self.cond_tensors[name + ".condinv"] = torch.from_numpy(inv).to(dev)
            cd.condfac[side][q] = self.cond_tensors[name + ".condfac"].data_ptr()
            cd.condinv[side][q] = self.cond_tensors[name + ".condinv"].data_ptr()
            if self.pml is not None:
                history = torch.zeros(grid.shape, dtype=torch.float32, device=dev)
                self.cond_history[name] = history
                cd.fcond[side][q] = history.data_ptr()
                cd.keeps[side][q] = keeps_mask(grid, self.pml.faces, sigma)
        if self.pml is not None:
            for lattice in (INTEGER, HALF):
                for axis in range(3):
                    line = piece_line(grid.shape[axis], self.pml.faces[axis], lattice, grid.axis_wraps(axis),
                                      grid.owned_cells(axis))
                    t = torch.from_numpy(line).to(dev)
                    self.cond_tensors[f"chunk_of.{lattice}.{axis}"] = t
                    cd.chunk_of[lattice][axis] = t.data_ptr()
        self.cond_desc = cd
        self.desc.conductivity = ctypes.pointer(cd)

    def _setup_folds(self) -> None:
        """The ghost lists of the mirror-folded axes (:func:`fold_ghosts`) on the device,
        with the zeroed scratch the library keeps each ghost's state in."""
        grid = self.grid
        d = self.desc
        self.fold_tables: Dict[str, torch.Tensor] = {}
        if not grid.has_symmetry:
            return
        for axis in range(3):
            d.mirror[axis] = grid.mirror_phase(axis) or 0
            d.full[axis] = grid.shape_full[axis]
        for h, family in ((0, "B"), (1, "D")):
            tables = fold_ghosts(grid, family)
            count = int(tables["ghost"].size)
            d.fold.count[h] = count
            if count == 0:
                continue
            for name, array in tables.items():
                tensor = torch.from_numpy(array).to(self.device)
                self.fold_tables[f"{name}{h}"] = tensor
                getattr(d.fold, name)[h] = tensor.data_ptr()
            saved = torch.zeros(_lib.MGB_FOLD_WORDS * count, dtype=torch.float32, device=self.device)
            self.fold_tables[f"saved{h}"] = saved
            d.fold.saved[h] = saved.data_ptr()

    def _setup_sources(self) -> None:
        d = self.desc
        # a source on a lossy D or B component deposits current * dt * condinv at its cell
        condinv = {}
        for index, name in enumerate(("Dx", "Dy", "Dz", "Bx", "By", "Bz")):
            sigma = self.conductivity.get(name)
            if sigma is not None:
                condinv[index] = coefficients(sigma, self.grid.dt)[1]
        self.src_scales = deposit_scales(self.sources, condinv)
        cells: List[int] = []
        comps: List[int] = []
        ny, nz = self.grid.ny, self.grid.nz
        for source in self.sources:
            for (i, j, k) in source.cells:
                cells.append((i * ny + j) * nz + k)
                comps.append(source.comp_index)
        d.nsrc = len(cells)
        if not cells:
            return
        self.src_cell = torch.tensor(cells, dtype=torch.int64, device=self.device)
        self.src_comp = torch.tensor(comps, dtype=torch.int32, device=self.device)
        d.src_cell = self.src_cell.data_ptr()
        d.src_comp = self.src_comp.data_ptr()
        d.nsrc_magnetic = sum(len(s.cells) for s in self.sources if s.magnetic)
        for magnetic, box in ((False, d.src_box), (True, d.src_box_magnetic)):
            ijk = np.array([c for s in self.sources if s.magnetic == magnetic for c in s.cells]).reshape(-1, 3)
            if ijk.size == 0:
                box[:] = [0, 0, 0, 0, 0, 0]
                continue
            lo, hi = ijk.min(axis=0), ijk.max(axis=0) + 1
            box[:] = [int(lo[0]), int(hi[0]), int(lo[1]), int(hi[1]), int(lo[2]), int(hi[2])]

    def _setup_monitors(self) -> None:
        d = self.desc
        if len(self.monitors) > _lib.MGB_MAX_MONITORS:
            raise _lib.MeepGBError(-3, f"at most {_lib.MGB_MAX_MONITORS} monitors per simulation")
        d.nmonitors = len(self.monitors)
        self.monitor_tensors = []
        for index, monitor in enumerate(self.monitors):
            entry = d.monitors[index]
            entry.region[:] = list(monitor.region)
            entry.ncomp = len(monitor.components)
            for q, comp in enumerate(monitor.components):
                entry.comp[q] = COMPONENTS.index(comp)
            entry.nfreq = monitor.num_frequencies
            entry.decimation = monitor.decimation_factor
            entry.scale = monitor.scale
            entry.dt = self.grid.dt
            omega = torch.from_numpy(monitor.omegas.copy()).to(self.device)
            acc = torch.zeros((entry.ncomp, entry.nfreq, 2, monitor.cells), dtype=torch.float32,
                              device=self.device)
            entry.omega = omega.data_ptr()
            entry.acc = acc.data_ptr()
            weights = None
            if isinstance(monitor, FluxMonitor):
                weights = torch.from_numpy(monitor.weights.reshape(-1).copy()).to(self.device)
            self.monitor_tensors.append((omega, acc, weights))
            if not self.own_monitors:
                continue
            monitor.accumulator = acc
            monitor._engine = self
            pending = getattr(monitor, "_pending", None)
            if pending is not None:  # transforms loaded before the run froze
                for q, name in enumerate(monitor.components):
                    _fill_accumulator(acc, q, pending[name].reshape(monitor.num_frequencies, -1))
                monitor._pending = None

    def _setup_dft_buffers(self, mode: Optional[str]) -> None:
        """Tensor-core accumulation (``"tensor"``, the default; ``MEEPGB_DFT`` overrides
        it) buffers MGB_DFT_DEPTH samples per monitor and contracts them on the tensor
        cores; ``"direct"`` adds every sample into the accumulators as it is taken."""
        mode = mode or os.environ.get("MEEPGB_DFT", "tensor")
        if mode not in ("tensor", "direct"):
            raise ValueError(f"DFT accumulation is 'tensor' or 'direct', not {mode!r}")
        self.dft_accumulation = mode
        self.dft_samples: List[Optional[torch.Tensor]] = [None] * len(self.monitors)
        self.dft_scratch = None
        if mode != "tensor" or not self.monitors:
            return
        eligible = [m.num_frequencies <= _lib.MGB_DFT_MAX_FREQ for m in self.monitors]
        if not any(eligible):
            return
        nbytes = max(self.lib.mgb_dft_scratch_bytes(m.num_frequencies)
                     for m, ok in zip(self.monitors, eligible) if ok)
        self.dft_scratch = torch.empty(nbytes // 4, dtype=torch.float32, device=self.device)
        for index, (monitor, ok) in enumerate(zip(self.monitors, eligible)):
            if not ok:
                continue
            samples = torch.empty((_lib.MGB_DFT_DEPTH, len(monitor.components) * monitor.cells),
                                  dtype=torch.float32, device=self.device)
            _lib.check(self.lib, self.lib.mgb_set_dft_buffer(self.handle, index, samples.data_ptr(),
                                                             self.dft_scratch.data_ptr(), nbytes))
            self.dft_samples[index] = samples

    def read_accumulator(self, monitor, q: int) -> np.ndarray:
        """Complex64 host copy ``[nf][cells]`` of component ``q`` of a monitor (buffered
        samples contracted first)."""
        return self.device_accumulator(monitor, q).cpu().numpy()

    def device_accumulator(self, monitor, q: int, imag: Optional["Engine"] = None) -> torch.Tensor:
        """Component ``q`` of a monitor as a complex64 device tensor ``[nf][cells]``,
        interleaved by the library (``mgb_read_accumulator``) so the host copy is one
        transfer; with ``imag`` (the imaginary-part plan of a complex run), the complex
        sum of the two parts' transforms."""
        index = self.monitors.index(monitor)
        nf, cells = self.monitor_tensors[index][1].shape[1], self.monitor_tensors[index][1].shape[3]
        out = torch.empty((nf, cells), dtype=torch.complex64, device=self.device)
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.lib, self.lib.mgb_read_accumulator(
            self.handle, None if imag is None else imag.handle, index, q, out.data_ptr(), stream.cuda_stream))
        current = torch.cuda.current_stream(self.device)
        if current != stream:
            current.wait_stream(stream)
        return out

    def write_accumulator(self, monitor, q: int, values: Optional[np.ndarray]) -> None:
        """Replace component ``q`` of a monitor by ``values`` (``[nf][cells]``; None: zero)."""
        self.flush_dft()
        acc = self.monitor_tensors[self.monitors.index(monitor)][1]
        _fill_accumulator(acc, q, values)

    def flush_dft(self) -> None:
        """Add buffered DFT samples to the accumulators; the current stream then sees them."""
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(self.lib, self.lib.mgb_dft_flush(self.handle, stream.cuda_stream))
        current = torch.cuda.current_stream(self.device)
        if current != stream:
            current.wait_stream(stream)

    # --- stepping -----------------------------------------------------------------------
    def set_launch_shape(self, block_z: int, block_y: int, x_chunk: int) -> None:
        _lib.check(self.lib, self.lib.mgb_set_launch_shape(self.handle, block_z, block_y, x_chunk))

    def _stream_handle(self) -> int:
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        return stream.cuda_stream

    def ensure_source_words(self, first_step: int, steps: int) -> None:
        """Upload the float64 deposit words covering ``[first_step, first_step + steps)``."""
        if self.desc.nsrc == 0 or steps <= 0:
            return
        if (self._words is not None and first_step >= self._words_first
                and first_step + steps <= self._words_first + self._words_steps):
            return
        count = max(steps, SOURCE_WINDOW)
        host = deposit_words(self.sources, first_step, count, self.grid.dt, self.src_scales, self.part)
        # The previous table may still be read by queued kernels: keep it alive until
        # the stream has passed them.
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        words = torch.from_numpy(host).to(self.device, non_blocking=False)
        if self._words is not None:
            self._words.record_stream(stream)
        self._words = words
        self._words_first = first_step
        self._words_steps = count
        _lib.check(self.lib, self.lib.mgb_set_source_words(self.handle, words.data_ptr(),
                                                             first_step, count))

    def step(self, first_step: int, nsteps: int) -> None:
        """Queue steps ``first_step .. first_step + nsteps - 1`` (asynchronous)."""
        done = 0
        while done < nsteps:
            chunk = min(nsteps - done, SOURCE_WINDOW)
            self.ensure_source_words(first_step + done, chunk)
            _lib.check(self.lib, self.lib.mgb_step(self.handle, first_step + done, chunk,
                                                   self._stream_handle()))
            done += chunk

    @property
    def uses_tiles(self) -> bool:
        """Whether the plan steps with the TMA tile kernels (else the generic ones)."""
        return bool(self.lib.mgb_uses_tiles(self.handle))

    @property
    def wave_eligible(self) -> bool:
        """Whether the wavefront path can step this plan (a 3-D run, metallic x, no folds,
        no Bloch phase, no conductivity)."""
        grid = self.grid
        return (grid.is_metallic(0) and not grid.has_symmetry and not grid.has_bloch
                and not self.conductivity and grid.dimensions == 3)

    @property
    def split_eligible(self) -> bool:
        """Whether the halves can be split into x-range launches (metallic x, no Bloch
        phase, generic kernel families; a folded run folds each range's ghosts with it)."""
        grid = self.grid
        return grid.is_metallic(0) and not grid.has_bloch and not self.uses_tiles

    def set_split(self, ranges: int) -> None:
        """Launch each half as ``ranges`` x-range launches on the plan's streams (0 or 1:
        one launch per half)."""
        _lib.check(self.lib, self.lib.mgb_set_split(self.handle, int(ranges)))
        self.split = int(ranges) if ranges > 1 else 0

    def set_wave(self, choice: Optional[Tuple[int, int, int, int, int]]) -> None:
        """Step with the wavefront path, (march family, block_z, block_y, x_chunk, window),
        or leave it (None). The counter buffer is this engine's (a torch allocation)."""
        stream = self._stream_handle()
        if choice is None:
            _lib.check(self.lib, self.lib.mgb_set_wave(self.handle, 0, 32, 4, 4, 1, 1, None, 0, stream))
            self.wave = None
            self.wave_buffer = None
            return
        family, bz, by, xc, window = (int(v) for v in choice)
        nbytes = self.lib.mgb_wave_bytes(self.handle, xc, window, WAVE_MAX_STEPS)
        if nbytes == 0:
            raise ValueError(f"bad wavefront choice {choice}")
        buffer = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.device)
        offset = (-buffer.data_ptr()) % 256
        _lib.check(self.lib, self.lib.mgb_set_wave(self.handle, family, bz, by, xc, window, WAVE_MAX_STEPS,
                                                   buffer.data_ptr() + offset, nbytes, stream))
        self.wave = (family, bz, by, xc, window)
        self.wave_buffer = buffer

    def select(self, choice) -> None:
        """Apply a kernel choice: one (family, block_z, block_y, x_chunk) for both halves,
        or a pair of them (H half, E half); (6, family, block_z, block_y, x_chunk, window)
        steps with the wavefront path (the halves keep their choice for single launches)."""
        if len(choice) == 6 and int(choice[0]) == WAVE_FAMILY:
            self.set_wave(tuple(int(v) for v in choice[1:]))
            return
        if len(choice) in (3, 4) and isinstance(choice[0], (tuple, list)):
            # (H half, E half, wavefront choice or None[, x-range split]): an autotuned result
            self.select((choice[0], choice[1]))
            self.set_wave(choice[2])
            if len(choice) == 4:
                self.set_split(choice[3])
            return
        if len(choice) == 2 and isinstance(choice[0], (tuple, list)):
            h, e = (tuple(int(v) for v in c) for c in choice)
        else:
            h = e = tuple(int(v) for v in choice)
        for part, (family, bz, by, xc) in enumerate((h, e)):
            if family in (1, 3):
                bz, by = 32, 8  # the tile kernels' block is fixed; the shape check still applies
            _lib.check(self.lib, self.lib.mgb_select_half(self.handle, part, family, bz, by, xc))
        self.choice = (h, e)

    def autotune(self, steps: int = 8):
        """Pick the fastest kernel choice of each half for this grid and apply them.

        Candidates are timed (CUDA events around each half) on a scratch engine with the
        same grid, absorber, materials and poles but zero fields and no sources or
        monitors, so this simulation's state is untouched; the H and E halves are
        separate launches, so each keeps its own fastest candidate. The result is cached
        per configuration for the life of the process.
        """
        key = autotune_key(self.grid, self.pml, len(getattr(self, "pole_tensors", [])),
                           len({t.data_ptr() for t in self.inv_eps}), bool(self.conductivity))
        key = key + (self.allowed_families,)
        if key in _AUTOTUNE_CACHE:
            self.select(_AUTOTUNE_CACHE[key])
            return self.choice
        scratch = Engine(self.grid, self.pml, host_volumes(self.inv_eps),
                         self._pole_specs, [], [], device=self.device, autotune=False,
                         conductivity=self.conductivity)
        stream = torch.cuda.current_stream(self.device)
        best = [None, None]
        best_ms = [float("inf"), float("inf")]
        timed: List[Dict[tuple, float]] = [{}, {}]  # every candidate's time, per half
        for choice in autotune_candidates(self.grid):
            if choice[0] not in self.allowed_families:
                continue
            # a candidate one half refuses is timed on the other half only
            applies = []
            for part in (0, 1):
                try:
                    family, bz, by, xc = choice
                    if family in (1, 3):
                        bz, by = 32, 8
                    _lib.check(self.lib, self.lib.mgb_select_half(scratch.handle, part, family, bz, by, xc))
                    applies.append(part)
                except _lib.MeepGBError:
                    _lib.check(self.lib, self.lib.mgb_select_half(scratch.handle, part, 0, 32, 4, 4))
            if not applies:
                continue
            for n in range(2):
                scratch.launch(n, 0, stream)
                scratch.launch(n, 1, stream)
            marks = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
            for t, ev in enumerate(marks):
                ev[0].record(stream)
                scratch.launch(2 + t, 0, stream)
                ev[1].record(stream)
                scratch.launch(2 + t, 1, stream)
                ev[2].record(stream)
            marks[-1][2].synchronize()
            for part in applies:
                # the fastest of the timed launches: the least disturbed by anything else
                ms = float(np.min([ev[part].elapsed_time(ev[part + 1]) for ev in marks]))
                timed[part][choice] = ms
                if ms < best_ms[part]:
                    best[part], best_ms[part] = choice, ms
        wave = None
        # the wavefront path is timed only on request: on the benchmarked grids it steps
        # slower than the best pair of per-half kernels
        if self.wave_eligible and os.environ.get("MEEPGB_WAVE", "0") == "1":
            wave = self._tune_wave(scratch, (best[0], best[1]), stream)
        split = 0
        if (wave is None and os.environ.get("MEEPGB_SPLIT", "1") != "0" and self.grid.is_metallic(0)
                and not self.grid.has_bloch):
            # the three fastest single launches of each half, paired and timed on whole
            # steps with every split: the fastest launch alone is not always the fastest
            # when the ranges of both halves overlap, and single launches a few per cent
            # apart can swap places (on the 192^3 sphere the E half that steps fastest
            # split came third alone)
            tops = [sorted(timed[part], key=timed[part].get)[:3] or [best[part]] for part in (0, 1)]
            best_step = float("inf")
            for h in tops[0]:
                for e in tops[1]:
                    ranges, ms = self._tune_split(scratch, (h, e), stream, with_time=True)
                    if ms < best_step:
                        best_step, best[0], best[1], split = ms, h, e, ranges
        scratch.close()
        del scratch
        _AUTOTUNE_CACHE[key] = (best[0], best[1], wave, split)
        self.select((best[0], best[1], wave, split))
        self.autotune_ms = best_ms[0] + best_ms[1]
        return self.choice

    def _run_ms(self, scratch: "Engine", stream, steps: int = 48) -> float:
        """The fastest of three timed runs of ``steps`` whole steps on the scratch engine
        (long enough that candidates a few per cent apart are told apart)."""
        scratch.step(0, 4)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best_ms = float("inf")
        for _ in range(3):
            start.record(stream)
            scratch.step(4, steps)
            end.record(stream)
            end.synchronize()
            best_ms = min(best_ms, start.elapsed_time(end))
        return best_ms

    def _tune_split(self, scratch: "Engine", halves, stream, with_time: bool = False):
        """The x-range split that steps fastest (0: none), whole steps timed; with
        ``with_time`` also that split's time (ms per timed run). More ranges are kept
        only when they step at least 1 % faster than fewer: on the scratch engine 3 and 4
        ranges of the 192^3 sphere time within 0.3 % of each other, while on the
        simulation itself 4 ranges stepped up to 3 % slower."""
        scratch.select(halves)
        scratch.set_split(0)
        best, best_ms = 0, self._run_ms(scratch, stream)
        for ranges in SPLIT_CANDIDATES:
            if ranges * 2 > self.grid.shape[0] or not scratch.split_eligible:
                continue
            scratch.set_split(ranges)
            ms = self._run_ms(scratch, stream)
            if ms < 0.99 * best_ms:
                best, best_ms = ranges, ms
        scratch.set_split(0)
        return (best, best_ms) if with_time else best

    def _tune_wave(self, scratch: "Engine", halves, stream, steps: int = 24):
        """The fastest wavefront choice, if it steps a run of ``steps`` steps faster than
        the chosen pair of per-half kernels (whole steps timed with CUDA events)."""
        def run_ms() -> float:
            scratch.step(0, 4)
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            best_ms = float("inf")
            for _ in range(2):
                start.record(stream)
                scratch.step(4, steps)
                end.record(stream)
                end.synchronize()
                best_ms = min(best_ms, start.elapsed_time(end))
            return best_ms

        scratch.select(halves)
        scratch.set_wave(None)
        best, best_ms = None, run_ms()
        for choice in WAVE_CANDIDATES:
            try:
                scratch.set_wave(choice)
            except (_lib.MeepGBError, ValueError):
                continue
            ms = run_ms()
            if scratch.device_status_word() & self.STATUS_WAVE_TIMEOUT:
                raise RuntimeError("a wavefront wait ran out on the device while the autotuner timed it")
            if ms < best_ms:
                best, best_ms = choice, ms
        scratch.set_wave(None)
        return best

    def launch(self, step: int, part: int, stream=None) -> None:
        """Launch one kernel of one step: 0 the H half, 1 the E half, 2 the monitors."""
        if part < 2:
            self.ensure_source_words(step, 1)
        handle = (stream if stream is not None else
                  (self.stream if self.stream is not None else torch.cuda.current_stream(self.device)))
        _lib.check(self.lib, self.lib.mgb_launch(self.handle, step, part, handle.cuda_stream))

    def algorithmic_bytes(self) -> Dict[str, int]:
        """Minimum HBM bytes one launch of each step kernel must move.

        H half: read E (3 volumes) and H (3), write H (3); on the PML slabs read and
        write ``fu`` of B and the slab B (``f_w`` of H is B's old word there: no bytes).
        E half: read H (3 volumes: the slab word or B's) and D (3) and each distinct
        inverse-epsilon volume, write D (3) and E (3); on the slabs read and write ``fu``
        of D and read E (``f_w`` of E is recomputed from the old D); per pole and driven
        component read
        P, P_prev and sigma and write P' over the polarization box.
        """
        cells = self.grid.total_cells
        word = 4
        aux = lambda name: sum(self.aux_cells[f"{name}{a}"] for a in "xyz") if self.pml is not None else 0  # noqa: E731
        h = 9 * cells + 2 * aux("fuB") + 2 * aux("B")
        distinct_inv = len({t.data_ptr() for t in self.inv_eps})
        e = (12 + distinct_inv) * cells + 2 * aux("fuD") + aux("fwE")
        for kept in getattr(self, "pole_tensors", []):
            for _, (s, p0, _p1) in kept.items():
                e += 4 * int(p0.numel())
        # a lossy component reads its condfac and condinv volumes (its conductive-stage
        # history, touched on part of the dsig membership only, is left out: a lower bound)
        for name in self.conductivity:
            if name[0] == "B":
                h += 2 * cells
            else:
                e += 2 * cells
        return {"h_half": word * h, "e_half": word * e}

    # status bits the kernels set: 1 a non-finite E was written; 2 a tile kernel's wait
    # for its shared-memory copies timed out; 4 a tensor-core contraction's wait timed out;
    # 8 a wavefront kernel's wait for the chunks it reads timed out
    STATUS_NONFINITE, STATUS_TILE_TIMEOUT, STATUS_MMA_TIMEOUT, STATUS_WAVE_TIMEOUT = 1, 2, 4, 8

    def device_status_word(self) -> int:
        """The raw status word (one small device-to-host read)."""
        return int(self.status.item())

    def device_status(self) -> int:
        """The status word (one small device-to-host read); raises if a kernel timed out."""
        word = int(self.status.item())
        timeouts = self.STATUS_TILE_TIMEOUT | self.STATUS_MMA_TIMEOUT | self.STATUS_WAVE_TIMEOUT
        if word & timeouts:
            what = []
            if word & self.STATUS_TILE_TIMEOUT:
                what.append("a tile kernel's wait for its staged planes")
            if word & self.STATUS_MMA_TIMEOUT:
                what.append("a tensor-core contraction's wait for its MMAs")
            if word & self.STATUS_WAVE_TIMEOUT:
                what.append("a wavefront kernel's wait for the chunks it reads")
            raise RuntimeError(f"{' and '.join(what)} timed out on the device; the results of "
                               "the steps since the last check are not valid")
        return word

    def nonfinite(self) -> bool:
        """Whether a non-finite E has been written (raises on a device timeout)."""
        return bool(self.device_status() & self.STATUS_NONFINITE)

    def queue_field_energy(self, out: torch.Tensor) -> None:
        """Add this plan's sum |E|^2 eps + |B|^2 (float64, on the device) into ``out``."""
        _lib.check(self.lib, self.lib.mgb_field_energy(self.handle, out.data_ptr(), self._stream_handle()))

    def energy_word(self) -> torch.Tensor:
        """A zeroed device double, zeroed on the stream the plan steps on."""
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(stream):
            return torch.zeros(1, dtype=torch.float64, device=self.device)

    def field_energy(self) -> float:
        """The divergence guard's scalar (reference ``FdtdDriver._field_energy``,
        driver.py:3634): one device reduction and one 8-byte read."""
        out = self.energy_word()
        self.queue_field_energy(out)
        return float(out.item())

    # --- read-out -----------------------------------------------------------------------
    def field(self, name: str) -> torch.Tensor:
        """Device tensor of one component's stored Yee words (H composed from B and slab)."""
        if name[0] in "EDH":
            return self.fields[name]
        if name[0] == "B":
            q = "xyz".index(name[1])
            h = self.fields["H" + name[1]]
            if self.pml is None:
                return h
            b = h.clone()
            record = self.records[(INTEGER, q)]
            rows = np.flatnonzero(slab_index(record, np.arange(self.grid.shape[q])) >= 0)
            if rows.size:
                index = [slice(None)] * 3
                index[q] = torch.from_numpy(rows).to(self.device)
                b[tuple(index)] = self.aux["B" + name[1]][tuple(index)]
            return b
        raise ValueError(f"unknown component {name!r}")

    def queue_flux_spectrum(self, monitor: FluxMonitor):
        """Queue one flux reduction and its read-back into pinned host memory on the
        engine's stream; returns ``(host, event)``. Once ``event`` has completed, the
        spectrum is ``host.numpy() * monitor.measure * monitor.weight``."""
        index = self.monitors.index(monitor)
        _, _, weights = self.monitor_tensors[index]
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(stream):  # zero fill, reduction and read-back in stream order
            out = torch.zeros(monitor.num_frequencies, dtype=torch.float64, device=self.device)
            _lib.check(self.lib, self.lib.mgb_flux_spectrum(self.handle, index, weights.data_ptr(),
                                                            out.data_ptr(), stream.cuda_stream))
            host = torch.empty(monitor.num_frequencies, dtype=torch.float64, pin_memory=True)
            host.copy_(out, non_blocking=True)
            event = torch.cuda.Event()
            event.record(stream)
        return host, event

    def flux_spectrum(self, monitor: FluxMonitor) -> np.ndarray:
        host, event = self.queue_flux_spectrum(monitor)
        event.synchronize()
        return host.numpy() * monitor.measure * monitor.weight

    def close(self) -> None:
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.mgb_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass


class ComplexEngine:
    """Complex fields at k = 0 (the reference's default ``force_complex_fields=True``).

    With every coefficient real and no Bloch phase, the real and imaginary parts step
    independently (the reference's complex run's real part is, word for word, the real
    run's): two real engines over the same coefficient tables, the real one driven by
    real(A) and the imaginary one by imag(A) (``sources.py:1357``: ``f[c][0] -= real(A);
    f[c][1] -= imag(A)``). A monitor's complex transform is the sum of the two parts'
    transforms, ``acc = acc_re + i * acc_im``, formed when it is read.
    """

    def __init__(self, grid: Grid, pml: Optional[PML], inv_eps, poles, sources, monitors, device=None,
                 stream=None, launch_shape=None, autotune: bool = True, kernels=None,
                 dft_accumulation: Optional[str] = None, conductivity=None):
        self.bloch = grid.has_bloch
        self.re = Engine(grid, pml, inv_eps, poles, sources, monitors, device=device, stream=stream,
                         launch_shape=launch_shape, autotune=autotune, kernels=kernels,
                         dft_accumulation=dft_accumulation, conductivity=conductivity, part="real",
                         create=False)
        self.im = Engine(grid, pml, inv_eps, poles, sources, monitors, device=device, stream=stream,
                         launch_shape=launch_shape, autotune=False, kernels=kernels,
                         dft_accumulation=dft_accumulation, conductivity=conductivity, part="imag",
                         own_monitors=False, create=False)
        if self.bloch:
            # the two parts meet across the phased faces: each plan reads the other's E, H
            axes = 0
            for a in range(3):
                phase = grid.bloch_phase(a)
                if phase is None:
                    continue
                axes |= 1 << a
                for engine in (self.re, self.im):
                    engine.desc.bloch_phase[a][0] = phase.real
                    engine.desc.bloch_phase[a][1] = phase.imag
            for engine, partner, part in ((self.re, self.im, 0), (self.im, self.re, 1)):
                engine.desc.bloch_axes = axes
                engine.desc.part = part
                for q, axis in enumerate("xyz"):
                    engine.desc.partner_E[q] = partner.fields["E" + axis].data_ptr()
                    engine.desc.partner_H[q] = partner.fields["H" + axis].data_ptr()
        self.re.finish()
        im_choice = kernels
        if self.re.choice is not None:
            im_choice = (self.re.choice[0], self.re.choice[1], self.re.wave, self.re.split)
        self.im._finish_args = (self.im._finish_args[0], im_choice, launch_shape, False)
        self.im.finish()
        self.grid = grid
        self.device = self.re.device
        self.monitors = self.re.monitors
        self.lib = self.re.lib
        self.dft_accumulation = self.re.dft_accumulation
        for monitor in self.monitors:
            monitor._engine = self

    # --- the Engine calls the driver and the monitors make ---------------------------------
    @property
    def choice(self):
        return self.re.choice

    @property
    def uses_tiles(self) -> bool:
        return self.re.uses_tiles

    def select(self, choice) -> None:
        self.re.select(choice)
        self.im.select(choice)

    def ensure_source_words(self, first_step: int, steps: int) -> None:
        self.re.ensure_source_words(first_step, steps)
        self.im.ensure_source_words(first_step, steps)

    def step(self, first_step: int, nsteps: int) -> None:
        if not self.bloch:
            self.re.step(first_step, nsteps)
            self.im.step(first_step, nsteps)
            return
        # the parts read each other across the phased faces: step them half by half
        done = 0
        while done < nsteps:
            chunk = min(nsteps - done, SOURCE_WINDOW)
            self.ensure_source_words(first_step + done, chunk)
            _lib.check(self.lib, self.lib.mgb_step_pair(self.re.handle, self.im.handle, first_step + done,
                                                        chunk, self.re._stream_handle()))
            done += chunk

    def launch(self, step: int, part: int, stream=None) -> None:
        self.re.launch(step, part, stream)
        self.im.launch(step, part, stream)

    def flush_dft(self) -> None:
        self.re.flush_dft()
        self.im.flush_dft()

    def read_accumulator(self, monitor, q: int) -> np.ndarray:
        # acc_re + i acc_im as the complex64 sum rounds it: (re.re - im.im) + i (re.im + im.re)
        return self.re.device_accumulator(monitor, q, imag=self.im).cpu().numpy()

    def write_accumulator(self, monitor, q: int, values: Optional[np.ndarray]) -> None:
        self.re.write_accumulator(monitor, q, values)
        self.im.write_accumulator(monitor, q, None)

    def _device_flux(self, monitor: FluxMonitor) -> torch.Tensor:
        """``sum w * Re(Ea conj(Hb) - Eb conj(Ha)) * dA`` of the complex transforms, summed
        in float64 on the device (the current stream)."""
        index = self.monitors.index(monitor)
        parts = []
        for engine in (self.re, self.im):
            acc = engine.monitor_tensors[index][1].to(torch.float64)  # [4][nf][2][cells]
            parts.append(torch.complex(acc[:, :, 0, :], acc[:, :, 1, :]))
        total = parts[0] + 1j * parts[1]
        ea, eb, ha, hb = total[0], total[1], total[2], total[3]
        weights = self.re.monitor_tensors[index][2].to(torch.float64)
        return torch.real(ea * torch.conj(hb) - eb * torch.conj(ha)) @ weights

    def flux_spectrum(self, monitor: FluxMonitor) -> np.ndarray:
        self.flush_dft()
        return self._device_flux(monitor).cpu().numpy() * monitor.measure * monitor.weight

    def queue_flux_spectrum(self, monitor: FluxMonitor):
        """The complex flux reduction and its read-back into pinned host memory, queued on
        the engines' stream; returns ``(host, event)`` as ``Engine.queue_flux_spectrum``."""
        stream = self.re.stream if self.re.stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(stream):
            for engine in (self.re, self.im):
                _lib.check(self.lib, self.lib.mgb_dft_flush(engine.handle, stream.cuda_stream))
            flux = self._device_flux(monitor)
            host = torch.empty(monitor.num_frequencies, dtype=torch.float64, pin_memory=True)
            host.copy_(flux, non_blocking=True)
            event = torch.cuda.Event()
            event.record(stream)
        return host, event

    def field(self, name: str) -> torch.Tensor:
        return torch.complex(self.re.field(name), self.im.field(name))

    def device_status(self) -> int:
        return self.re.device_status() | self.im.device_status()

    def nonfinite(self) -> bool:
        return self.re.nonfinite() or self.im.nonfinite()

    def field_energy(self) -> float:
        """|E|^2 eps + |B|^2 over both parts: re^2 + im^2 of every word."""
        out = self.re.energy_word()
        self.re.queue_field_energy(out)
        self.im.queue_field_energy(out)
        return float(out.item())

    def algorithmic_bytes(self) -> Dict[str, int]:
        a, b = self.re.algorithmic_bytes(), self.im.algorithmic_bytes()
        return {k: a[k] + b[k] for k in a}

    def close(self) -> None:
        self.re.close()
        self.im.close()
