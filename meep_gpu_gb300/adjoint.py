"""Adjoint gradient of a flux objective with respect to the permittivity of a design box.

The objective is J = sum_f c_f * flux_f over one flux monitor's frequencies (c_f = 1 by
default), after ``steps`` steps of the configured simulation. The forward run keeps a
copy of the whole state every ``checkpoint_every`` steps. The backward run walks the
segments last to first: it restores the segment's checkpoint, recomputes the segment
forward (H and E halves only) saving D over the design box after every step, and then
steps the adjoint state back through the segment with the reverse-time kernels of
``libmeepgb.so`` (``mgb_adjoint_step``: the transpose of each half step, UPML recurrences
included), adding the adjoint of every monitor sample (``mgb_adjoint_inject``) where the
forward took one. The kernels accumulate dJ/d(inverse epsilon) over the box; the
permittivity gradient is -that / eps^2.

The reference has no adjoint (``meep_gpu`` exposes none; MEEP's ``meep.adjoint`` is a
separate package), so the gradient is checked against central finite differences of
the float64 oracle.
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .dft import FluxMonitor
from .grid import Unsupported


class FluxAdjoint:
    """dJ/d(eps) over ``box`` for the flux objective of ``monitor`` (a FluxMonitor of
    ``driver``); ``driver`` is configured but not yet stepped, isotropic, without poles."""

    def __init__(self, driver, monitor: FluxMonitor, box: Sequence[Tuple[int, int]], steps: int,
                 checkpoint_every: int = 200, frequency_weights: Optional[Sequence[float]] = None,
                 dft_accumulation: Optional[str] = None):
        if not isinstance(monitor, FluxMonitor) or monitor not in driver._flux_monitors:
            raise ValueError("the objective's monitor must be a flux monitor of the driver")
        if driver._poles:
            raise Unsupported("the adjoint step does not carry susceptibility poles")
        if driver.has_conductivity:
            raise Unsupported("the adjoint step does not carry a conductivity")
        if driver.complex_fields:
            raise Unsupported("the adjoint gradient takes real fields (force_complex_fields=False)")
        if driver.grid.has_symmetry:
            raise Unsupported("the adjoint step does not carry mirror symmetry")
        if driver.engine is not None:
            raise RuntimeError("the adjoint problem needs a driver that has not been stepped")
        if steps < 1 or checkpoint_every < 1:
            raise ValueError("steps and checkpoint_every must be positive")
        self.driver = driver
        self.monitor = monitor
        self.steps = int(steps)
        self.every = int(checkpoint_every)
        self.box = tuple((int(a), int(b)) for a, b in box)
        shape = driver.grid.shape
        for (a, b), n in zip(self.box, shape):
            if not 0 <= a < b <= n:
                raise ValueError(f"design box {self.box} is outside the grid {shape}")
        self.engine = driver.freeze(dft_accumulation=dft_accumulation)
        engine = self.engine
        if len({t.data_ptr() for t in engine.inv_eps}) != 1:
            raise Unsupported("the adjoint gradient takes an isotropic permittivity (set_epsilon)")
        self.device = engine.device
        self.stream = torch.cuda.current_stream(self.device)
        nf = monitor.num_frequencies
        weights = np.ones(nf) if frequency_weights is None else np.asarray(frequency_weights, dtype=np.float64)
        if weights.shape != (nf,):
            raise ValueError(f"frequency_weights needs {nf} values")
        self.frequency_weights = torch.from_numpy(weights).to(self.device)
        self.index = engine.monitors.index(monitor)
        # forward state saved at checkpoints: fields and PML auxiliaries
        self.state: List[torch.Tensor] = list(engine.fields.values()) + list(engine.aux.values())
        self.checkpoints: List[List[torch.Tensor]] = []
        self._make_adjoint_plan()
        (i0, i1), (j0, j1), (k0, k1) = self.box
        self.box_shape = (i1 - i0, j1 - j0, k1 - k0)
        self.box_cells = int(np.prod(self.box_shape))
        self.d_history = torch.empty((self.every, 3, self.box_cells), dtype=torch.float32, device=self.device)
        self.grad_inv = torch.zeros(self.box_cells, dtype=torch.float32, device=self.device)
        self._box_arg = (ctypes.c_int32 * 6)(i0, i1, j0, j1, k0, k1)
        self.eps_box: Optional[torch.Tensor] = None
        self.value: Optional[float] = None

    # --- plans --------------------------------------------------------------------------
    def _make_adjoint_plan(self) -> None:
        engine = self.engine
        zeros = lambda: torch.zeros(engine.grid.shape, dtype=torch.float32, device=self.device)  # noqa: E731
        self.lam = {name: zeros() for name in engine.fields}
        self.lam_aux = {name: zeros() for name in engine.aux}
        self.mu_b = [zeros() for _ in range(3)]
        self.mu_d = [zeros() for _ in range(3)]
        nf, cells = self.monitor.num_frequencies, self.monitor.cells
        self.coef = torch.zeros((4, nf, 2, cells), dtype=torch.float32, device=self.device)
        self.adj_status = torch.zeros(1, dtype=torch.int32, device=self.device)
        d = _lib.MgbSimDesc()
        ctypes.memmove(ctypes.byref(d), ctypes.byref(engine.desc), ctypes.sizeof(d))  # a copy
        for q, axis in enumerate("xyz"):
            d.E[q] = self.lam["E" + axis].data_ptr()
            d.D[q] = self.lam["D" + axis].data_ptr()
            d.H[q] = self.lam["H" + axis].data_ptr()
        for family in ("B", "fwH", "fwE", "fuB", "fuD"):
            slots = getattr(d, family)
            for q, axis in enumerate("xyz"):
                name = family + axis
                if name in self.lam_aux:
                    slots[q].data = self.lam_aux[name].data_ptr()
        d.npoles = 0
        d.nsrc = 0
        d.nsrc_magnetic = 0
        d.src_cell = None
        d.src_comp = None
        d.monitors[0] = engine.desc.monitors[self.index]
        d.monitors[0].acc = self.coef.data_ptr()
        d.nmonitors = 1
        d.status = self.adj_status.data_ptr()
        self.adj_desc = d
        handle = ctypes.c_void_p()
        _lib.check(engine.lib, engine.lib.mgb_create(ctypes.byref(d), ctypes.byref(handle)))
        self.adj_handle = handle
        self.adj = _lib.MgbAdjoint()
        for q in range(3):
            self.adj.mu_b[q] = self.mu_b[q].data_ptr()
            self.adj.mu_d[q] = self.mu_d[q].data_ptr()

    # --- forward --------------------------------------------------------------------------
    def _reset(self) -> None:
        engine = self.engine
        for t in self.state:
            t.zero_()
        for _omega, acc, _w in engine.monitor_tensors:
            acc.zero_()
        engine.status.zero_()

    def forward(self, eps_box: torch.Tensor) -> float:
        """J for the given box permittivity; keeps the checkpoints for :meth:`backward`."""
        engine = self.engine
        eps = eps_box.detach().to(self.device, torch.float64).reshape(self.box_shape)
        if torch.any(eps <= 0) or not torch.all(torch.isfinite(eps)):
            raise ValueError("design permittivity must be finite and positive")
        (i0, i1), (j0, j1), (k0, k1) = self.box
        engine.inv_eps[0][i0:i1, j0:j1, k0:k1] = (1.0 / eps).to(torch.float32)
        self.eps_box = eps
        self._reset()
        self.checkpoints = []
        n = 0
        while n < self.steps:
            self.checkpoints.append([t.clone() for t in self.state])
            chunk = min(self.every, self.steps - n)
            engine.step(n, chunk)
            n += chunk
        spectrum = self.monitor.get_flux_spectrum()
        if engine.nonfinite():
            raise RuntimeError("the forward run wrote a non-finite field")
        self.spectrum = spectrum
        self.value = float(np.dot(self.frequency_weights.cpu().numpy(), spectrum))
        return self.value

    # --- backward -------------------------------------------------------------------------
    def _coefficients(self) -> None:
        """dJ/d(accumulator words), in the accumulator layout: Ea pairs with Hb, Eb with Ha."""
        engine = self.engine
        _omega, acc, weights = engine.monitor_tensors[self.index]
        scale = self.monitor.measure * self.monitor.weight
        cw = self.frequency_weights.to(torch.float32)[:, None, None] * float(scale) * weights[None, None, :]
        ea, eb, ha, hb = acc[0], acc[1], acc[2], acc[3]
        self.coef[0] = cw * hb
        self.coef[1] = -cw * ha
        self.coef[2] = -cw * eb
        self.coef[3] = cw * ea

    def backward(self) -> torch.Tensor:
        """dJ/d(eps) over the box (float64, box-shaped), for the last :meth:`forward`."""
        if self.value is None:
            raise RuntimeError("backward() needs a forward() first")
        engine, lib = self.engine, self.engine.lib
        stream = self.stream
        handle = stream.cuda_stream
        self._coefficients()
        for t in list(self.lam.values()) + list(self.lam_aux.values()) + self.mu_b + self.mu_d:
            t.zero_()
        self.grad_inv.zero_()
        self.adj.grad_inv = self.grad_inv.data_ptr()
        self.adj.box[:] = list(self._box_arg)
        self.adj.d_after = self.d_history.data_ptr()
        for seg in range(len(self.checkpoints) - 1, -1, -1):
            n0 = seg * self.every
            n1 = min(self.steps, n0 + self.every)
            for t, saved in zip(self.state, self.checkpoints[seg]):
                t.copy_(saved)
            engine.ensure_source_words(n0, n1 - n0)
            # recompute the segment and step the adjoint back through it (one library call)
            _lib.check(lib, lib.mgb_adjoint_segment(engine.handle, self.adj_handle, ctypes.byref(self.adj),
                                                    n0, n1 - n0, 0, self.d_history.data_ptr(), handle))
        grad_inv = self.grad_inv.to(torch.float64).reshape(self.box_shape)
        return -grad_inv / (self.eps_box * self.eps_box)

    def objective(self, eps_box: torch.Tensor) -> torch.Tensor:
        """J as a differentiable function of the box permittivity (torch.autograd)."""
        return _FluxObjective.apply(eps_box, self)

    def close(self) -> None:
        if getattr(self, "adj_handle", None) is not None and self.adj_handle.value:
            self.engine.lib.mgb_destroy(self.adj_handle)
            self.adj_handle = None
        self.checkpoints = []

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass


class _FluxObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps_box: torch.Tensor, problem: FluxAdjoint) -> torch.Tensor:  # noqa: D401
        value = problem.forward(eps_box)
        ctx.problem = problem
        ctx.shape = eps_box.shape
        ctx.dtype = eps_box.dtype
        return torch.tensor(value, dtype=torch.float64, device=eps_box.device)

    @staticmethod
    def backward(ctx, grad_output: torch.Tensor):
        grad = ctx.problem.backward().reshape(ctx.shape).to(grad_output.device)
        return (grad_output.to(torch.float64) * grad).to(ctx.dtype), None
