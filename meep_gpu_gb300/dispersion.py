"""Lorentz / Drude susceptibilities and MEEP's float32 recurrence constants.

Follows the reference's ``meep_gpu/dispersion.py``: ``Susceptibility`` (:184) with
MEEP-unit ``frequency`` and ``gamma`` (the 2*pi is MEEP's own), and
``realnum_constants`` (:243), each word rounded where MEEP 1.33.0 rounds it
(susceptibility.cpp:191-195)::

    omega2pi = f32(2*pi*f32(omega_0)),  g2pi = f32(f32(gamma*2)*pi)
    omega0dtsqr = ((omega2pi*omega2pi)*dt)*dt,  gamma1inv = 1/(1 + g2pi*dt/2)
    gamma1 = 1 - g2pi*dt/2,  two_minus_od = 2 - (Drude ? 0 : omega0dtsqr)

The isotropic update (``PolarizationState.update`` :689) that the E-kernel runs is
``P' = gamma1inv*(((P*A) - (gamma1*Pprev)) + (omega0dtsqr*(sigma*W)))`` with
``W = (D - sum P) * chi1inv``, the rounded float32 operations in that order.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import NamedTuple

import numpy as np

LORENTZ = "lorentzian"
DRUDE = "drude"


class RealnumConstants(NamedTuple):
    two_minus_od: np.float32
    gamma1: np.float32
    omega0dtsqr: np.float32
    gamma1inv: np.float32


class Float64Constants(NamedTuple):
    two_minus_od: float
    gamma1: float
    omega0dtsqr: float
    gamma1inv: float


@dataclass(frozen=True)
class Susceptibility:
    """One Lorentz (or Drude) pole: ``sigma * f0^2 / (f0^2 - f^2 - i f gamma)``."""

    frequency: float
    gamma: float = 0.0
    kind: str = LORENTZ

    def __post_init__(self):
        if self.kind not in (LORENTZ, DRUDE):
            raise ValueError(f"susceptibility kind must be 'lorentzian' or 'drude', got {self.kind!r}")
        if not math.isfinite(self.frequency) or self.frequency < 0:
            raise ValueError(f"susceptibility frequency must be finite and >= 0, got {self.frequency!r}")
        if not math.isfinite(self.gamma) or self.gamma < 0:
            raise ValueError(f"susceptibility gamma must be finite and >= 0, got {self.gamma!r}")

    @property
    def is_drude(self) -> bool:
        return self.kind == DRUDE

    def realnum_constants(self, dt: float) -> RealnumConstants:
        f32 = np.float32
        omega_0 = f32(self.frequency)
        gamma = f32(self.gamma)
        dt_r = f32(dt)
        omega2pi = f32((2.0 * math.pi) * float(omega_0))
        g2pi = f32(float(gamma * f32(2)) * math.pi)
        omega0dtsqr = ((omega2pi * omega2pi) * dt_r) * dt_r
        half_g2pi_dt = (g2pi * dt_r) / f32(2)
        gamma1inv = f32(1) / (f32(1) + half_g2pi_dt)
        gamma1 = f32(1) - half_g2pi_dt
        denom = f32(0) if self.is_drude else omega0dtsqr
        return RealnumConstants(f32(2) - denom, gamma1, omega0dtsqr, gamma1inv)

    def float64_constants(self, dt: float) -> Float64Constants:
        """The same recurrence formed in double, for the float64 restatement."""
        omega2pi = 2.0 * math.pi * self.frequency
        g2pi = 2.0 * math.pi * self.gamma
        omega0dtsqr = omega2pi * omega2pi * dt * dt
        gamma1inv = 1.0 / (1.0 + g2pi * dt / 2)
        gamma1 = 1.0 - g2pi * dt / 2
        denom = 0.0 if self.is_drude else omega0dtsqr
        return Float64Constants(2.0 - denom, gamma1, omega0dtsqr, gamma1inv)

    def stability_radius(self, dt: float) -> float:
        """Largest root modulus of the float64 recurrence's characteristic polynomial.

        ``g1inv * (z^2 * ... )``: the homogeneous part ``P' = g1inv*(A P - g1 Pp)`` has
        roots of ``z^2 - g1inv*A z + g1inv*g1``; above 1 the pole blows up on its own.
        """
        c = self.float64_constants(dt)
        roots = np.roots([1.0, -c.gamma1inv * c.two_minus_od, c.gamma1inv * c.gamma1])
        return float(np.max(np.abs(roots)))
