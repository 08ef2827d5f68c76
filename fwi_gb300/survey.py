"""Survey description shared by the device path and its checkers.

A survey is what one calculate_misfit_gradient call sees
(src/calculate_misfit_gradient.f90:73-360): a model of ny x nx_model cells,
one time axis (dt, nt, store_snap) and a list of shots, each with its own
window of model columns, sources, receivers and observed traces.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


@dataclass
class ShotSpec:
    x0: int                     # first model column of the window (0-based)
    nx: int                     # window width
    nxSou: np.ndarray           # window-relative 1-based grid indices
    nySou: np.ndarray
    nxRec: np.ndarray
    nyRec: np.ndarray
    src: Optional[np.ndarray]   # S(nt, num_sou) float32, Fortran order (None: zeros)
    obs: Optional[np.ndarray] = None   # Data_target(nt, num_rec)
    grad_weight: float = 1.0
    misfit_weight: float = 1.0


@dataclass
class SurveySpec:
    ny: int
    nx_model: int
    d: float
    dt: float
    nt: int
    shots: List[ShotSpec] = field(default_factory=list)
    store_snap: int = 10
    acc: int = 3
    dpml: int = 20
    numtasks: int = 1
    water_rows: Optional[np.ndarray] = None   # bat_model_grid(nx_model)

    @property
    def nt_store(self) -> int:
        return self.nt // self.store_snap

    def obs_packed(self) -> np.ndarray:
        return np.concatenate([np.asarray(s.obs, np.float32).reshape(-1, order="F") for s in self.shots])

    def step_bytes(self) -> float:
        """Algorithmic HBM bytes of one time step over all shots: 16 B per
        padded cell below the free surface (read p, p_1, c2; write p_3) and
        16 B per CPML direction-cell (read+write phi, chi)."""
        dn = self.dpml + 2 * self.acc
        b = 0.0
        for s in self.shots:
            cells = (self.ny + dn) * (s.nx + 2 * dn)
            cpml = 2 * self.ny * dn + dn * s.nx + 4 * dn * dn
            b += 16.0 * cells + 16.0 * cpml
        return b

    def gradient_bytes(self, snap_bytes: int = 4) -> float:
        """Algorithmic bytes of one shot-gradient pass over all shots:
        forward + adjoint steps plus snapshot write/read and the gradient
        read-modify-write every store_snap steps."""
        b = 2.0 * self.nt * self.step_bytes()
        for s in self.shots:
            b += self.nt_store * self.ny * s.nx * (2 * snap_bytes + 8)
        return b
