"""Simulation knobs and the (delta, Delta, b) storage grid.

Mirrors ``madi/config.py`` of the reference (SimConfig at madi/config.py:179-369,
grid helpers at :149-172, constants at :36-113) field for field, so that a
caller of the reference can pass the same configuration here.  Two additions
are made for the GB300 walker and both default to the reference behaviour:

* ``boundary_mode="periodic"``: a periodic cubic box of ``n_cells`` Voronoi
  seeds (the reference only accepts ``"si_fatal_escape"``, madi/config.py:330).
* ``directions``: an optional (D, 3) list of unit gradient directions.  ``None``
  means the reference's harvest of the three Cartesian axes of every walk
  (madi/walker_gpu.py:148-151, :673-679).

Units: um, ms.  b in s/mm^2.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

D0_UM2_MS = 3.0
D0_MOUSE = 2.0
GAMMA_RAD = 2.675222e8

# Legacy fixed-delta constants, used only to describe pre-v2 library files.
DELTA_SMALL = 20.0
DELTAS_BIG = [50.0]
BVALS_S_MM2 = np.array([0, *([500] * 24), *([1000] * 24), *([1500] * 24),
                        *([2000] * 24), *([2500] * 24)])
BVALS_UNIQUE = np.array([500, 1000, 1500, 2000, 2500])
BVALS_UNIQUE_INT = BVALS_UNIQUE / 1e6

H_MS = 1.0
SMALL_DELTAS_MS: List[float] = list(range(1, 31))
BIG_DELTAS_MS: List[float] = list(range(1, 51)) + list(range(55, 81, 5))
T_MAX_MS = 128.0

PRODUCTION_WALKERS_PER_ENSEMBLE = 50_000
PRODUCTION_ENSEMBLES_PER_ENTRY = 40
PRODUCTION_AXIS_WALKS_PER_ENTRY = 3 * PRODUCTION_WALKERS_PER_ENSEMBLE * PRODUCTION_ENSEMBLES_PER_ENTRY
PRODUCTION_CLASSIFIER_MODE = "exact_cached"
PRODUCTION_CLASSIFIER_CACHE_DELTA_MAX_UM = 2.0
PRODUCTION_CLASSIFIER_CACHE_MIN_SAFE_RADIUS_UM = 0.0
PRODUCTION_CLASSIFIER_CACHE_CANDIDATE_CAPACITY = 256

B_MAX_S_MM2 = 12000.0
B_STEP_S_MM2 = 500.0

ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS: tuple = (
    (5.0, 15.0), (7.0, 25.0), (10.0, 30.0), (12.0, 36.0),
    (15.0, 40.0), (20.0, 50.0), (25.0, 60.0), (30.0, 80.0),
)
ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2 = np.arange(int(B_MAX_S_MM2 / B_STEP_S_MM2) + 1,
                                                dtype=float) * B_STEP_S_MM2

BOUNDARY_MODES = ("si_fatal_escape", "periodic")


def sqrt_spaced_bvalues(b_max: float = B_MAX_S_MM2, n: int = 28) -> np.ndarray:
    """b values evenly spaced in sqrt(b), b=0 included (madi/config.py:116)."""
    return np.linspace(0.0, np.sqrt(b_max), n) ** 2


def evenly_spaced_bvalues(step: float = B_STEP_S_MM2, b_max: float = B_MAX_S_MM2) -> np.ndarray:
    """b values 0, step, ..., b_max (madi/config.py:135)."""
    count = int(round(b_max / step)) + 1
    return step * np.arange(count, dtype=float)


def valid_delta_pairs(small_deltas=None, big_deltas=None) -> List[Tuple[float, float]]:
    """Triangular PGSE grid: every (delta, Delta) with Delta >= delta (madi/config.py:149)."""
    smalls = SMALL_DELTAS_MS if small_deltas is None else small_deltas
    bigs = BIG_DELTAS_MS if big_deltas is None else big_deltas
    out = []
    for d in smalls:
        for D in bigs:
            if D >= d:
                out.append((float(d), float(D)))
    return out


def grid_time_index(t_ms: float, h_ms: float = H_MS, tol: float = 1e-6) -> int:
    """Index of ``t_ms`` on the Y(t) grid; raises ValueError off-grid (madi/config.py:156)."""
    q = t_ms / h_ms
    k = round(q)
    if abs(q - k) > tol:
        raise ValueError(
            f"t={t_ms} ms is not an exact integer multiple of h={h_ms} ms "
            "(grid misalignment: Y would have to be interpolated, which is forbidden).")
    return int(k)


def fibonacci_directions(n: int) -> np.ndarray:
    """``n`` unit vectors on a golden-angle (Fibonacci) spiral, z from +1 to -1.

    u_i has z_i = 1 - (2 i + 1)/n and azimuth i * pi * (3 - sqrt 5); the set is
    deterministic and nearly uniform on the sphere.
    """
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * np.pi * (3.0 - np.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


@dataclass
class SimConfig:
    """Walk, geometry, classifier and storage-grid knobs (madi/config.py:179)."""

    D0: float = D0_UM2_MS
    ts: float = 1e-3
    T_max_ms: float = T_MAX_MS
    n_walkers: int = PRODUCTION_WALKERS_PER_ENSEMBLE
    n_ensembles: int = 4
    walker_chunk: Optional[int] = None

    classifier_mode: str = "exact"
    classifier_cache_delta_max_um: float = 1.0
    classifier_cache_min_safe_radius_um: float = 0.0
    classifier_cache_candidate_capacity: int = 256

    L: Optional[float] = None
    source_fraction: float = 0.40
    kappa: float = 0.90
    population_initial_margin_cell_spacings: float = 3.0
    population_certification_spacing_um: float = 8.0
    population_max_expansions: int = 8
    geometry_reference_path: Optional[str] = None
    allow_uncertified_geometry_reference: bool = False
    geometry_reference_required_cells: int = 5_000_000
    geometry_reference_required_alpha_values: int = 26
    geometry_validation_points: int = 200_000
    geometry_vi_tolerance: float = 0.005
    boundary_mode: str = "si_fatal_escape"

    phase_model: str = "finite_lobe"

    h_ms: float = H_MS
    small_deltas: list = field(default_factory=lambda: list(SMALL_DELTAS_MS))
    big_deltas: list = field(default_factory=lambda: list(BIG_DELTAS_MS))
    b_values: list = field(default_factory=lambda: list(evenly_spaced_bvalues()))

    # --- GB300 additions (no reference counterpart) ---------------------------
    # Seeds in one periodic box (boundary_mode="periodic" only).
    n_cells: int = 64
    # Optional (D, 3) gradient directions; None = the reference's x/y/z axes.
    directions: Optional[list] = None

    @property
    def sigma(self) -> float:
        return float(np.sqrt(2.0 * self.D0 * self.ts))

    @property
    def ls_rms(self) -> float:
        return float(np.sqrt(6.0 * self.D0 * self.ts))

    @property
    def n_steps(self) -> int:
        return int(round(self.T_max_ms / self.ts))

    @property
    def tRW_max(self) -> float:
        return self.n_steps * self.ts

    @property
    def steps_per_h(self) -> int:
        q = self.h_ms / self.ts
        k = round(q)
        if abs(q - k) > 1e-6:
            raise ValueError(
                f"h_ms={self.h_ms} is not an exact integer multiple of ts={self.ts}: "
                "Y(t) samples would drift off the step grid.")
        return int(k)

    @property
    def n_grid(self) -> int:
        return int(round(self.T_max_ms / self.h_ms)) + 1

    @staticmethod
    def tD(delta: float, Delta: float) -> float:
        return Delta - delta / 3.0

    def delta_pairs(self) -> List[Tuple[float, float]]:
        return valid_delta_pairs(self.small_deltas, self.big_deltas)

    def direction_array(self) -> np.ndarray:
        """(D, 3) float64 gradient directions; identity rows when unset."""
        if self.directions is None:
            return np.eye(3, dtype=np.float64)
        u = np.asarray(self.directions, dtype=np.float64)
        if u.ndim != 2 or u.shape[1] != 3 or len(u) == 0:
            raise ValueError("directions must have shape (D, 3)")
        norms = np.linalg.norm(u, axis=1)
        if np.any(np.abs(norms - 1.0) > 1e-9):
            raise ValueError("directions must be unit vectors")
        return u

    def assert_grid_alignment(self) -> None:
        """Loud validation of grid, physics and geometry knobs (madi/config.py:307-359)."""
        for d in self.small_deltas:
            grid_time_index(d, self.h_ms)
        for D in self.big_deltas:
            grid_time_index(D, self.h_ms)
        longest = 0.0
        for d, D in self.delta_pairs():
            grid_time_index(D + d, self.h_ms)
            longest = max(longest, D + d)
        if longest > self.T_max_ms:
            raise ValueError(
                f"(δ,Δ) grid needs Δ+δ up to {longest} ms but T_max_ms={self.T_max_ms} ms.")
        self.steps_per_h
        if self.phase_model not in ("finite_lobe", "narrow_pulse"):
            raise ValueError(f"phase_model must be 'finite_lobe' or 'narrow_pulse', got {self.phase_model!r}.")
        if self.boundary_mode not in BOUNDARY_MODES:
            raise ValueError(
                "boundary_mode must be 'si_fatal_escape' or 'periodic', got "
                f"{self.boundary_mode!r}.")
        if self.boundary_mode == "periodic" and int(self.n_cells) < 2:
            raise ValueError("a periodic box needs at least two cells")
        if not (0.0 < self.source_fraction <= 1.0):
            raise ValueError("source_fraction must lie in (0, 1].")
        if abs(self.kappa - 0.90) > 1e-12:
            raise ValueError("kappa must be the SI-specified 0.90.")
        if self.population_initial_margin_cell_spacings <= 0.0:
            raise ValueError("population_initial_margin_cell_spacings must be positive.")
        if self.population_certification_spacing_um <= 0.0:
            raise ValueError("population_certification_spacing_um must be positive.")
        if self.population_max_expansions < 1:
            raise ValueError("population_max_expansions must be positive.")
        if self.geometry_validation_points <= 0:
            raise ValueError("geometry_validation_points must be positive.")
        if self.geometry_reference_required_cells < 1:
            raise ValueError("geometry_reference_required_cells must be positive.")
        if self.geometry_reference_required_alpha_values < 1:
            raise ValueError("geometry_reference_required_alpha_values must be positive.")
        if self.classifier_mode not in ("exact", "exact_cached"):
            raise ValueError("classifier_mode must be 'exact' or 'exact_cached'.")
        if self.classifier_cache_delta_max_um <= 0.0:
            raise ValueError("classifier_cache_delta_max_um must be positive.")
        if self.classifier_cache_min_safe_radius_um < 0.0:
            raise ValueError("classifier_cache_min_safe_radius_um must be non-negative.")
        if self.classifier_cache_candidate_capacity < 2:
            raise ValueError("classifier_cache_candidate_capacity must be at least two.")
        self.direction_array()

    @property
    def grid_size(self) -> int:
        """Removed in the reference (madi/config.py:361-369); kept raising."""
        raise RuntimeError("the SI-exact classifier has no voxel cache grid")
