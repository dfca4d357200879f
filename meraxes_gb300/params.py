"""Run parameters of the reionization grid step and the named workloads.

`MxParams` mirrors `mx_params` in include/mx_reion.h field for field; the field
names map onto the reference's parameter names (src/meraxes.h run_params_t /
physics_params_t / run_units_t; defaults from input/params/defaults.par and the
Genesis simulation file input/params/simulations/Genesis_L210_N4320.par).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Dict, List, Optional

ABI_VERSION = 1

_FIELDS = [
    ("grid_dim", ctypes.c_int32),
    ("abi_version", ctypes.c_int32),
    ("box_size", ctypes.c_double),
    ("hubble_h", ctypes.c_double),
    ("omega_m", ctypes.c_double),
    ("omega_lambda", ctypes.c_double),
    ("omega_r", ctypes.c_double),
    ("omega_k", ctypes.c_double),
    ("baryon_frac", ctypes.c_double),
    ("w_lambda", ctypes.c_double),
    ("unit_length_cm", ctypes.c_double),
    ("unit_mass_g", ctypes.c_double),
    ("unit_velocity_cm_s", ctypes.c_double),
    ("flag_recombinations", ctypes.c_int32),
    ("flag_spin_temp", ctypes.c_int32),
    ("flag_21cm", ctypes.c_int32),
    ("flag_pecvel", ctypes.c_int32),
    ("uvb_flag", ctypes.c_int32),
    ("filter_type", ctypes.c_int32),
    ("rtom_filter_type", ctypes.c_int32),
    ("ts_heating_filter_type", ctypes.c_int32),
    ("ts_num_filter_steps", ctypes.c_int32),
    ("trees_id", ctypes.c_int32),
    ("delta_r_factor", ctypes.c_double),
    ("r_bubble_min", ctypes.c_double),
    ("r_bubble_max", ctypes.c_double),
    ("r_bubble_max_recomb", ctypes.c_double),
    ("reion_efficiency", ctypes.c_double),
    ("nion_phot_per_bary", ctypes.c_double),
    ("gamma_halo_bias", ctypes.c_double),
    ("alpha_uv", ctypes.c_double),
    ("y_he", ctypes.c_double),
    ("max_heating_redshift", ctypes.c_double),
    ("lx_gal", ctypes.c_double),
    ("nu_xray_gal_threshold", ctypes.c_double),
    ("spec_index_xray_gal", ctypes.c_double),
    ("nu_xray_soft_cut", ctypes.c_double),
    ("nu_xray_max", ctypes.c_double),
    ("reion_sfr_timescale", ctypes.c_double),
    ("clumping_factor", ctypes.c_double),
]


class MxParams(ctypes.Structure):
    """ctypes image of `mx_params` (include/mx_reion.h)."""

    _fields_ = _FIELDS


class MxGlobals(ctypes.Structure):
    """ctypes image of `mx_globals` (include/mx_reion.h)."""

    _fields_ = [
        ("volume_weighted_global_xH", ctypes.c_double),
        ("volume_weighted_global_J_21", ctypes.c_double),
        ("mass_weighted_global_xH", ctypes.c_double),
        ("volume_ave_J_alpha", ctypes.c_double),
        ("volume_ave_xalpha", ctypes.c_double),
        ("volume_ave_Xheat", ctypes.c_double),
        ("volume_ave_Xion", ctypes.c_double),
        ("volume_ave_TS", ctypes.c_double),
        ("volume_ave_TK", ctypes.c_double),
        ("volume_ave_xe", ctypes.c_double),
        ("volume_ave_Tb", ctypes.c_double),
        ("x_e_ave", ctypes.c_double),
        ("collapse_fraction", ctypes.c_double),
        ("n_radii", ctypes.c_int32),
        ("gpu_launches", ctypes.c_int32),
    ]

    def as_dict(self) -> Dict[str, float]:
        return {name: getattr(self, name) for name, _ in self._fields_}


GRID_NAMES = [
    "deltax",
    "stars",
    "weighted_sfr",
    "sfr",
    "sfr_histories",
    "N_rec",
    "x_e_box",
    "x_e_box_prev",
    "Tk_box",
    "TS_box",
    "xH",
    "z_at_ionization",
    "r_bubble",
    "J_21",
    "J_21_at_ionization",
    "Gamma12",
    "delta_T",
    "vel",
]

PADDED_GRIDS = {"deltax", "stars", "weighted_sfr", "sfr", "N_rec", "x_e_box", "x_e_box_prev", "vel"}


class MxGrids(ctypes.Structure):
    """ctypes image of `mx_grids` (include/mx_reion.h)."""

    _fields_ = [(n, ctypes.c_void_p) for n in GRID_NAMES]


GALAXY_FIELDS = ["pos", "type", "fesc_weighted_gsm", "gross_stellar_mass", "black_hole_mass", "effective_bhm"]


class MxGalaxies(ctypes.Structure):
    """ctypes image of `mx_galaxies` (include/mx_reion.h)."""

    _fields_ = [("n", ctypes.c_int64)] + [(n, ctypes.c_void_p) for n in GALAXY_FIELDS]


@dataclasses.dataclass
class ReionParams:
    """Hot-path parameters with the reference defaults (defaults.par)."""

    grid_dim: int = 64
    box_size: float = 50.0
    # cosmology: Genesis_L210_N4320.par:14-22
    hubble_h: float = 0.6751
    omega_m: float = 0.3121
    omega_lambda: float = 0.6879
    omega_r: float = 0.0
    omega_k: float = 0.0
    baryon_frac: float = 0.15714
    w_lambda: float = -1.0
    # units: Genesis_L210_N4320.par:27-29
    unit_length_cm: float = 3.08568e24
    unit_mass_g: float = 1.989e43
    unit_velocity_cm_s: float = 1e5
    flag_recombinations: int = 0
    flag_spin_temp: int = 0
    flag_21cm: int = 1
    flag_pecvel: int = 0
    uvb_flag: int = 1
    filter_type: int = 0
    rtom_filter_type: int = 0
    ts_heating_filter_type: int = 1
    ts_num_filter_steps: int = 40
    trees_id: int = 0
    delta_r_factor: float = 1.1
    r_bubble_min: float = 0.4068
    r_bubble_max: float = 20.34
    r_bubble_max_recomb: float = 33.9
    reion_efficiency: float = 1.0
    nion_phot_per_bary: float = 4000.0
    gamma_halo_bias: float = 2.0
    alpha_uv: float = 5.0
    y_he: float = 0.24
    max_heating_redshift: float = 30.0
    lx_gal: float = 3.16e40
    nu_xray_gal_threshold: float = 500.0
    spec_index_xray_gal: float = 1.0
    nu_xray_soft_cut: float = 2000.0
    nu_xray_max: float = 10000.0
    reion_sfr_timescale: float = 0.5
    # x_e sink clumping (XRayHeatingFunctions.h:30-32 hard-codes 2)
    clumping_factor: float = 2.0

    def to_ctypes(self) -> MxParams:
        p = MxParams()
        for name, _ in _FIELDS:
            if name == "abi_version":
                p.abi_version = ABI_VERSION
            else:
                setattr(p, name, getattr(self, name))
        return p

    @property
    def n_padded(self) -> int:
        D = self.grid_dim
        return D * D * 2 * (D // 2 + 1)

    @property
    def n_real(self) -> int:
        return self.grid_dim ** 3

    def filter_radii(self) -> List[float]:
        """Radius schedule of find_HII_bubbles.c:184-207, 445 (largest first)."""
        D, L = self.grid_dim, self.box_size
        clf = 0.620350491
        if L / D < 1.0:
            clf = 1.0
        rmax = self.r_bubble_max_recomb if self.flag_recombinations else self.r_bubble_max
        R = min(rmax, 0.620350491 * L)
        out = []
        while True:
            last = (R / self.delta_r_factor) <= (clf * L / D) or (R / self.delta_r_factor) <= self.r_bubble_min
            if last:
                R = clf * L / D
            out.append(R)
            if last:
                return out
            R /= self.delta_r_factor


@dataclasses.dataclass
class Workload:
    """A named workload: parameters, seed and snapshot redshift list."""

    name: str
    params: ReionParams
    seed: int
    redshifts: List[float]
    snapshots: List[int]
    fesc: float = 1.0

    @property
    def description(self) -> str:
        p = self.params
        return (f"{self.name}: {p.grid_dim}^3 L={p.box_size} Mpc/h seed={self.seed} "
                f"z={[round(self.redshifts[s], 3) for s in self.snapshots]}")


def workload(name: str, grid_dim: Optional[int] = None) -> Workload:
    """Named workloads of the measurement plan.

    plain_64   : find_HII_bubbles + delta_T at z=8, 64^3, L=50, seed 0, tophat,
                 R from 20 Mpc/h down by 1.1, ReionEfficiency=1, no
                 recombinations (the CPU-runnable case).
    full_256   : the full step at z=10, 256^3, L=100, seed 1: recombinations,
                 ComputeTs (40 shells, L_X=1e40, E0=500 eV) and delta_T; x_e sink
                 clumping factor 3.
    diff_256   : the full step's physics at z=12, 256^3, L=100, seed 3: the
                 power-spectrum-loss gradient case.
    evolve_512 : 20 snapshots z=15..6 at 512^3, L=200, seed 2, fields grown
                 linearly with the growth factor; recombinations (R_max 20),
                 ComputeTs and delta_T every snapshot.
    `grid_dim` rescales the box at fixed cell size (for small test cases).
    """
    if name == "plain_64":
        p = ReionParams(grid_dim=64, box_size=50.0, r_bubble_max=20.0, reion_efficiency=1.0,
                        flag_recombinations=0, flag_spin_temp=0, flag_21cm=1)
        w = Workload(name, p, 0, [8.5, 8.0], [1])
    elif name == "full_256":
        p = ReionParams(grid_dim=256, box_size=100.0, r_bubble_max=20.0, reion_efficiency=1.0,
                        flag_recombinations=1, flag_spin_temp=1, flag_21cm=1, lx_gal=1e40,
                        nu_xray_gal_threshold=500.0, clumping_factor=3.0)
        w = Workload(name, p, 1, [10.5, 10.0], [1])
    elif name == "diff_256":
        # the differentiation case: the full step's physics at z=12, seed 3; the
        # loss target is made at L_X = 2e40 (autograd.py)
        p = ReionParams(grid_dim=256, box_size=100.0, r_bubble_max=20.0, reion_efficiency=1.0,
                        flag_recombinations=1, flag_spin_temp=1, flag_21cm=1, lx_gal=1e40,
                        nu_xray_gal_threshold=500.0, clumping_factor=3.0)
        w = Workload(name, p, 3, [12.5, 12.0], [1])
    elif name == "evolve_512":
        p = ReionParams(grid_dim=512, box_size=200.0, r_bubble_max=20.0, r_bubble_max_recomb=20.0,
                        reion_efficiency=1.0, flag_recombinations=1, flag_spin_temp=1, flag_21cm=1)
        zs = [15.0 - 9.0 * i / 19.0 for i in range(20)]
        w = Workload(name, p, 2, zs, list(range(20)))
    else:
        raise KeyError(f"unknown workload {name!r}")
    if grid_dim is not None and grid_dim != w.params.grid_dim:
        cell = w.params.box_size / w.params.grid_dim
        w.params.grid_dim = int(grid_dim)
        w.params.box_size = cell * grid_dim
        w.name = f"{name}@{grid_dim}"
    return w


def sfr_timescale_internal_myr(myr: float, p: ReionParams) -> float:
    """Convert a time in Myr to internal time units (UnitLength/UnitVelocity)."""
    unit_time_s = p.unit_length_cm / p.unit_velocity_cm_s
    return myr * 3.155e13 / unit_time_s


def growth_factor(z: float, p: ReionParams) -> float:
    """dicke(z) for a flat Lambda universe (XRayHeatingFunctions.c:1469-1503)."""
    om, ol, orr = p.omega_m, p.omega_lambda, p.omega_r
    omz = om * (1 + z) ** 3 / (ol + om * (1 + z) ** 3 + orr * (1 + z) ** 4)
    dz = 2.5 * omz / (1.0 / 70.0 + omz * (209 - omz) / 140.0 + omz ** (4.0 / 7.0))
    d0 = 2.5 * om / (1.0 / 70.0 + om * (209 - om) / 140.0 + om ** (4.0 / 7.0))
    return dz / (d0 * (1.0 + z))


__all__ = ["MxParams", "MxGlobals", "MxGrids", "ReionParams", "Workload", "workload", "GRID_NAMES",
           "PADDED_GRIDS", "growth_factor", "sfr_timescale_internal_myr", "math"]
