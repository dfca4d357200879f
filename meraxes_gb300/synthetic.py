"""Seeded synthetic input grids for the reionization step.

No N-body or galaxy input is read: the density field and the stellar-mass and
SFR grids are generated from a seed, following the recipe of the measurement
plan:

* deltax: FP64 Gaussian white noise (numpy PCG64, `seed`), filtered in Fourier
  space by sqrt(P(k)), P(k) ~ k^-2 exp(-(k/k_Ny)^2), k_Ny = pi D / L, P(0) = 0;
  rescaled to sigma = 0.6 at the reference redshift, grown linearly with the
  growth factor to other redshifts, clipped at -0.99, stored as FP32 in the
  PADDED layout.
* stars = 1e7 Msun/h * exp(2 deltax) where deltax > 0.5, else 0 (internal mass
  unit 1e10 Msun/h); sfr = stars / 20 Myr; weighted_sfr = fesc * sfr and the
  ionising stars grid is fesc * stars.
* sfr_histories: slice j holds the sfr grid of snapshot (s - j) in the PADDED
  layout, as construct_baryon_grids writes it (src/core/reionization.c:1386-1390,
  1578-1587).
* spin-temperature state before the first computed snapshot: homogeneous
  x_e and T_K from the RECFAST table at the previous redshift (what the
  reference's homogeneous branch, ComputeTs.c:189-262, leaves behind).
"""
from __future__ import annotations

import os
from typing import Dict, Optional

import numpy as np

from .params import ReionParams, Workload, growth_factor, sfr_timescale_internal_myr

TABLES_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tables", "21cmFAST")


def padded_shape(D: int):
    return (D, D, 2 * (D // 2 + 1))


def to_padded(real: np.ndarray) -> np.ndarray:
    D = real.shape[0]
    out = np.zeros(padded_shape(D), dtype=np.float32)
    out[:, :, :D] = real
    return out


def from_padded(padded: np.ndarray, D: int) -> np.ndarray:
    return np.ascontiguousarray(padded.reshape(padded_shape(D))[:, :, :D])


def gaussian_field(D: int, L: float, seed: int, sigma: float = 0.6) -> np.ndarray:
    """Unit-variance-rescaled Gaussian random field (FP64, REAL layout)."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((D, D, D))
    fk = np.fft.rfftn(noise)
    kf = 2.0 * np.pi / L
    kx = np.fft.fftfreq(D, d=1.0 / D) * kf
    kz = np.fft.rfftfreq(D, d=1.0 / D) * kf
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    k_ny = np.pi * D / L
    with np.errstate(divide="ignore"):
        pk = np.where(k2 > 0, np.exp(-k2 / k_ny ** 2) / k2, 0.0)
    field = np.fft.irfftn(fk * np.sqrt(pk), s=(D, D, D), axes=(0, 1, 2))
    field *= sigma / field.std()
    return field


def recfast_table(tables_dir: str = TABLES_DIR):
    """(z, x_e, T_K) columns of recfast_LCDM.dat, float-rounded like the reader
    at XRayHeatingFunctions.c:125-131 (ascending z)."""
    data = np.loadtxt(os.path.join(tables_dir, "recfast_LCDM.dat"))
    data = data.astype(np.float32).astype(np.float64)[::-1]
    return data[:, 0], data[:, 1], data[:, 3]


def recfast_state(z: float, tables_dir: str = TABLES_DIR):
    """Homogeneous (x_e, T_K) at redshift z via a natural cubic spline."""
    from scipy.interpolate import CubicSpline

    zt, xe, tk = recfast_table(tables_dir)
    zf = float(np.float32(z))
    return float(CubicSpline(zt, xe, bc_type="natural")(zf)), float(CubicSpline(zt, tk, bc_type="natural")(zf))


class FieldGenerator:
    """Generates the input grids of a workload snapshot by snapshot."""

    def __init__(self, w: Workload, z_norm: Optional[float] = None):
        self.w = w
        p = w.params
        self.p = p
        self.base = gaussian_field(p.grid_dim, p.box_size, w.seed)
        self.z_norm = z_norm if z_norm is not None else w.redshifts[w.snapshots[-1]]
        self.d_norm = growth_factor(self.z_norm, p)
        self.t20 = sfr_timescale_internal_myr(20.0, p)

    def deltax_real(self, snapshot: int) -> np.ndarray:
        z = self.w.redshifts[snapshot]
        d = self.base * (growth_factor(z, self.p) / self.d_norm)
        return np.maximum(d, -0.99).astype(np.float32)

    def velocity_real(self, snapshot: int) -> np.ndarray:
        """Line-of-sight velocity grid in the trees' units: a Gaussian field
        (seed + 7919) smoothed over 3 cells, with 50 km/s rms peculiar
        velocity at the normalisation redshift, grown like the density (in
        the small test boxes |dv/dx| stays below half the Hubble rate, away
        from the caustics where the optical-depth form is ill-conditioned);
        divided by (1+z) for the VELOCIRAPTOR convention (the step multiplies
        it back), times 1000 sqrt(1+z) for GBPTREES."""
        if not hasattr(self, "_vbase"):
            D, L = self.p.grid_dim, self.p.box_size
            v = gaussian_field(D, L, self.w.seed + 7919, sigma=1.0)
            k = 2.0 * np.pi * np.fft.fftfreq(D, d=L / D)
            kz = 2.0 * np.pi * np.fft.rfftfreq(D, d=L / D)
            k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
            rs = 3.0 * L / D
            v = np.fft.irfftn(np.fft.rfftn(v) * np.exp(-0.5 * k2 * rs * rs), s=(D, D, D), axes=(0, 1, 2))
            self._vbase = v / v.std()
        z = self.w.redshifts[snapshot]
        v = 50.0 * self._vbase * (growth_factor(z, self.p) / self.d_norm)
        if self.p.trees_id == 1:
            v = v * 1000.0 * np.sqrt(1.0 + z)
        else:
            v = v / (1.0 + z)
        return v.astype(np.float32)

    def stars_sfr_real(self, snapshot: int):
        d = self.deltax_real(snapshot).astype(np.float64)
        stars = np.where(d > 0.5, 1e-3 * np.exp(2.0 * d), 0.0)
        sfr = stars / self.t20
        return stars.astype(np.float32), sfr.astype(np.float32)

    def inputs(self, snapshot: int, n_sfr_hist: int = 0) -> Dict[str, np.ndarray]:
        """Input grids for `snapshot` (PADDED arrays where the reference uses
        the padded layout).  The caller owns persistent state grids."""
        fesc = self.w.fesc
        delta = self.deltax_real(snapshot)
        stars, sfr = self.stars_sfr_real(snapshot)
        out = {
            "deltax": to_padded(delta),
            "stars": to_padded((fesc * stars.astype(np.float64)).astype(np.float32)),
            "weighted_sfr": to_padded((fesc * sfr.astype(np.float64)).astype(np.float32)),
            "sfr": to_padded(sfr),
        }
        if self.p.flag_pecvel > 0 and self.p.flag_spin_temp:
            out["vel"] = to_padded(self.velocity_real(snapshot))
        if n_sfr_hist > 0:
            D = self.p.grid_dim
            n_pad = int(np.prod(padded_shape(D)))
            hist = np.zeros((n_sfr_hist, n_pad), dtype=np.float32)
            for j in range(n_sfr_hist):
                s = snapshot - j
                if s < 0:
                    break
                hist[j] = to_padded(self.stars_sfr_real(s)[1]).ravel()
            out["sfr_histories"] = hist
        return out


def initial_state(p: ReionParams, z_prev: float, tables_dir: str = TABLES_DIR) -> Dict[str, np.ndarray]:
    """Persistent grids before the first computed snapshot."""
    D = p.grid_dim
    st = {
        "xH": np.ones((D, D, D), np.float32),
        "z_at_ionization": np.full((D, D, D), -1.0, np.float32),
        "r_bubble": np.zeros((D, D, D), np.float32),
        "J_21": np.zeros((D, D, D), np.float32),
        "J_21_at_ionization": np.zeros((D, D, D), np.float32),
        "Gamma12": np.zeros((D, D, D), np.float32),
        "N_rec": np.zeros(padded_shape(D), np.float32),
        "delta_T": np.zeros((D, D, D), np.float32),
        "TS_box": np.zeros((D, D, D), np.float32),
    }
    if p.flag_spin_temp:
        xe, tk = recfast_state(z_prev, tables_dir)
        prev = np.zeros(padded_shape(D), np.float32)
        prev[:, :, :D] = np.float32(xe)
        st["x_e_box_prev"] = prev
        st["x_e_box"] = prev.copy()
        st["Tk_box"] = np.full((D, D, D), np.float32(tk), np.float32)
    return st
