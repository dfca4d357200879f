"""Parity checks between two runs of the grid step (test helpers).

Tolerances, from the acceptance rule of the step:
  * global volume / mass weighted xHI within 1e-5 relative, plus the share
    of the cells whose flags may disagree (below): each such cell moves the
    mean by its own xH difference times its weight;
  * ionisation flags may disagree in at most 1e-4 of the cells, and only in
    cells whose threshold margin |f_coll*eff/(nf(1+rec)) - 1| (from the oracle)
    is below 1e-5, except that at most 1e-7 of the cells (at least one) may
    lie between 1e-5 and 1e-4.  That allowance is the reference's own platform
    spread: its float top-hat weight 3(sinf x/x^3 - cosf x/x^2) cancels at the
    lowest modes of the smallest radius and amplifies a last-bit difference
    of sinf, cosf or powf by 3/x^2; the oracle with correctly rounded sin and
    cos in that expression (everything else unchanged, FP64 transforms)
    flips one cell of the 512^3 benchmark snapshot at margin 1.4e-5 against
    the oracle built on the host libm;
  * r_bubble, the smallest radius at which a cell passes the test, likewise,
    with the smallest margin over all radii (a flip at any radius moves it,
    also in cells whose flags agree);
  * T_S, T_K, delta_T and the other grids within 1e-4 relative per cell, with
    an absolute floor of 10 * 2^-24 * log2(N) * max|x| that bounds the rounding
    error of an FP32 FFT of N points (the reference's FFTW single-precision
    path carries an error of the same size); values that depend on the radius
    of first crossing (J_21, Gamma12, N_rec) are compared where that radius
    agrees: where the first-crossing margin is at least 1e-5.  N_rec, which
    is updated from Gamma12 through the recombination rate table, also passes
    on Gamma12's relative difference at the cell.

The report gives, per grid, the largest relative difference, the cells
outside tolerance and, as `<grid>_floor_only`, the cells that are inside it
only through the absolute FFT floor (outside the relative rule alone).
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

REL_TOL = 1e-5          # REL_TOL of the reference: ionised means xH < 1e-5
FLAG_FRACTION = 1e-4
MARGIN = 1e-5
LIBM_MARGIN = 1e-4
LIBM_FRACTION = 1e-7
GRID_RTOL = 1e-4
XH_ATOL = 1e-4


def fft_floor(n: int) -> float:
    return 10.0 * 2.0 ** -24 * np.log2(n)


def _real(a: np.ndarray, D: int) -> np.ndarray:
    if a.size == D ** 3:
        return a.reshape(-1)
    return np.ascontiguousarray(a.reshape(D, D, -1)[:, :, :D]).reshape(-1)


def compare(ref: Dict[str, np.ndarray], test: Dict[str, np.ndarray], ref_globals: Dict[str, float],
            test_globals: Dict[str, float], margin: Optional[np.ndarray] = None, report: Optional[dict] = None):
    """Raises AssertionError with a readable message on a parity violation."""
    rep = report if report is not None else {}
    D = ref["xH"].shape[0]
    n = D ** 3
    floor = fft_floor(n)
    fa = ref["xH"].reshape(-1) < REL_TOL
    fb = test["xH"].reshape(-1) < REL_TOL
    dis = fa != fb
    rb_dis = ref["r_bubble"].reshape(-1) != test["r_bubble"].reshape(-1)
    rep["flag_disagree"] = int(dis.sum())
    rep["rbubble_disagree"] = int(rb_dis.sum())
    assert dis.sum() <= FLAG_FRACTION * n, f"flags differ in {dis.sum()} of {n} cells"
    if margin is not None:
        m_first, m_all = margin[0].reshape(-1), margin[1].reshape(-1)
        edges = (1e-6, 1e-5, 1e-4)
        for name, sel_, m in (("flag", dis, m_first), ("rbubble", rb_dis, m_all)):
            mm = m[sel_]
            rep[name + "_margin_buckets"] = [int((mm < edges[0]).sum())] + \
                [int(((mm >= lo) & (mm < hi)).sum()) for lo, hi in zip(edges[:-1], edges[1:])] + \
                [int((mm >= edges[-1]).sum())]
        libm_cells = max(1, int(LIBM_FRACTION * n))
        if dis.any():
            rep["flag_margin_max"] = float(m_first[dis].max())
            rep["flag_disagree_above_1e-5"] = int((m_first[dis] >= MARGIN).sum())
            assert np.all(m_first[dis] < LIBM_MARGIN) and rep["flag_disagree_above_1e-5"] <= libm_cells, \
                f"flag disagreement at margin {m_first[dis].max():.3e} ({rep})"
        if rb_dis.any():
            rep["rbubble_margin_max"] = float(m_all[rb_dis].max())
            rep["rbubble_disagree_above_1e-5"] = int((m_all[rb_dis] >= MARGIN).sum())
            assert rb_dis.sum() <= FLAG_FRACTION * n, f"r_bubble differs in {rb_dis.sum()} of {n} cells"
            assert np.all(m_all[rb_dis] < LIBM_MARGIN) and rep["rbubble_disagree_above_1e-5"] <= libm_cells, \
                f"r_bubble disagreement at margin {m_all[rb_dis].max():.3e} ({rep})"
        near_first = m_first < MARGIN
    else:
        assert rb_dis.sum() <= FLAG_FRACTION * n, f"r_bubble differs in {rb_dis.sum()} of {n} cells"
        near_first = np.zeros(n, bool)
    dxh = np.abs(ref["xH"].reshape(-1).astype(np.float64) - test["xH"].reshape(-1).astype(np.float64))
    flip = {"volume_weighted_global_xH": float(dxh[dis].sum()) / n}
    if "deltax" in ref and ref["deltax"] is not None:
        wm = 1.0 + _real(ref["deltax"], D).astype(np.float64)
        flip["mass_weighted_global_xH"] = float((dxh * wm)[dis].sum() / wm.sum())
    else:
        flip["mass_weighted_global_xH"] = 0.0
    for k in ("volume_weighted_global_xH", "mass_weighted_global_xH"):
        if k in ref_globals and k in test_globals:
            a, b = ref_globals[k], test_globals[k]
            r = abs(a - b) / max(abs(a), 1e-30)
            rep[k] = r
            ok = abs(a - b) <= REL_TOL * abs(a) + flip[k] * (1 + 1e-6)
            assert ok or (a == 0 and b == 0), f"{k}: {a} vs {b} ({r:.3e}, flipped-cell share {flip[k]:.3e})"
    for k in ("volume_ave_TS", "volume_ave_TK", "volume_ave_Tb"):
        if k in ref_globals and k in test_globals and ref_globals[k] != 0:
            r = abs(ref_globals[k] - test_globals[k]) / abs(ref_globals[k])
            rep[k] = r
            assert r <= GRID_RTOL, f"{k}: {ref_globals[k]} vs {test_globals[k]} ({r:.3e})"

    same = ~(dis | rb_dis)
    # grid -> (cells compared, allowed fraction of outliers without margins)
    first_dep = same & ~near_first
    checks = {
        "xH": same,
        "z_at_ionization": same,
        "delta_T": same,
        "TS_box": np.ones(n, bool),
        "Tk_box": np.ones(n, bool),
        "x_e_box_prev": np.ones(n, bool),
        "vel": np.ones(n, bool),
        "J_21": first_dep,
        "J_21_at_ionization": first_dep,
        "Gamma12": first_dep,
        "N_rec": first_dep,
    }
    for k, sel in checks.items():
        if k not in ref or k not in test or ref[k] is None or test[k] is None:
            continue
        a = _real(ref[k], D).astype(np.float64)
        b = _real(test[k], D).astype(np.float64)
        if not sel.any():
            continue
        scale = max(float(np.abs(a).max()), 1e-300)
        if k == "xH":
            bad = np.abs(a - b) > XH_ATOL + floor
            rep[k + "_floor_only"] = int((sel & ~bad & (np.abs(a - b) > XH_ATOL)).sum())
        elif k == "z_at_ionization":
            bad = a != b
        else:
            tol = GRID_RTOL * np.abs(a) + floor * scale
            if k == "N_rec" and "Gamma12" in ref and "Gamma12" in test and ref["Gamma12"] is not None:
                # N_rec grows by RR(z, Gamma12): the rate rises more slowly
                # than Gamma12, so Gamma12's own relative difference at the
                # cell (itself within its FFT floor) bounds what it passes on
                ga = _real(ref["Gamma12"], D).astype(np.float64)
                gb = _real(test["Gamma12"], D).astype(np.float64)
                tol = tol + np.abs(a) * np.abs(ga - gb) / np.maximum(np.abs(ga), 1e-300)
            bad = np.abs(a - b) > tol
            # cells inside the tolerance only through the FFT floor
            rep[k + "_floor_only"] = int((sel & ~bad & (np.abs(a - b) > tol - floor * scale)).sum())
        bad &= sel
        err = np.abs(a - b)[sel] / np.maximum(np.abs(a[sel]), floor * scale)
        rep[k] = float(err.max()) if err.size else 0.0
        rep[k + "_outliers"] = int(bad.sum())
        allowed = 0 if margin is not None or k in ("TS_box", "Tk_box", "x_e_box_prev", "xH", "delta_T", "vel") \
            else FLAG_FRACTION * n
        if bad.sum() > allowed:
            i = int(np.flatnonzero(bad)[0])
            ctx = {g: (float(_real(ref[g], D)[i]), float(_real(test[g], D)[i]))
                   for g in ("xH", "Gamma12", "J_21", "N_rec", "deltax", "r_bubble")
                   if g in ref and g in test and ref[g] is not None and test[g] is not None}
            if margin is not None:
                ctx["margins"] = (float(margin[0].reshape(-1)[i]), float(margin[1].reshape(-1)[i]))
            ctx["max_abs"] = scale
        assert bad.sum() <= allowed, \
            f"{k}: {bad.sum()} cells outside tolerance (max rel {rep[k]:.3e}); first at {ctx if bad.sum() > allowed else ''}"
    return rep
