"""Parity checks between two runs of the grid step (test helpers).

Tolerances follow the acceptance rule of the GB300 step: mean xHI within 1e-5
relative; ionisation flags may disagree in at most 1e-4 of the cells and only
where the oracle's threshold margin |f_coll*eff/(nf(1+rec)) - 1| is below 1e-5;
T_S and delta_T within 1e-4 relative; the other grids within 1e-4 relative
(or a small absolute floor) where the flags agree.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

REL_TOL = 1e-5
FLAG_FRACTION = 1e-4
MARGIN = 1e-5
GRID_RTOL = 1e-4


def _rel(a, b, floor):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return np.abs(a - b) / np.maximum(np.abs(a), floor)


def compare(ref: Dict[str, np.ndarray], test: Dict[str, np.ndarray], ref_globals: Dict[str, float],
            test_globals: Dict[str, float], margin: Optional[np.ndarray] = None, exact: bool = False,
            report: Optional[dict] = None):
    """Raises AssertionError with a readable message on a parity violation."""
    rep = report if report is not None else {}
    D = ref["xH"].shape[0]
    n = D ** 3
    fa = ref["xH"].reshape(-1) < REL_TOL
    fb = test["xH"].reshape(-1) < REL_TOL
    dis = fa != fb
    rep["flag_disagree"] = int(dis.sum())
    # r_bubble / first-crossing quantities can differ in near-threshold cells
    rb_dis = ref["r_bubble"].reshape(-1) != test["r_bubble"].reshape(-1)
    rep["rbubble_disagree"] = int(rb_dis.sum())
    if exact:
        assert dis.sum() == 0, f"flags differ in {dis.sum()} cells"
    else:
        assert dis.sum() <= max(FLAG_FRACTION * n, 0), f"flags differ in {dis.sum()} of {n} cells"
        if margin is not None and dis.any():
            m = margin.reshape(-1)[dis]
            assert np.all(m < MARGIN), f"flag disagreement at margin {m.max():.3e}"
        if margin is not None and rb_dis.any():
            m = margin.reshape(-1)[rb_dis]
            rep["rbubble_margin_max"] = float(m.max())
            assert np.all(m < MARGIN), f"r_bubble disagreement at margin {m.max():.3e}"
    same = ~(dis | rb_dis)
    for k in ("volume_weighted_global_xH", "mass_weighted_global_xH"):
        if k in ref_globals:
            a, b = ref_globals[k], test_globals[k]
            r = abs(a - b) / max(abs(a), 1e-30)
            rep[k] = r
            assert r <= (1e-12 if exact else REL_TOL) or (a == 0 and b == 0), f"{k}: {a} vs {b} ({r:.3e})"
    for k in ("volume_ave_TS", "volume_ave_TK", "volume_ave_Tb"):
        if k in ref_globals and k in test_globals and ref_globals[k] != 0:
            r = abs(ref_globals[k] - test_globals[k]) / abs(ref_globals[k])
            rep[k] = r
            assert r <= (1e-12 if exact else GRID_RTOL), f"{k}: {ref_globals[k]} vs {test_globals[k]} ({r:.3e})"
    checks = {
        "xH": (1e-4, 1.0),
        "z_at_ionization": (0.0, 1.0),
        "J_21": (GRID_RTOL, 1e-3),
        "J_21_at_ionization": (GRID_RTOL, 1e-3),
        "Gamma12": (GRID_RTOL, 1e-6),
        "N_rec": (GRID_RTOL, 1e-6),
        "delta_T": (GRID_RTOL, 1e-3),
        "TS_box": (GRID_RTOL, 1e-3),
        "Tk_box": (GRID_RTOL, 1e-3),
    }
    for k, (rtol, floor) in checks.items():
        if k not in ref or k not in test or ref[k] is None or test[k] is None:
            continue
        a = ref[k].reshape(-1)[: n] if ref[k].size == n else _real(ref[k], D)
        b = test[k].reshape(-1)[: n] if test[k].size == n else _real(test[k], D)
        sel = same if k in ("xH", "z_at_ionization", "J_21", "J_21_at_ionization", "Gamma12", "delta_T", "N_rec") \
            else np.ones(n, bool)
        if not sel.any():
            continue
        if k == "xH":
            err = np.abs(a[sel].astype(np.float64) - b[sel])
        else:
            err = _rel(a[sel], b[sel], floor * max(np.abs(a).max(), 1e-30) if k not in ("xH",) else floor)
        worst = float(err.max()) if err.size else 0.0
        rep[k] = worst
        if exact:
            assert worst == 0.0, f"{k}: max error {worst:.3e}"
        else:
            assert worst <= rtol + (0 if rtol else 0), f"{k}: max error {worst:.3e} > {rtol}"
    return rep


def _real(padded: np.ndarray, D: int) -> np.ndarray:
    return np.ascontiguousarray(padded.reshape(D, D, -1)[:, :, :D]).reshape(-1)
