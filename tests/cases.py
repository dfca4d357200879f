"""Parity cases shared by the golden generator, the CPU tests and the GPU tests.

A case is a workload (meraxes_gb300.params.workload) at a small grid size,
with overrides, run for a list of snapshots through the full step.  Inputs are
the seeded synthetic grids; the persistent state starts from
synthetic.initial_state.
"""
from __future__ import annotations

import copy
import dataclasses
from typing import Dict, List, Optional

import numpy as np

from meraxes_gb300 import synthetic as syn
from meraxes_gb300.params import ReionParams, Workload, workload


@dataclasses.dataclass
class Case:
    name: str
    base: str
    grid_dim: int
    overrides: Dict[str, float]
    fesc: float = 1.0
    snapshots: Optional[List[int]] = None  # default: the workload's snapshots

    def workload(self) -> Workload:
        w = workload(self.base, self.grid_dim)
        for k, v in self.overrides.items():
            setattr(w.params, k, v)
        w.fesc = self.fesc
        if self.snapshots is not None:
            w.snapshots = list(self.snapshots)
        w.name = self.name
        return w


REION_EFF = 1.0 / 0.15714 * 4000.0 / (1.0 - 0.75 * 0.24)  # set_ReionEfficiency, reionization.c:181-210

CASES = {
    # config-1 literal (ReionEfficiency = 1): almost nothing ionises
    "plain32_eff1": Case("plain32_eff1", "plain_64", 32, {}),
    # mixed ionisation state, tophat / sharp-k / Gaussian filters
    "plain32_tophat": Case("plain32_tophat", "plain_64", 32, {"reion_efficiency": 3000.0}),
    "plain32_sharpk": Case("plain32_sharpk", "plain_64", 32, {"reion_efficiency": 3000.0, "filter_type": 1}),
    "plain32_gauss": Case("plain32_gauss", "plain_64", 32, {"reion_efficiency": 3000.0, "filter_type": 2,
                                                             "rtom_filter_type": 1}),
    # full step: recombinations + spin temperature + 21cm (reference clumping 2)
    "full24": Case("full24", "full_256", 24, {"reion_efficiency": REION_EFF, "clumping_factor": 2.0}, fesc=0.01),
    # several snapshots with the SFR-history reweighting and persistent state
    "evolve16": Case("evolve16", "evolve_512", 16, {"reion_efficiency": REION_EFF, "clumping_factor": 2.0},
                     fesc=0.01, snapshots=[0, 1, 2, 3, 4, 5]),
    # peculiar-velocity modes of the brightness temperature: 1 capped
    # gradient, 2 optical depth (GBPTREES velocity units), 3 with the
    # line-of-sight redshift-space remap
    "full24_pv1": Case("full24_pv1", "full_256", 24, {"reion_efficiency": REION_EFF, "clumping_factor": 2.0,
                                                      "flag_pecvel": 1}, fesc=0.01),
    "full24_pv2": Case("full24_pv2", "full_256", 24, {"reion_efficiency": REION_EFF, "clumping_factor": 2.0,
                                                      "flag_pecvel": 2, "trees_id": 1}, fesc=0.01),
    "full24_pv3": Case("full24_pv3", "full_256", 24, {"reion_efficiency": REION_EFF, "clumping_factor": 2.0,
                                                      "flag_pecvel": 3}, fesc=0.01),
}


def initial(w: Workload, n_hist: int) -> Dict[str, np.ndarray]:
    s0 = w.snapshots[0]
    z_prev = w.redshifts[s0 - 1] if s0 > 0 else w.redshifts[s0]
    st = syn.initial_state(w.params, z_prev)
    return st


def run_case(backend, w: Workload, gen: Optional[syn.FieldGenerator] = None, state=None):
    """Runs the full step for every snapshot of `w` on `backend` (an object
    with .step(snapshot, grids) and .n_sfr_histories).  Returns the final
    state dict and the per-snapshot globals."""
    gen = gen or syn.FieldGenerator(w)
    st = state if state is not None else initial(w, backend.n_sfr_histories)
    glob = []
    for s in w.snapshots:
        st.update(gen.inputs(s, backend.n_sfr_histories))
        glob.append(backend.step(s, st))
    return st, glob


OUTPUT_GRIDS = ["xH", "z_at_ionization", "r_bubble", "J_21", "J_21_at_ionization", "Gamma12", "N_rec", "delta_T",
                "TS_box", "Tk_box", "x_e_box_prev", "x_e_box", "vel"]


def galaxies(D: int, L: float, n: int, seed: int) -> Dict[str, np.ndarray]:
    """Seeded galaxy list for the deposit: uniform positions (a few exactly on
    the far box face, which the nearest-grid-point rule wraps to cell 0), ~10%
    dead galaxies (Type 3, skipped), lognormal masses in internal units
    (1e10 Msun/h), and black holes."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, (n, 3)).astype(np.float32)
    pos[: max(1, n // 50), 0] = np.float32(L)
    typ = rng.choice([0, 1, 2, 3], size=n, p=[0.5, 0.3, 0.1, 0.1]).astype(np.int32)
    gsm = 10.0 ** rng.normal(-4.0, 1.0, n)
    return {"pos": np.ascontiguousarray(pos), "type": typ, "fesc_gsm": 0.1 * gsm, "gross_sm": gsm,
            "bhm": 10.0 ** rng.normal(-5.0, 1.0, n), "ebhm": 10.0 ** rng.normal(-6.0, 1.0, n)}
