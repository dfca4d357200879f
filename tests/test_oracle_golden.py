"""The C restatement (oracle) against the golden fixtures produced by the
reference's own sources (tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from cases import CASES, OUTPUT_GRIDS
from compare import compare
from meraxes_gb300 import synthetic as syn
from oracle import OracleBackend

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(bytes(d["meta"]).decode())
    return d, meta


def golden_inputs(d, meta):
    init = {k[5:]: np.array(d[k]) for k in d.files if k.startswith("init/")}
    per = {}
    for s in meta["snapshots"]:
        per[s] = {k.split("/", 1)[1]: np.array(d[k]) for k in d.files if k.startswith(f"in{s}/")}
    out = {k[4:]: np.array(d[k]) for k in d.files if k.startswith("out/")}
    return init, per, out


def run_on(backend, meta, init, per):
    st = {k: v.copy() for k, v in init.items()}
    glob = []
    for s in meta["snapshots"]:
        st.update({k: v.copy() for k, v in per[s].items()})
        glob.append(backend.step(s, st))
    return st, glob


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_reference_fixture(name, tables_dir):
    d, meta = load_golden(name)
    w = CASES[name].workload()
    init, per, out = golden_inputs(d, meta)
    orc = OracleBackend(w.params, meta["redshifts"], tables_dir)
    assert orc.n_sfr_histories == meta["n_sfr_histories"]
    st, glob = run_on(orc, meta, init, per)
    # same FFT and numerics restatement on both sides: agreement to FP32
    # rounding of differently compiled arithmetic (bit-exact on the machine
    # that generated the fixtures)
    for k in OUTPUT_GRIDS:
        if k in out:
            a, b = out[k].astype(np.float64), st[k].astype(np.float64)
            err = np.abs(a - b) / np.maximum(np.abs(a), 1e-30 + 1e-6 * np.abs(a).max())
            assert err.max() < 1e-5, (k, err.max())
    for g_ref, g_orc in zip(meta["globals"], glob):
        for k, v in g_ref.items():
            if k in g_orc and k not in ("n_radii", "gpu_launches") and v != 0:
                assert abs(g_orc[k] - v) <= 1e-6 * abs(v), (k, v, g_orc[k])


def test_fixture_cases_cover_the_paths():
    seen = {CASES[n].workload().params.filter_type for n in CASES}
    assert seen == {0, 1, 2}
    assert any(CASES[n].workload().params.flag_recombinations for n in CASES)
    assert any(CASES[n].workload().params.flag_spin_temp for n in CASES)
    assert any(len(CASES[n].workload().snapshots) > 1 for n in CASES)


def test_oracle_power_spectrum_matches_reference_fixture():
    """Compute_PS restated == the reference's Compute_PS on the reference's
    own delta_T output (bit-exact)."""
    import os

    from cases import CASES
    from meraxes_gb300 import synthetic as syn
    from oracle import OracleBackend

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ps_plain32_tophat.npz"))
    w = CASES["plain32_tophat"].workload()
    orc = OracleBackend(w.params, w.redshifts, syn.TABLES_DIR)
    k, P, err = orc.power_spectrum(d["delta_T"])
    assert np.array_equal(k, d["k"], equal_nan=True)
    assert np.array_equal(P, d["P"], equal_nan=True)
    assert np.array_equal(err, d["error"], equal_nan=True)


def test_oracle_lightcone_matches_reference_fixture():
    """ConstructLightcone restated == the reference's, over 10 snapshots."""
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import LC_ZZ, lightcone_inputs

    from meraxes_gb300.params import ReionParams

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lightcone16.npz"))
    p = ReionParams(grid_dim=16, box_size=float(d["box_size"]), flag_21cm=1)
    orc = OracleBackend(p, LC_ZZ, syn.TABLES_DIR)
    n, end = orc.lightcone_init(float(d["end_redshift"]), len(LC_ZZ) - 1)
    assert (n, end) == (int(d["length"]), int(d["end_snapshot"]))
    prev = np.zeros((16, 16, 16), np.float32)
    lc = np.zeros((16, 16, n), np.float32)
    lz = np.zeros(n, np.float32)
    for s, dT in enumerate(lightcone_inputs(16)):
        orc.construct_lightcone(s, dT, prev, lc, lz)
    assert np.array_equal(lc, d["lightcone"]) and np.array_equal(lz, d["redshifts"])
    assert np.array_equal(prev, d["delta_T_prev"])


def test_oracle_deposit_and_Mvir_crit_match_reference_fixture():
    """construct_baryon_grids (two snapshots, without and with BH feedback)
    and calculate_Mvir_crit restated == the reference's, bit for bit."""
    import os
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    from make_golden import DEPOSIT_BH, DEPOSIT_CASE, MVIR_SM

    from cases import Case

    d = np.load(os.path.join(here, "golden", "deposit16.npz"))
    name, kind, D, over = DEPOSIT_CASE
    w = Case(name, kind, D, over, fesc=0.01).workload()
    orc = OracleBackend(w.params, w.redshifts, syn.TABLES_DIR)
    npad = D * D * 2 * (D // 2 + 1)
    st = {k: np.zeros(npad, np.float32).reshape(D, D, -1) for k in ("stars", "weighted_sfr", "sfr")}
    st["sfr_histories"] = d["sfr_histories_init"].copy()
    assert st["sfr_histories"].shape[0] == orc.n_sfr_histories
    for s, bh in enumerate(DEPOSIT_BH):
        gal = {k: d[f"gal{s}/{k}"] for k in ("pos", "type", "fesc_gsm", "gross_sm", "bhm", "ebhm")}
        orc.construct_baryon_grids(s, gal, st, bh)
        for k in ("stars", "weighted_sfr", "sfr", "sfr_histories"):
            assert np.array_equal(st[k], d[f"out{s}/{k}"]), (s, k)
    assert (d["out1/stars"] > 0).sum() > 1000
    out = orc.calculate_Mvir_crit(10.0, MVIR_SM, d["J_21_at_ionization"], d["z_at_ionization"])
    assert np.array_equal(out, d["Mvir_crit"]) and (out > 0).sum() > 1000
