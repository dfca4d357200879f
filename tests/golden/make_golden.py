"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

The reference's own reionization sources (src/core/*.c of meraxes) are
compiled unmodified against the shims in oracle/shims/ (`make -C oracle ref`,
which needs the reference tree) and run on the seeded synthetic cases of
tests/cases.py.  Each fixture stores the inputs of every snapshot, the final
grids and the per-snapshot global scalars.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py full24     # one case
    python tests/golden/make_golden.py ps         # power spectrum fixture
    python tests/golden/make_golden.py lightcone  # light-cone fixture
    python tests/golden/make_golden.py deposit    # galaxy deposit + Mvir_crit

Each case runs in a fresh process because the reference keeps its state in
globals.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def make_one(name: str):
    import numpy as np

    from cases import CASES, OUTPUT_GRIDS, initial
    from meraxes_gb300 import synthetic as syn
    from oracle import RefBackend

    case = CASES[name]
    w = case.workload()
    ref = RefBackend(w.params, w.redshifts, syn.TABLES_DIR)
    gen = syn.FieldGenerator(w)
    st = initial(w, ref.n_sfr_histories)
    arrays = {}
    for k, v in st.items():
        arrays["init/" + k] = v.copy()
    glob = []
    for s in w.snapshots:
        inp = gen.inputs(s, ref.n_sfr_histories)
        for k, v in inp.items():
            arrays[f"in{s}/{k}"] = v.copy()
        st.update(inp)
        glob.append(ref.step(s, st))
    for k in OUTPUT_GRIDS:
        if k in st and st[k] is not None:
            arrays["out/" + k] = st[k]
    meta = {"case": name, "snapshots": w.snapshots, "redshifts": w.redshifts, "globals": glob,
            "n_sfr_histories": ref.n_sfr_histories, "grid_dim": w.params.grid_dim}
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    print(name, "written")


def make_ps(name: str = "plain32_tophat"):
    """Compute_PS of the reference on the reference's own delta_T output of a
    golden case: ps_<case>.npz holds delta_T, k, P and error per bin."""
    import numpy as np

    from cases import CASES
    from meraxes_gb300 import synthetic as syn
    from oracle import RefBackend

    d = np.load(os.path.join(HERE, f"{name}.npz"))
    dT = d["out/delta_T"]
    w = CASES[name].workload()
    ref = RefBackend(w.params, w.redshifts, syn.TABLES_DIR)
    k, P, err = ref.power_spectrum(dT)
    np.savez_compressed(os.path.join(HERE, f"ps_{name}.npz"), delta_T=dT, k=k, P=P, error=err,
                        box_size=w.params.box_size, hubble_h=w.params.hubble_h)
    print(f"ps_{name} written")


LC_ZZ = [12.0 - 4.0 * i / 9 for i in range(10)]


def lightcone_inputs(D: int = 16):
    """Seeded delta_T boxes of the light-cone fixture, one per snapshot."""
    import numpy as np

    rng = np.random.default_rng(3)
    return [rng.normal(10, 3, (D, D, D)).astype(np.float32) for _ in LC_ZZ]


def make_lightcone(D: int = 16, L: float = 64.0, end_z: float = 8.6):
    """ConstructLightcone of the reference over the 10-snapshot list LC_ZZ."""
    import numpy as np

    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.params import ReionParams
    from oracle import RefBackend

    p = ReionParams(grid_dim=D, box_size=L, flag_21cm=1)
    ref = RefBackend(p, LC_ZZ, syn.TABLES_DIR)
    n, end = ref.lightcone_init(end_z, len(LC_ZZ) - 1)
    prev = np.zeros((D, D, D), np.float32)
    lc = np.zeros((D, D, n), np.float32)
    lz = np.zeros(n, np.float32)
    for s, dT in enumerate(lightcone_inputs(D)):
        ref.construct_lightcone(s, dT, prev, lc, lz)
    np.savez_compressed(os.path.join(HERE, "lightcone16.npz"), lightcone=lc, redshifts=lz, delta_T_prev=prev,
                        length=n, end_snapshot=end, box_size=L, end_redshift=end_z)
    print("lightcone16 written")


DEPOSIT_CASE = ("dep16", "evolve_512", 16, {"reion_efficiency": 31043.3, "clumping_factor": 2.0})
DEPOSIT_BH = ((0, 0.0, 0.0), (1, 1e-5, 1.57))  # Flag_BHFeedback, BlackHoleMassLimitReion, ReionAlphaUVBH
MVIR_SM = (0.049, 0.17, -2.1, 2.0, 2.5)  # ReionSMParam_m0, a, b, c, d


def deposit_history_init(n_slices: int, npad: int):
    """A non-zero starting sfr_histories, so that the shift is visible."""
    import numpy as np

    base = (np.arange(npad) % 97).astype(np.float32) * np.float32(1e-4)
    return np.stack([base + np.float32(k) for k in range(n_slices)]).astype(np.float32)


def mvir_inputs(D: int):
    """Seeded J_21 and z at ionisation (60% of the cells ionised)."""
    import numpy as np

    rng = np.random.default_rng(2)
    J = (10.0 ** rng.normal(-1, 0.5, (D,) * 3)).astype(np.float32)
    zi = np.where(rng.random((D,) * 3) < 0.6, rng.uniform(9.0, 14.0, (D,) * 3), -1.0).astype(np.float32)
    return J, zi


def make_deposit(n: int = 2000):
    """construct_baryon_grids of the reference for two snapshots (without,
    then with BH feedback) on seeded galaxy lists, and calculate_Mvir_crit at
    z = 10 on seeded ionisation histories."""
    import numpy as np

    from cases import Case, galaxies
    from meraxes_gb300 import synthetic as syn
    from oracle import RefBackend

    name, kind, D, over = DEPOSIT_CASE
    w = Case(name, kind, D, over, fesc=0.01).workload()
    ref = RefBackend(w.params, w.redshifts, syn.TABLES_DIR)
    npad = D * D * 2 * (D // 2 + 1)
    st = {k: np.zeros(npad, np.float32).reshape(D, D, -1) for k in ("stars", "weighted_sfr", "sfr")}
    st["sfr_histories"] = deposit_history_init(ref.n_sfr_histories, npad)
    arrays = {"sfr_histories_init": st["sfr_histories"].copy()}
    for s, bh in enumerate(DEPOSIT_BH):
        gal = galaxies(D, w.params.box_size, n, 11 + s)
        for k, v in gal.items():
            arrays[f"gal{s}/{k}"] = v
        ref.construct_baryon_grids(s, gal, st, bh)
        for k in ("stars", "weighted_sfr", "sfr", "sfr_histories"):
            arrays[f"out{s}/{k}"] = st[k].copy()
    J, zi = mvir_inputs(D)
    arrays.update(J_21_at_ionization=J, z_at_ionization=zi, Mvir_crit=ref.calculate_Mvir_crit(10.0, MVIR_SM, J, zi))
    np.savez_compressed(os.path.join(HERE, "deposit16.npz"), **arrays)
    print("deposit16 written")


if __name__ == "__main__":
    from cases import CASES

    if sys.argv[1:2] == ["ps"]:
        make_ps()
        sys.exit(0)
    if sys.argv[1:2] == ["lightcone"]:
        make_lightcone()
        sys.exit(0)
    if sys.argv[1:2] == ["deposit"]:
        make_deposit()
        sys.exit(0)
    names = sys.argv[1:] or list(CASES)
    if len(names) == 1:
        make_one(names[0])
    else:
        for n in names:
            subprocess.run([sys.executable, os.path.abspath(__file__), n], check=True)
