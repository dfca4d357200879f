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


if __name__ == "__main__":
    from cases import CASES

    if sys.argv[1:2] == ["ps"]:
        make_ps()
        sys.exit(0)
    if sys.argv[1:2] == ["lightcone"]:
        make_lightcone()
        sys.exit(0)
    names = sys.argv[1:] or list(CASES)
    if len(names) == 1:
        make_one(names[0])
    else:
        for n in names:
            subprocess.run([sys.executable, os.path.abspath(__file__), n], check=True)
