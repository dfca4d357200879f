"""Live check of the restatement against the reference's own sources compiled
with the shims (only where the reference tree is present)."""
import subprocess
import sys
import os

import pytest

from oracle import ref_available

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference tree not present")

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from cases import Case, run_case, OUTPUT_GRIDS
from meraxes_gb300 import synthetic as syn
from oracle import OracleBackend, RefBackend
c = Case('live', {base!r}, {D}, {ov!r}, fesc={fesc})
w = c.workload()
ref = RefBackend(w.params, w.redshifts, syn.TABLES_DIR)
orc = OracleBackend(w.params, w.redshifts, syn.TABLES_DIR)
a, ga = run_case(ref, w)
b, gb = run_case(orc, w)
bad = []
for k in OUTPUT_GRIDS:
    if k in a and a[k] is not None and not np.array_equal(a[k], b[k], equal_nan=True):
        bad.append(k)
for x, y in zip(ga, gb):
    for k in x:
        if k in y and k not in ('n_radii', 'gpu_launches') and x[k] != y[k] and abs(x[k]-y[k]) > 1e-14*abs(x[k]):
            bad.append(k)
print('MISMATCH' if bad else 'OK', bad)
"""


@pytest.mark.parametrize("base,D,ov,fesc", [
    ("plain_64", 16, {"reion_efficiency": 2000.0, "delta_r_factor": 1.3}, 1.0),
    ("plain_64", 20, {"reion_efficiency": 5000.0, "filter_type": 1, "uvb_flag": 0}, 1.0),
    ("full_256", 16, {"reion_efficiency": 31043.0, "clumping_factor": 2.0, "filter_type": 2}, 0.02),
    # peculiar-velocity modes of the brightness temperature (half-neutral
    # boxes: mean xH ~0.5, delta_T ~10 mK, every mode changes it)
    ("full_256", 16, {"reion_efficiency": 31043.3, "clumping_factor": 2.0, "flag_pecvel": 1}, 0.01),
    ("full_256", 16, {"reion_efficiency": 31043.3, "clumping_factor": 2.0, "flag_pecvel": 2, "trees_id": 1}, 0.01),
    ("full_256", 20, {"reion_efficiency": 31043.3, "clumping_factor": 2.0, "flag_pecvel": 3}, 0.01),
])
def test_restatement_bit_exact_against_reference(base, D, ov, fesc):
    here = os.path.dirname(os.path.abspath(__file__))
    code = SCRIPT.format(root=os.path.dirname(here), tests=here, base=base, D=D, ov=ov, fesc=fesc)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().startswith("OK"), r.stdout


PS_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from meraxes_gb300.params import ReionParams
from meraxes_gb300 import synthetic as syn
from oracle import OracleBackend, RefBackend
p = ReionParams(grid_dim={D}, box_size={L}, flag_21cm=1)
rng = np.random.default_rng(5)
dT = (rng.normal(10.0, 4.0, ({D},) * 3)).astype(np.float32)
a = RefBackend(p, [8.5, 8.0], syn.TABLES_DIR).power_spectrum(dT)
b = OracleBackend(p, [8.5, 8.0], syn.TABLES_DIR).power_spectrum(dT)
ok = all(np.array_equal(x, y, equal_nan=True) for x, y in zip(a, b))
print('OK' if ok else 'MISMATCH', [np.max(np.abs(x - y)) for x, y in zip(a, b)])
"""


@pytest.mark.parametrize("D,L", [(16, 40.0), (24, 30.0)])
def test_power_spectrum_restatement_bit_exact_against_reference(D, L):
    here = os.path.dirname(os.path.abspath(__file__))
    code = PS_SCRIPT.format(root=os.path.dirname(here), tests=here, D=D, L=L)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().startswith("OK"), r.stdout


LC_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from meraxes_gb300.params import ReionParams
from meraxes_gb300 import synthetic as syn
from oracle import OracleBackend, RefBackend
D = {D}
p = ReionParams(grid_dim=D, box_size={L}, flag_21cm=1)
zz = [12.0 - 4.0 * i / 9 for i in range(10)]
out = []
for B in (RefBackend, OracleBackend):
    b = B(p, zz, syn.TABLES_DIR)
    n, end = b.lightcone_init(8.6, len(zz) - 1)
    prev = np.zeros((D, D, D), np.float32)
    lc = np.zeros((D, D, n), np.float32); lz = np.zeros(n, np.float32)
    rng = np.random.default_rng(3)
    for s in range(len(zz)):
        dT = rng.normal(10, 3, (D, D, D)).astype(np.float32)
        b.construct_lightcone(s, dT, prev, lc, lz)
    out.append((n, end, lc, lz, prev))
a, c = out
ok = a[0] == c[0] and a[1] == c[1] and all(np.array_equal(x, y) for x, y in zip(a[2:], c[2:]))
print('OK' if ok else 'MISMATCH', a[0], a[1], c[0], c[1])
"""


@pytest.mark.parametrize("D,L", [(16, 64.0), (20, 200.0)])
def test_lightcone_restatement_bit_exact_against_reference(D, L):
    here = os.path.dirname(os.path.abspath(__file__))
    code = LC_SCRIPT.format(root=os.path.dirname(here), tests=here, D=D, L=L)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().startswith("OK"), r.stdout


DEPOSIT_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from cases import Case, initial, galaxies
from meraxes_gb300 import synthetic as syn
from oracle import OracleBackend, RefBackend
c = Case('dep', 'full_256', {D}, {{'reion_efficiency': 31043.3, 'clumping_factor': 2.0}}, fesc=0.01)
w = c.workload()
outs = []
for B in (RefBackend, OracleBackend):
    b = B(w.params, w.redshifts, syn.TABLES_DIR)
    st = initial(w, b.n_sfr_histories)
    D = w.params.grid_dim
    npad = D * D * 2 * (D // 2 + 1)
    st.update({{k: np.zeros(npad, np.float32).reshape(D, D, -1) for k in ('stars', 'weighted_sfr', 'sfr')}})
    st['sfr_histories'] = np.random.default_rng(1).random((b.n_sfr_histories, npad)).astype(np.float32)
    res = []
    for s, bh in ((0, (0, 0.0, 0.0)), (1, (1, 1e-5, 1.57))):
        b.construct_baryon_grids(s, galaxies(D, w.params.box_size, {n}, 11 + s), st, bh)
        res += [st[k].copy() for k in ('stars', 'weighted_sfr', 'sfr', 'sfr_histories')]
    rng = np.random.default_rng(2)
    J = (10.0 ** rng.normal(-1, 0.5, (D,) * 3)).astype(np.float32)
    zi = np.where(rng.random((D,) * 3) < 0.6, rng.uniform(9.0, 14.0, (D,) * 3), -1.0).astype(np.float32)
    res.append(b.calculate_Mvir_crit(10.0, (0.049, 0.17, -2.1, 2.0, 2.5), J, zi))
    outs.append(res)
ok = all(np.array_equal(x, y) for x, y in zip(*outs))
print('OK' if ok else 'MISMATCH', [float(np.abs(x - y).max()) for x, y in zip(*outs)],
      'nonzero stars', int((outs[0][0] > 0).sum()), 'Mvir_crit>0', int((outs[0][-1] > 0).sum()))
"""


@pytest.mark.parametrize("D,n", [(16, 3000), (24, 20000)])
def test_deposit_and_Mvir_crit_restatements_bit_exact_against_reference(D, n):
    here = os.path.dirname(os.path.abspath(__file__))
    code = DEPOSIT_SCRIPT.format(root=os.path.dirname(here), tests=here, D=D, n=n)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().startswith("OK"), r.stdout
