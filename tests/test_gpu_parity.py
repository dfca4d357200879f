"""CUDA path against the oracle and the reference fixtures (GB300)."""
import os

import numpy as np
import pytest

from cases import CASES, Case, OUTPUT_GRIDS, run_case
from compare import compare
from test_oracle_golden import golden_inputs, load_golden, run_on

pytestmark = pytest.mark.gpu


class GpuBackend:
    """The product through its host-pointer C ABI entry point mx_step."""

    def __init__(self, params, redshifts):
        from meraxes_gb300.api import ReionGridStep

        self.step_obj = ReionGridStep(params, redshifts)
        self.n_sfr_histories = self.step_obj.n_sfr_histories
        self.launches = []

    def step(self, snapshot, state):
        g = self.step_obj.step(snapshot, state)
        self.launches.append(self.step_obj.last_launches)
        return g


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_matches_reference_fixture(name):
    d, meta = load_golden(name)
    w = CASES[name].workload()
    init, per, out = golden_inputs(d, meta)
    gpu = GpuBackend(w.params, meta["redshifts"])
    assert gpu.n_sfr_histories == meta["n_sfr_histories"]
    st, glob = run_on(gpu, meta, init, per)
    assert all(n > 0 for n in gpu.launches)
    rep = {}
    compare(out, st, meta["globals"][-1], glob[-1], report=rep)
    print(name, rep)


def _run_against_oracle(name, D, tables_dir):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from oracle import OracleBackend

    c = CASES[name]
    case = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots)
    w = case.workload()
    orc = OracleBackend(w.params, w.redshifts, tables_dir)
    gpu = GpuBackend(w.params, w.redshifts)
    gen = syn.FieldGenerator(w)
    sa = initial(w, orc.n_sfr_histories)
    sb = {k: v.copy() for k, v in sa.items()}
    for s in w.snapshots:
        inp = gen.inputs(s, orc.n_sfr_histories)
        sa.update({k: v.copy() for k, v in inp.items()})
        sb.update({k: v.copy() for k, v in inp.items()})
        ga = orc.step(s, sa)
        margin = orc.margin()
        gb = gpu.step(s, sb)
        rep = {}
        compare(sa, sb, ga, gb, margin=margin, report=rep)
    return rep


@pytest.mark.parametrize("name,D", [("plain32_tophat", 64), ("plain32_sharpk", 64), ("plain32_gauss", 48),
                                    ("full24", 48), ("evolve16", 32)])
def test_gpu_matches_oracle_with_margins(name, D, tables_dir):
    print(name, D, _run_against_oracle(name, D, tables_dir))


# Power-of-two grids from 32^3 and the grids 24^3, 48^3, 96^3 and 192^3 (a
# factor 3: radix-3 tile steps and the factor-3 z-pass) run the fused
# transforms by default; MX_TRANSFORM=cufft selects cuFFT C2R with separate
# filter and test passes.  Both must meet the same tolerances against the
# oracle.
@pytest.mark.parametrize("transform", ["fused", "cufft"])
@pytest.mark.parametrize("name,D", [("full24", 64), ("plain32_gauss", 64), ("evolve16", 32),
                                    ("full24", 96), ("plain32_sharpk", 48), ("evolve16", 24)])
def test_both_transform_paths_match_oracle(name, D, transform, tables_dir, monkeypatch):
    monkeypatch.setenv("MX_TRANSFORM", transform)
    print(name, D, transform, _run_against_oracle(name, D, tables_dir))


# The block-size autotuner may pick 256 or 512 threads for the x- and
# y-pass; every choice must give bit-identical grids.
@pytest.mark.parametrize("name,D", [("full24", 64), ("evolve16", 128)])
def test_fft_block_sizes_give_identical_results(name, D, monkeypatch):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    runs = []
    for tx, ty in ((256, 256), (512, 512), (256, 512), (512, 256)):
        monkeypatch.setenv("MX_XPASS_THREADS", str(tx))
        monkeypatch.setenv("MX_YPASS_THREADS", str(ty))
        step = ReionGridStep(w.params, w.redshifts)
        assert step.fft_block_sizes() == (tx, ty)
        gen = syn.FieldGenerator(w)
        st = initial(w, step.n_sfr_histories)
        glob = []
        for s in w.snapshots:
            st.update(gen.inputs(s, step.n_sfr_histories))
            glob.append(step.step(s, st))
        runs.append((st, glob))
        step.close()
    st0, g0 = runs[0]
    for st, g in runs[1:]:
        for k in OUTPUT_GRIDS:
            if k in st0:
                assert np.array_equal(st0[k], st[k]), k
        for a, b in zip(g0, g):
            assert a["volume_weighted_global_xH"] == b["volume_weighted_global_xH"]
    monkeypatch.delenv("MX_XPASS_THREADS")
    monkeypatch.delenv("MX_YPASS_THREADS")
    tuned = ReionGridStep(w.params, w.redshifts)
    assert tuned.fft_block_sizes()[0] in (256, 512) and tuned.fft_block_sizes()[1] in (256, 512)
    tuned.close()


# The evolve kernel takes each tile's shell rows by one tensor copy when the
# context has a tensor map of the shells, else by one bulk copy per row
# (MX_SHELL_MAP=0); the shared-memory tiles, hence the grids, are the same.
@pytest.mark.parametrize("name,D", [("evolve16", 32), ("full24", 64)])
def test_shell_map_gives_identical_results(name, D, monkeypatch):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    runs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("MX_SHELL_MAP", flag)
        step = ReionGridStep(w.params, w.redshifts)
        gen = syn.FieldGenerator(w)
        st = initial(w, step.n_sfr_histories)
        glob = []
        for s in w.snapshots:
            st.update(gen.inputs(s, step.n_sfr_histories))
            glob.append(step.step(s, st))
        runs.append((st, glob))
        step.close()
    (sa, ga), (sb, gb) = runs
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
            assert a[k] == b[k], k


# mx_step on host grids starts ComputeTs's shells as soon as sfr has landed
# and computes the collapse fraction on a side stream (MX_TS_EARLY_SHELLS=0:
# the collapse fraction first, on the compute stream): the same grids.
@pytest.mark.parametrize("name,D", [("evolve16", 32), ("full24", 64)])
def test_early_shells_give_identical_results(name, D, monkeypatch):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    runs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("MX_TS_EARLY_SHELLS", flag)
        step = ReionGridStep(w.params, w.redshifts)
        gen = syn.FieldGenerator(w)
        st = initial(w, step.n_sfr_histories)
        glob = []
        for s in w.snapshots:
            st.update(gen.inputs(s, step.n_sfr_histories))
            glob.append(step.step(s, st))
        runs.append((st, glob))
        step.close()
    (sa, ga), (sb, gb) = runs
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb", "volume_ave_xe", "x_e_ave",
                  "collapse_fraction"):
            assert a[k] == b[k], k


# Radii (and ComputeTs shells) go through the transforms in batches sized by
# the work buffer; at 512^3 find_HII_bubbles takes two.  Small batches
# (MX_MAX_BATCH_SPECTRA) must give the same grids as one batch, bit for bit.
@pytest.mark.parametrize("transform", ["fused", "cufft"])
@pytest.mark.parametrize("name,D,spectra", [("full24", 64, 15), ("plain32_tophat", 64, 6), ("evolve16", 32, 10),
                                            ("full24", 48, 15)])
def test_radius_batches_give_identical_results(name, D, spectra, transform, monkeypatch):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    monkeypatch.setenv("MX_TRANSFORM", transform)
    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    runs = []
    for cap in (None, str(spectra)):
        if cap is None:
            monkeypatch.delenv("MX_MAX_BATCH_SPECTRA", raising=False)
        else:
            monkeypatch.setenv("MX_MAX_BATCH_SPECTRA", cap)
        step = ReionGridStep(w.params, w.redshifts)
        gen = syn.FieldGenerator(w)
        st = initial(w, step.n_sfr_histories)
        glob = []
        for s in w.snapshots:
            st.update(gen.inputs(s, step.n_sfr_histories))
            glob.append(step.step(s, st))
        runs.append((st, glob))
        step.close()
    (sa, ga), (sb, gb) = runs
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
            assert a[k] == b[k], k


def test_device_entry_points_match_host_entry_points():
    import torch

    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    w = CASES["full24"].workload()
    host = ReionGridStep(w.params, w.redshifts)
    dev = ReionGridStep(w.params, w.redshifts)
    gen = syn.FieldGenerator(w)
    s = w.snapshots[0]
    st = initial(w, host.n_sfr_histories)
    st.update(gen.inputs(s, host.n_sfr_histories))
    tst = {k: torch.from_numpy(v.copy()).cuda() for k, v in st.items()}
    gh = host.step(s, st)
    gd = dev.step(s, tst)
    torch.cuda.synchronize()
    for k in OUTPUT_GRIDS:
        if k in st:
            assert np.array_equal(st[k], tst[k].cpu().numpy()), k
    for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
        assert gh[k] == gd[k]


def test_errors_are_reported_not_raised_on_device():
    from meraxes_gb300 import _lib
    from meraxes_gb300.api import ReionGridStep

    w = CASES["plain32_tophat"].workload()
    st = ReionGridStep(w.params, w.redshifts)
    with pytest.raises(_lib.MxError) as e:
        st.find_HII_bubbles(99, {"deltax": np.zeros(1, np.float32)})
    assert e.value.code == -1
    with pytest.raises(_lib.MxError) as e:
        st.find_HII_bubbles(1, {})
    assert e.value.code == -1
    # the context stays usable after an error
    from cases import initial
    from meraxes_gb300 import synthetic as syn

    gen = syn.FieldGenerator(w)
    s = w.snapshots[0]
    g = initial(w, 0)
    g.update(gen.inputs(s, 0))
    out = st.step(s, g)
    assert 0.0 <= out["volume_weighted_global_xH"] <= 1.0


def test_unaligned_device_grids_are_rejected():
    """Device grids 4 bytes past an 8-byte boundary (legal for float*, not for
    cuFFT's real inputs) are refused with MX_EINVAL; the context stays usable."""
    import torch

    from cases import initial
    from meraxes_gb300 import _lib
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    w = CASES["plain32_tophat"].workload()
    step = ReionGridStep(w.params, w.redshifts)
    gen = syn.FieldGenerator(w)
    s = w.snapshots[0]
    st = initial(w, 0)
    st.update(gen.inputs(s, 0))

    def unaligned(a):
        flat = torch.empty(a.size + 1, dtype=torch.float32, device="cuda")
        v = flat[1:].view(a.shape)
        v.copy_(torch.from_numpy(a))
        assert v.data_ptr() % 8 == 4
        return v

    bad = {k: (unaligned(v) if k == "deltax" else torch.from_numpy(v.copy()).cuda()) for k, v in st.items()}
    with pytest.raises(_lib.MxError) as e:
        step.step(s, bad)
    assert e.value.code == -1 and "aligned" in str(e.value)
    good = {k: torch.from_numpy(v.copy()).cuda() for k, v in st.items()}
    out = step.step(s, good)
    assert 0.0 <= out["volume_weighted_global_xH"] <= 1.0


# Power spectrum: the transform is FP32 (cuFFT against the reference's FFTW
# stand-in), so per-bin power agrees to 1e-4 relative; mean |k| per bin to
# 1e-6 (the same float |k| summed in another order); bins and counts exactly
# (error / power = 1 / sqrt(count)).
def _ps_close(a, b):
    ka, Pa, ea = a
    kb, Pb, eb = b
    assert ka.shape == kb.shape
    np.testing.assert_allclose(kb, ka, rtol=1e-6, atol=0)
    np.testing.assert_allclose(Pb, Pa, rtol=1e-4, atol=1e-7 * float(np.nanmax(np.abs(Pa))))
    with np.errstate(invalid="ignore", divide="ignore"):
        np.testing.assert_allclose(eb / Pb, ea / Pa, rtol=1e-5)


def test_gpu_power_spectrum_matches_reference_fixture():
    import torch

    from meraxes_gb300.api import ReionGridStep

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ps_plain32_tophat.npz"))
    w = CASES["plain32_tophat"].workload()
    step = ReionGridStep(w.params, w.redshifts)
    host = step.Compute_PS(d["delta_T"])
    _ps_close((d["k"], d["P"], d["error"]), host)
    dev = step.Compute_PS(torch.from_numpy(d["delta_T"].copy()).cuda())
    for x, y in zip(host, dev):
        assert np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("D,L", [(64, 100.0), (96, 60.0)])
def test_gpu_power_spectrum_matches_oracle(D, L, tables_dir):
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.params import ReionParams
    from oracle import OracleBackend

    p = ReionParams(grid_dim=D, box_size=L, flag_21cm=1)
    rng = np.random.default_rng(D)
    dT = (rng.normal(12.0, 5.0, (D, D, D)) * np.exp(rng.normal(0, 0.3, (D, D, D)))).astype(np.float32)
    ref = OracleBackend(p, [8.5, 8.0], tables_dir).power_spectrum(dT)
    got = ReionGridStep(p, [8.5, 8.0]).Compute_PS(dT)
    _ps_close(ref, got)


@pytest.mark.parametrize("device", [False, True])
def test_gpu_lightcone_matches_reference_fixture_and_oracle(device, tables_dir):
    """Light cone through the C ABI, host and device families: equal to the
    oracle run on this machine (same double arithmetic and host times), and to
    the reference fixture within one float rounding (its host times were made
    with another machine's libm)."""
    import sys

    import torch

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import LC_ZZ, lightcone_inputs

    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.params import ReionParams
    from oracle import OracleBackend

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lightcone16.npz"))
    p = ReionParams(grid_dim=16, box_size=float(d["box_size"]), flag_21cm=1)
    runs = []
    for backend in ("oracle", "gpu"):
        b = OracleBackend(p, LC_ZZ, tables_dir) if backend == "oracle" else ReionGridStep(p, LC_ZZ)
        n, end = b.lightcone_init(float(d["end_redshift"]), len(LC_ZZ) - 1)
        assert (n, end) == (int(d["length"]), int(d["end_snapshot"]))
        prev = np.zeros((16, 16, 16), np.float32)
        lc = np.zeros((16, 16, n), np.float32)
        lz = np.zeros(n, np.float32)
        if backend == "gpu" and device:
            prev_t, lc_t = torch.from_numpy(prev).cuda(), torch.from_numpy(lc).cuda()
            for s, dT in enumerate(lightcone_inputs(16)):
                b.ConstructLightcone(s, torch.from_numpy(dT).cuda(), prev_t, lc_t, lz)
            torch.cuda.synchronize()
            prev, lc = prev_t.cpu().numpy(), lc_t.cpu().numpy()
        else:
            for s, dT in enumerate(lightcone_inputs(16)):
                (b.construct_lightcone if backend == "oracle" else b.ConstructLightcone)(s, dT, prev, lc, lz)
        runs.append((lc, lz, prev))
    (lo, zo, po), (lg, zg, pg) = runs
    assert np.array_equal(lg, lo) and np.array_equal(zg, zo) and np.array_equal(pg, po)
    np.testing.assert_allclose(lg, d["lightcone"], rtol=2 ** -23, atol=0)
    np.testing.assert_allclose(zg, d["redshifts"], rtol=2 ** -23, atol=0)


# galaxy arrays: the oracle's names -> the mx_galaxies names of the API
GAL_API = {"pos": "pos", "type": "type", "fesc_gsm": "fesc_weighted_gsm", "gross_sm": "gross_stellar_mass",
           "bhm": "black_hole_mass", "ebhm": "effective_bhm"}
DEPOSIT_GRIDS = ("stars", "weighted_sfr", "sfr", "sfr_histories")


def _deposit_state(D, hist0):
    npad = D * D * 2 * (D // 2 + 1)
    st = {k: np.zeros(npad, np.float32).reshape(D, D, -1) for k in ("stars", "weighted_sfr", "sfr")}
    if hist0 is not None:
        st["sfr_histories"] = hist0.copy()
    return st


def _deposit_gpu(step, D, hist0, gal_list, bhs, device):
    """construct_baryon_grids through the API for snapshots 0, 1, ...; the
    grids after each snapshot as numpy arrays."""
    import torch

    st = _deposit_state(D, hist0)
    if device:
        st = {k: torch.from_numpy(v).cuda() for k, v in st.items()}
    outs = []
    for s, (gal, bh) in enumerate(zip(gal_list, bhs)):
        g = {GAL_API[k]: np.ascontiguousarray(v) for k, v in gal.items()}
        if device:
            g = {k: torch.from_numpy(v).cuda() for k, v in g.items()}
        step.construct_baryon_grids(s, g, st, *bh)
        if device:
            torch.cuda.synchronize()
        outs.append({k: (v.cpu().numpy() if device else v.copy()) for k, v in st.items()})
    return outs


def _deposit_oracle(orc, D, hist0, gal_list, bhs):
    st = _deposit_state(D, hist0)
    outs = []
    for s, (gal, bh) in enumerate(zip(gal_list, bhs)):
        orc.construct_baryon_grids(s, gal, st, bh)
        outs.append({k: v.copy() for k, v in st.items()})
    return outs


def _within_one_ulp(a, b):
    """Equal, or one float32 rounding apart (CUDA's pow against glibc's)."""
    return bool(np.all((a == b) | (np.abs(a - b) <= np.spacing(np.maximum(np.abs(a), np.abs(b))))))


def _mvir_gpu(step, z, sm, J, zi, device):
    import torch

    if device:
        out = torch.zeros(J.shape, dtype=torch.float32, device="cuda")
        step.calculate_Mvir_crit(z, sm, torch.from_numpy(J).cuda(), torch.from_numpy(zi).cuda(), out)
        torch.cuda.synchronize()
        return out.cpu().numpy()
    out = np.zeros_like(J)
    step.calculate_Mvir_crit(z, sm, J, zi, out)
    return out


@pytest.mark.parametrize("device", [False, True])
def test_gpu_deposit_and_Mvir_crit_match_reference_fixture(device):
    """The reference's own deposit (two snapshots: without, then with BH
    feedback; the SFR history shift included) bit for bit, and its
    Mvir_crit grid within one float ulp."""
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_golden import DEPOSIT_BH, DEPOSIT_CASE, MVIR_SM

    from meraxes_gb300.api import ReionGridStep

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "deposit16.npz"))
    name, kind, D, over = DEPOSIT_CASE
    w = Case(name, kind, D, over, fesc=0.01).workload()
    step = ReionGridStep(w.params, w.redshifts)
    assert step.n_sfr_histories == d["sfr_histories_init"].shape[0]
    gal_list = [{k: d[f"gal{s}/{k}"] for k in GAL_API} for s in range(len(DEPOSIT_BH))]
    outs = _deposit_gpu(step, D, d["sfr_histories_init"], gal_list, DEPOSIT_BH, device)
    for s in range(len(DEPOSIT_BH)):
        for k in DEPOSIT_GRIDS:
            assert np.array_equal(outs[s][k], d[f"out{s}/{k}"]), (s, k)
    got = _mvir_gpu(step, 10.0, MVIR_SM, d["J_21_at_ionization"], d["z_at_ionization"], device)
    ref = d["Mvir_crit"]
    assert np.array_equal(got > 0, ref > 0) and _within_one_ulp(got, ref)


@pytest.mark.parametrize("D,n,base,clustered",
                         [(64, 400000, "evolve_512", True), (48, 60000, "plain_64", False)])
def test_gpu_deposit_matches_oracle(D, n, base, clustered, tables_dir):
    """Against the oracle at larger sizes; `clustered` puts 400k galaxies in
    1/64 of the box (about 100 per occupied cell: long float sums in galaxy
    order)."""
    from cases import galaxies
    from meraxes_gb300.api import ReionGridStep
    from oracle import OracleBackend

    w = Case("dep", base, D, {"reion_efficiency": 3000.0}, fesc=0.01).workload()
    orc = OracleBackend(w.params, w.redshifts, tables_dir)
    step = ReionGridStep(w.params, w.redshifts)
    assert step.n_sfr_histories == orc.n_sfr_histories
    spin = bool(w.params.flag_spin_temp)
    npad = D * D * 2 * (D // 2 + 1)
    hist0 = (np.random.default_rng(5).random((orc.n_sfr_histories, npad)).astype(np.float32) if spin else None)
    gal_list = []
    for s in range(2):
        g = galaxies(D, w.params.box_size, n, 40 + s)
        if clustered:
            g["pos"] = np.ascontiguousarray((g["pos"] * np.float32(0.25)).astype(np.float32))
        gal_list.append(g)
    bhs = ((1, 1e-5, 1.57), (0, 0.0, 0.0))
    want = _deposit_oracle(orc, D, hist0, gal_list, bhs)
    for device in (False, True):
        got = _deposit_gpu(step, D, hist0, gal_list, bhs, device)
        for s in range(2):
            for k in want[s]:
                assert np.array_equal(got[s][k], want[s][k]), (device, s, k)
    occupied = (want[0]["stars"] > 0).sum()
    assert occupied > (1000 if clustered else 10000)
    rng = np.random.default_rng(7)
    J = (10.0 ** rng.normal(-1, 0.5, (D,) * 3)).astype(np.float32)
    zi = np.where(rng.random((D,) * 3) < 0.5, rng.uniform(8.0, 15.0, (D,) * 3), -1.0).astype(np.float32)
    sm = (0.049, 0.17, -2.1, 2.0, 2.5)
    ref = orc.calculate_Mvir_crit(9.0, sm, J, zi)
    for device in (False, True):
        got = _mvir_gpu(step, 9.0, sm, J, zi, device)
        assert np.array_equal(got > 0, ref > 0) and _within_one_ulp(got, ref), device


def test_gpu_deposit_edge_cases():
    """No galaxies, only dead galaxies (Type 3), and a galaxy below the box:
    empty grids with the history shifted; MX_EINVAL for the last, after which
    the context still works."""
    from meraxes_gb300._lib import MxError
    from meraxes_gb300.api import ReionGridStep

    D = 16
    w = Case("dep", "evolve_512", D, {}, fesc=0.01).workload()
    step = ReionGridStep(w.params, w.redshifts)
    nh = step.n_sfr_histories
    assert nh >= 2
    npad = D * D * 2 * (D // 2 + 1)
    hist0 = np.random.default_rng(3).random((nh, npad)).astype(np.float32)
    empty = {"pos": np.zeros((0, 3), np.float32), "type": np.zeros(0, np.int32),
             "fesc_gsm": np.zeros(0), "gross_sm": np.zeros(0)}
    dead = {"pos": np.full((100, 3), 10.0, np.float32), "type": np.full(100, 3, np.int32),
            "fesc_gsm": np.ones(100), "gross_sm": np.ones(100)}
    for gal in (empty, dead):
        for device in (False, True):
            out = _deposit_gpu(step, D, hist0, [gal], [(0, 0.0, 0.0)], device)[0]
            for k in ("stars", "weighted_sfr", "sfr"):
                assert not out[k].any(), (k, device)
            h = out["sfr_histories"]
            assert np.array_equal(h[1:], hist0[:-1])
            cells = h[0].reshape(D, D, -1)
            assert not cells[:, :, :D].any()
            assert np.array_equal(cells[:, :, D:], hist0[0].reshape(D, D, -1)[:, :, D:])
    below = {"pos": np.array([[-w.params.box_size / D, 1.0, 1.0]], np.float32), "type": np.zeros(1, np.int32),
             "fesc_gsm": np.ones(1), "gross_sm": np.ones(1)}
    with pytest.raises(MxError) as e:
        _deposit_gpu(step, D, hist0, [below], [(0, 0.0, 0.0)], False)
    assert e.value.code == -1
    ok = {"pos": np.array([[1.0, 1.0, 1.0]], np.float32), "type": np.zeros(1, np.int32),
          "fesc_gsm": np.ones(1), "gross_sm": np.ones(1)}
    out = _deposit_gpu(step, D, hist0, [ok], [(0, 0.0, 0.0)], False)[0]
    assert out["stars"].sum() == np.float32(1.0)


# The autotuner budgets the threshold z-pass's registers for 2 or 3 resident
# blocks per SM (MX_ZPASS_BLOCKS fixes it); both give the same grids.
@pytest.mark.parametrize("name,D", [("full24", 64), ("evolve16", 32)])
def test_zpass_register_budgets_give_identical_results(name, D, monkeypatch):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    runs = []
    for b in ("2", "3"):
        monkeypatch.setenv("MX_ZPASS_BLOCKS", b)
        step = ReionGridStep(w.params, w.redshifts)
        assert step.zpass_blocks() == int(b)
        gen = syn.FieldGenerator(w)
        st = initial(w, step.n_sfr_histories)
        glob = []
        for s in w.snapshots:
            st.update(gen.inputs(s, step.n_sfr_histories))
            glob.append(step.step(s, st))
        runs.append((st, glob))
        step.close()
    (sa, ga), (sb, gb) = runs
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        assert a["volume_weighted_global_xH"] == b["volume_weighted_global_xH"]
    monkeypatch.delenv("MX_ZPASS_BLOCKS")
    tuned = ReionGridStep(w.params, w.redshifts)
    assert tuned.zpass_blocks() in (2, 3)
    tuned.close()
