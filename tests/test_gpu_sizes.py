"""The fused transforms at the grid sizes the benchmark runs (GB300).

The kernels of the fused inverse transforms are compiled per grid size:
k_fft_x_filter<D, threads>, k_fft_y<D, threads>,
k_fft_z_threshold<D, spin, recombinations> and k_fft_z_store<D>.  Here the
<256> builds run against the oracle (the full step of the 256^3 workload, and
two snapshots of the evolving workload at 256^3 with its own cell size); the
<512> builds run one snapshot of the 512^3 benchmark workload against the
oracle, through the captured device step the benchmark times, and against the
cuFFT path
(MX_TRANSFORM=cufft: cuFFT C2R with filter and threshold kernels that do not
depend on the grid size and are held to the oracle at small sizes).  At 512^3
find_HII_bubbles takes two radius batches and mx_step's threshold pass runs in
eight row slabs.  Every run's reported global means are also checked against
FP64 sums of the grids it returned (find_HII_bubbles.c:451-470,
ComputeTs.c:942-974, BrightnessTemperature.c:530-545).
"""
import os

import numpy as np
import pytest

from cases import OUTPUT_GRIDS
from compare import compare

pytestmark = pytest.mark.gpu

REION_EFF = 1.0 / 0.15714 * 4000.0 / (1.0 - 0.75 * 0.24)  # set_ReionEfficiency, reionization.c:181-210
MEAN_RTOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _real(a, D):
    a = np.asarray(a)
    if a.size == D ** 3:
        return a.reshape(D, D, D)
    return a.reshape(D, D, -1)[:, :, :D]


def check_means(st, glob, D, p):
    """Reported volume / mass averages against FP64 sums of the returned
    grids; returns the largest relative difference."""
    n = float(D) ** 3
    worst = 0.0

    def rel(a, b):
        return abs(a - b) / max(abs(b), 1e-300)

    xh = _real(st["xH"], D).astype(np.float64)
    want = {"volume_weighted_global_xH": xh.sum() / n}
    dom = 1.0 + _real(st["deltax"], D).astype(np.float64)
    want["mass_weighted_global_xH"] = (xh * dom).sum() / dom.sum()
    if p.uvb_flag and "J_21" in st:
        want["volume_weighted_global_J_21"] = _real(st["J_21"], D).astype(np.float64).sum() / n
    if p.flag_spin_temp:
        want["volume_ave_TS"] = _real(st["TS_box"], D).astype(np.float64).sum() / n
        want["volume_ave_TK"] = _real(st["Tk_box"], D).astype(np.float64).sum() / n
    if p.flag_21cm:
        want["volume_ave_Tb"] = _real(st["delta_T"], D).astype(np.float64).sum() / n
    for k, v in want.items():
        r = rel(glob[k], v)
        worst = max(worst, r)
        assert r <= MEAN_RTOL, f"{k}: reported {glob[k]!r}, FP64 sum of the grid {v!r} ({r:.2e})"
    return worst


def _workload(name, D, snapshots=None):
    from meraxes_gb300.params import workload

    w = workload(name, D)
    w.params.reion_efficiency = REION_EFF
    w.fesc = 0.01
    if snapshots is not None:
        w.snapshots = list(snapshots)
    return w


def _oracle_vs_gpu(w, tables_dir):
    """Runs w's snapshots on the oracle and through mx_step on the same
    inputs; compares every snapshot with the oracle's margins.  Each snapshot
    starts from the same state on both sides (the GPU's is replaced by the
    oracle's after each comparison): a cell whose decision flips near
    threshold changes its N_rec, z_at_ionization and x_e, and through the
    filters its neighbours' margins in the next snapshot, so margins hold
    only for a step on identical inputs."""
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep
    from oracle import OracleBackend

    orc = OracleBackend(w.params, w.redshifts, tables_dir)
    gpu = ReionGridStep(w.params, w.redshifts)
    assert gpu.n_sfr_histories == orc.n_sfr_histories
    gen = syn.FieldGenerator(w)
    sa = initial(w, orc.n_sfr_histories)
    sb = {k: v.copy() for k, v in sa.items()}
    reps = []
    for s in w.snapshots:
        inp = gen.inputs(s, orc.n_sfr_histories)
        sa.update({k: v.copy() for k, v in inp.items()})
        sb.update({k: v.copy() for k, v in inp.items()})
        ga = orc.step(s, sa)
        margin = orc.margin()
        gb = gpu.step(s, sb)
        assert gpu.last_launches > 0
        rep = {}
        compare(sa, sb, ga, gb, margin=margin, report=rep)
        rep["means_rel"] = check_means(sb, gb, w.params.grid_dim, w.params)
        reps.append(rep)
        sb = {k: v.copy() for k, v in sa.items()}
    gpu.close()
    orc.close()
    return reps


def test_full_step_256_matches_oracle(tables_dir):
    """The 256^3 full-step workload (L=100 Mpc/h, z=10, recombinations with
    clumping 3, 40 ComputeTs shells, delta_T) with the benchmark's ionising
    efficiency and escape fraction: the <256> transforms against the oracle."""
    w = _workload("full_256", 256)
    reps = _oracle_vs_gpu(w, tables_dir)
    print("full_256", reps)


def test_evolving_workload_at_256_matches_oracle(tables_dir):
    """Two consecutive snapshots of the evolving workload at 256^3 (its cell
    size, 41 radii): SFR-history reweighting and state carried between
    snapshots on the <256> transforms, against the oracle."""
    w = _workload("evolve_512", 256, snapshots=[9, 10])
    reps = _oracle_vs_gpu(w, tables_dir)
    print("evolve_512@256", reps)


def test_evolving_workload_512_matches_oracle(tables_dir):
    """One snapshot of the benchmark workload at its own size (512^3, z =
    10.26, 41 radii x 5 fields, 40 shells, delta_T) through the path the
    benchmark times: device grids, the step captured as one CUDA graph, the
    fused <512> transforms; against the oracle with its margins.  The oracle
    snapshot takes a few minutes on the host cores and about 60 GB of host
    memory."""
    import torch

    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep
    from oracle import OracleBackend

    w = _workload("evolve_512", 512, snapshots=[10])
    D = w.params.grid_dim
    orc = OracleBackend(w.params, w.redshifts, tables_dir)
    s = w.snapshots[0]
    sa = initial(w, orc.n_sfr_histories)
    sa.update(syn.FieldGenerator(w).inputs(s, orc.n_sfr_histories))
    sa.setdefault("delta_T", np.zeros((D, D, D), np.float32))
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in sa.items()}
    gpu = ReionGridStep(w.params, w.redshifts)
    gpu.set_graph(True)
    gb = gpu.step(s, dev)
    torch.cuda.synchronize()
    gpu.close()
    sb = {k: v.cpu().numpy() for k, v in dev.items()}
    del dev
    torch.cuda.empty_cache()
    ga = orc.step(s, sa)
    margin = orc.margin()
    orc.close()
    rep = {}
    compare(sa, sb, ga, gb, margin=margin, report=rep)
    rep["means_rel"] = check_means(sb, gb, D, w.params)
    print("evolve_512 vs oracle", rep)


def _run_512(transform, device, inputs, w, monkeypatch):
    from meraxes_gb300.api import ReionGridStep

    import torch

    if transform == "cufft":
        monkeypatch.setenv("MX_TRANSFORM", "cufft")
    else:
        monkeypatch.delenv("MX_TRANSFORM", raising=False)
    step = ReionGridStep(w.params, w.redshifts)
    s = w.snapshots[0]
    if device:
        st = {k: torch.from_numpy(v).cuda() for k, v in inputs.items()}
        g = step.step(s, st)
        torch.cuda.synchronize()
        out = {k: v.cpu().numpy() for k, v in st.items()}
        del st
    else:
        out = {k: v.copy() for k, v in inputs.items()}
        g = step.step(s, out)
    step.close()
    torch.cuda.empty_cache()
    return out, g


def test_evolving_workload_512_fused_matches_cufft(monkeypatch):
    """One snapshot of the 512^3 workload (z = 10.26, 41 radii x 5 fields, 40
    shells) on the fused <512> transforms, through mx_step (host grids: the
    remainder radius batch first, the last batch's threshold in eight row
    slabs) and through mx_step_device (remainder last), against the cuFFT
    path on the same inputs.  The two fused runs must agree bit for bit; the
    fused and cuFFT runs within the parity tolerances (without oracle
    margins: flags and r_bubble may differ in at most 1e-4 of the cells)."""
    from cases import initial
    from meraxes_gb300 import synthetic as syn

    from oracle import OracleBackend

    w = _workload("evolve_512", 512, snapshots=[10])
    D = w.params.grid_dim
    # the number of SFR-history slices (the oracle context allocates no grids)
    n_hist = OracleBackend(w.params, w.redshifts, syn.TABLES_DIR).n_sfr_histories
    inputs = initial(w, n_hist)
    inputs.update(syn.FieldGenerator(w).inputs(10, n_hist))
    inputs.setdefault("delta_T", np.zeros((D, D, D), np.float32))

    fused_host, g_host = _run_512("fused", False, inputs, w, monkeypatch)
    fused_dev, g_dev = _run_512("fused", True, inputs, w, monkeypatch)
    for k in OUTPUT_GRIDS:
        if k in fused_host:
            assert np.array_equal(fused_host[k], fused_dev[k]), k
    for k in ("volume_weighted_global_xH", "mass_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
        assert g_host[k] == g_dev[k], k
    del fused_dev
    plain, g_plain = _run_512("cufft", False, inputs, w, monkeypatch)
    rep = {}
    compare(plain, fused_host, g_plain, g_host, report=rep)
    rep["means_rel_fused"] = check_means(fused_host, g_host, D, w.params)
    rep["means_rel_cufft"] = check_means(plain, g_plain, D, w.params)
    assert g_host["n_radii"] == g_plain["n_radii"] == len(w.params.filter_radii())
    print("evolve_512 fused vs cufft", rep)
