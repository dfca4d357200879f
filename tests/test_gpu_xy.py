"""The x- and y-pass as one persistent kernel (k_fft_xy, the spectra between
the passes kept in L2) against the two separate passes (MX_XY_PASS=split):
every item of the persistent kernel runs the arithmetic of one block of the
separate passes, so every grid and global agrees bit for bit.  Covered: the
find_HII_bubbles batches (5 fields with recombinations and the spin
temperature) and the ComputeTs shell batches (one field), power-of-two grids
(128, 256) and grids with a factor 3 (96, 192; the 384-thread engine), one
radius batch and several (MX_MAX_BATCH_SPECTRA), and a wait limit short
enough that y items give up (the error is reported, the context stays
usable)."""
import numpy as np
import pytest

from cases import CASES, OUTPUT_GRIDS, Case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _run(w, monkeypatch, split, n_snap=None):
    from cases import initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    if split:
        monkeypatch.setenv("MX_XY_PASS", "split")
    else:
        monkeypatch.delenv("MX_XY_PASS", raising=False)
    step = ReionGridStep(w.params, w.redshifts)
    assert step.xy_fused() == (not split)
    gen = syn.FieldGenerator(w)
    st = initial(w, step.n_sfr_histories)
    glob = []
    for s in w.snapshots[:n_snap]:
        st.update(gen.inputs(s, step.n_sfr_histories))
        glob.append(step.step(s, st))
    step.close()
    return st, glob


@pytest.mark.parametrize("name,D,batch", [("full24", 128, None), ("full24", 96, None), ("evolve16", 192, 10),
                                          ("evolve16", 128, 10), ("full24", 256, 15)])
def test_xy_kernel_matches_separate_passes(name, D, batch, monkeypatch):
    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    if batch is not None:
        monkeypatch.setenv("MX_MAX_BATCH_SPECTRA", str(batch))
    n_snap = 2 if D >= 192 else None
    sa, ga = _run(w, monkeypatch, split=False, n_snap=n_snap)
    sb, gb = _run(w, monkeypatch, split=True, n_snap=n_snap)
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        for k in ("volume_weighted_global_xH", "mass_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
            if k in a:
                assert a[k] == b[k], k


def test_xy_kernel_wait_limit_reports_error(monkeypatch):
    """With a wait limit of one poll the y items that find their chunk
    unfinished give up: the step raises the pipeline-timeout error instead
    of returning wrong grids, and the next context (default limit) works."""
    from cases import initial
    from meraxes_gb300 import _lib
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    c = CASES["plain32_tophat"]
    w = Case("plain32_tophat", c.base, 256, c.overrides, c.fesc, c.snapshots).workload()
    monkeypatch.delenv("MX_XY_PASS", raising=False)
    monkeypatch.setenv("MX_WAIT_POLL_LIMIT", "1")
    step = ReionGridStep(w.params, w.redshifts)
    assert step.xy_fused()
    gen = syn.FieldGenerator(w)
    st = initial(w, step.n_sfr_histories)
    s = w.snapshots[0]
    st.update(gen.inputs(s, step.n_sfr_histories))
    with pytest.raises(_lib.MxError) as e:
        step.step(s, {k: v.copy() for k, v in st.items()})
    assert "timed out (x+y pass)" in str(e.value)
    step.close()
    monkeypatch.delenv("MX_WAIT_POLL_LIMIT")
    ok = ReionGridStep(w.params, w.redshifts)
    ok.step(s, {k: v.copy() for k, v in st.items()})
    ok.close()
