"""The give-up path of the bounded pipeline waits (GB300).

Every wait of a kernel on its own bulk or tensor copies (the z-pass ring of
the transforms, the shell ring of the evolve kernels) gives up after a poll
limit, sets an error bit, waits with the full limit for the block's copies
still in flight and returns; the host then reports MX_ECUDA.  Here the
consumers' limit is lowered to one poll (MX_WAIT_POLL_LIMIT, read when a
context is created), so that the first wait on a copy that has not landed
yet gives up.  Nothing faults: every copy is valid and is waited for before
its block exits.  A context created afterwards with the default limit runs
the same step and gives the same grids as one that never saw the error.
"""
import numpy as np
import pytest

from cases import CASES, Case, OUTPUT_GRIDS, initial

pytestmark = pytest.mark.gpu


def _case():
    c = CASES["full24"]
    return Case("wait_limit", c.base, 32, c.overrides, c.fesc).workload()


def _run(w):
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    step = ReionGridStep(w.params, w.redshifts)
    s = w.snapshots[0]
    st = initial(w, step.n_sfr_histories)
    st.update(syn.FieldGenerator(w).inputs(s, step.n_sfr_histories))
    try:
        return st, step.step(s, st)
    finally:
        step.close()


def test_pipeline_wait_gives_up_and_reports(monkeypatch):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meraxes_gb300 import _lib

    w = _case()
    ref, gref = _run(w)
    monkeypatch.setenv("MX_WAIT_POLL_LIMIT", "1")
    with pytest.raises(_lib.MxError) as e:
        _run(w)
    assert e.value.code == -3  # MX_ECUDA
    assert "timed out" in str(e.value)
    monkeypatch.delenv("MX_WAIT_POLL_LIMIT")
    st, g = _run(w)
    for k in OUTPUT_GRIDS:
        if k in ref:
            assert np.array_equal(ref[k], st[k]), k
    assert g["volume_weighted_global_xH"] == gref["volume_weighted_global_xH"]
