"""The whole step captured as one CUDA graph (GB300).

mx_set_step_graph makes mx_step_device capture ComputeTs -> find_HII_bubbles
-> 21cm box into one graph: the reads back are deferred until the graph has
completed and ComputeTs's frequency tables are built by a host node on a side
branch while the shells are smoothed.  The grids and globals must equal those
of the uncaptured step bit for bit, snapshot after snapshot, on both transform
paths, and per-kernel profiling must see the kernels inside the graph.
"""
import numpy as np
import pytest

from cases import CASES, Case, OUTPUT_GRIDS, initial

pytestmark = pytest.mark.gpu

GLOBALS = ("volume_weighted_global_xH", "mass_weighted_global_xH", "volume_weighted_global_J_21", "volume_ave_TS",
           "volume_ave_TK", "volume_ave_xe", "volume_ave_Tb", "x_e_ave", "collapse_fraction", "volume_ave_J_alpha",
           "volume_ave_Xheat", "n_radii", "gpu_launches")


def _evolve(w, graph, profile=False):
    import torch

    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    step = ReionGridStep(w.params, w.redshifts)
    step.set_graph(graph)
    if profile:
        step.profile(True)
    gen = syn.FieldGenerator(w)
    st = initial(w, step.n_sfr_histories)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in st.items()}
    glob = []
    for s in w.snapshots:
        for k, v in gen.inputs(s, step.n_sfr_histories).items():
            dev[k] = torch.from_numpy(v.copy()).cuda()
        glob.append(step.step(s, dev))
    torch.cuda.synchronize()
    stats = step.profile_read() if profile else None
    step.close()
    return {k: v.cpu().numpy() for k, v in dev.items()}, glob, stats


@pytest.mark.parametrize("transform", ["fused", "cufft"])
@pytest.mark.parametrize("name,D", [("evolve16", 32), ("full24", 64), ("plain32_tophat", 64)])
def test_step_graph_matches_uncaptured_step(name, D, transform, monkeypatch):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    monkeypatch.setenv("MX_TRANSFORM", transform)
    c = CASES[name]
    w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
    sa, ga, _ = _evolve(w, False)
    sb, gb, _ = _evolve(w, True)
    for k in OUTPUT_GRIDS:
        if k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    for a, b in zip(ga, gb):
        for k in GLOBALS:
            assert a[k] == b[k], (k, a[k], b[k])


def test_step_graph_profiles_its_kernels():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = CASES["full24"]
    w = Case("graph_prof", c.base, 64, c.overrides, c.fesc).workload()
    _, ga, pa = _evolve(w, False, profile=True)
    _, gb, pb = _evolve(w, True, profile=True)
    assert set(pa) == set(pb)
    for k in pa:
        assert pa[k][0] == pb[k][0], k  # launches
        assert pb[k][1] > 0, k          # event time inside the graph
