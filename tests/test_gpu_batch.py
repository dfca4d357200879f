"""The batch of independent boxes (meraxes_gb300/batch.py) and the native
executor (mx_batch_run, mx_batch_run_graph): boxes of several sizes (powers of
two, and 24^3 / 48^3 on the factor-3 transforms) give the same results, bit
for bit, as each box run alone."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_batch_matches_single_box_runs():
    from meraxes_gb300.batch import BatchRunner, uneven_batch

    insts = uneven_batch(2, (32, 48))
    runner = BatchRunner(insts, max_workers_per_size=2)
    plan = runner.make_plan()
    assert set(plan) == {32, 48}
    out = runner.run()
    assert len(out["results"]) == 4
    for inst, res in zip(insts, out["results"]):
        alone = BatchRunner([inst], max_workers_per_size=1).run()["results"][0]
        assert res == alone, (inst, res, alone)
        assert res["loss"] > 0 and res["dL_dLX"] != 0 and res["dL_dfesc"] != 0


def _native_items(specs):
    """Batch items for run_batch: (case name, grid size, L_X) -> params,
    redshifts, first snapshot and host grids of that case."""
    import dataclasses

    from cases import CASES, Case, initial
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep

    items = []
    for name, D, lx in specs:
        c = CASES[name]
        w = Case(name, c.base, D, c.overrides, c.fesc, c.snapshots).workload()
        p = w.params
        if lx is not None:
            p = dataclasses.replace(p, lx_gal=lx)
        n_hist = ReionGridStep(p, w.redshifts).n_sfr_histories
        st = initial(w, n_hist)
        s = w.snapshots[0]
        st.update(syn.FieldGenerator(w).inputs(s, n_hist))
        items.append({"params": p, "redshifts": w.redshifts, "snapshot": s, "grids": st})
    return items


def test_native_batch_matches_single_box_runs():
    """mx_batch_run: boxes of two sizes and two X-ray luminosities on 3
    workers (contexts reused across the luminosities) give each box's grids
    and globals bit for bit as ReionGridStep.step of that box alone."""
    import numpy as np

    from meraxes_gb300.api import ReionGridStep, run_batch

    specs = [("full24", 32, 1e40), ("full24", 48, 1e40), ("full24", 32, 3e40), ("full24", 48, 3e40),
             ("plain32_tophat", 64, None)]
    items = _native_items(specs)
    alone = []
    for it in items:
        g = {k: v.copy() for k, v in it["grids"].items()}
        step = ReionGridStep(it["params"], it["redshifts"])
        glob = step.step(it["snapshot"], g)
        step.close()
        alone.append((g, glob))
    outs = run_batch(items, max_workers=3)
    for it, out, (g, glob) in zip(items, outs, alone):
        for k in g:
            assert np.array_equal(it["grids"][k], g[k]), k
        for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb"):
            assert out[k] == glob[k], k


def test_native_batch_reports_failed_items():
    """A bad item fails alone: its status is reported, the others run."""
    from meraxes_gb300 import _lib
    from meraxes_gb300.api import run_batch

    items = _native_items([("plain32_tophat", 32, None), ("plain32_tophat", 32, None)])
    items[1]["snapshot"] = 999  # beyond the redshift list
    with pytest.raises(_lib.MxError) as e:
        run_batch(items, max_workers=2)
    assert e.value.code == -1 and "item 1" in str(e.value)


def test_native_batch_object_reuses_contexts_across_runs():
    """A Batch object keeps its workers' contexts between runs: a second run
    on fresh copies of the inputs gives the same grids as the first."""
    import numpy as np

    from meraxes_gb300.api import Batch

    items = _native_items([("full24", 32, 1e40), ("full24", 32, 2e40), ("plain32_tophat", 48, None)])
    fresh = [{k: v.copy() for k, v in it["grids"].items()} for it in items]
    b = Batch(max_workers=2)
    first = b.run(items)
    grids_first = [{k: v.copy() for k, v in it["grids"].items()} for it in items]
    for it, f in zip(items, fresh):
        it["grids"] = {k: v.copy() for k, v in f.items()}
    second = b.run(items)
    b.close()
    assert first == second
    for it, g in zip(items, grids_first):
        for k in g:
            assert np.array_equal(it["grids"][k], g[k]), k


def _pinned(grids):
    """Copies of the grids in page-locked host memory (what the batch graph's
    copy nodes need)."""
    import torch

    return {k: torch.from_numpy(v).pin_memory().numpy() for k, v in grids.items()}


def test_batch_graph_matches_single_box_runs():
    """mx_batch_run_graph: boxes of three sizes (a power of two, and 24^3 and
    48^3 on the factor-3 transforms) and two X-ray luminosities stepped in
    one CUDA graph launch give each box's grids and globals bit for bit as
    ReionGridStep.step of that box alone, on a first run (contexts created)
    and a second (contexts reused)."""
    import numpy as np

    from meraxes_gb300.api import Batch, ReionGridStep

    specs = [("full24", 32, 1e40), ("full24", 48, 1e40), ("full24", 24, 3e40), ("full24", 48, 3e40),
             ("plain32_tophat", 64, None), ("evolve16", 32, None)]
    items = _native_items(specs)
    fresh = [{k: v.copy() for k, v in it["grids"].items()} for it in items]
    alone = []
    for it in items:
        g = {k: v.copy() for k, v in it["grids"].items()}
        step = ReionGridStep(it["params"], it["redshifts"])
        glob = step.step(it["snapshot"], g)
        step.close()
        alone.append((g, glob))
    b = Batch(max_workers=2)
    for run in range(2):
        for it, f in zip(items, fresh):
            it["grids"] = _pinned(f)
        outs = b.run(items, graph=True)
        for it, out, (g, glob) in zip(items, outs, alone):
            for k in g:
                assert np.array_equal(it["grids"][k], g[k]), (run, k)
            for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb", "x_e_ave"):
                assert out[k] == glob[k], (run, k)
            assert out["gpu_launches"] > 0
    b.close()


def test_batch_graph_rejects_pageable_grids():
    from meraxes_gb300 import _lib
    from meraxes_gb300.api import Batch

    items = _native_items([("plain32_tophat", 32, None)])
    b = Batch(max_workers=1)
    with pytest.raises(_lib.MxError) as e:
        b.run(items, graph=True)
    b.close()
    assert e.value.code == -1 and "page-locked" in str(e.value)
