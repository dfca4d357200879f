"""The batch of independent boxes (meraxes_gb300/batch.py): boxes of two
sizes (a power of two on the fused transforms, 48^3 on cuFFT) run by
concurrent workers give the same losses and gradients, bit for bit, as each
box run alone."""
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
