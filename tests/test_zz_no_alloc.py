"""mx_brightness_temperature_noalloc against the context entry point (GB300).

The no-allocation entry point keeps its reduction scratch in a fixed device
array inside the library.  Two calls in a row must both agree with
mx_ComputeBrightnessTemperatureBox_device: the delta_T box per cell within
1e-6 relative, and the volume average within 1e-12 relative (the two
reductions sum the same doubles in different fixed orders).  Grid sizes whose
cell count is not a multiple of a block's 16384 cells (24^3: one partly
filled block; 100^3: 62 blocks, the last partly filled) exercise the early
exit of the last block and the last-block reduction.  One case also runs on
the reference's own final grids of the full24 fixture.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, params, z, deltax, xH, TS, out, mean, torch):
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mx_brightness_temperature_noalloc(
        ctypes.byref(params), z, deltax.data_ptr(), xH.data_ptr(), TS.data_ptr() if TS is not None else None,
        out.data_ptr(), mean.data_ptr(), stream, err, len(err))
    return rc, err.value.decode()


@pytest.mark.parametrize("D", [24, 64, 100])
@pytest.mark.parametrize("spin", [1, 0])
def test_noalloc_matches_context_entry_point_twice(spin, D):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meraxes_gb300 import _lib
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.params import ReionParams

    p = ReionParams(grid_dim=D, box_size=100.0, flag_spin_temp=spin, flag_21cm=1)
    zz = [10.5, 10.0]
    ctx_step = ReionGridStep(p, zz)
    rng = np.random.default_rng(7)
    H = D // 2 + 1
    dev = torch.device("cuda:0")
    deltax = torch.from_numpy(rng.normal(0, 0.5, (D, D, 2 * H)).astype(np.float32)).to(dev)
    xH = torch.from_numpy(rng.uniform(0, 1, (D, D, D)).astype(np.float32)).to(dev)
    TS = torch.from_numpy(rng.uniform(5, 300, (D, D, D)).astype(np.float32)).to(dev)
    ref = torch.zeros((D, D, D), dtype=torch.float32, device=dev)
    g = ctx_step.ComputeBrightnessTemperatureBox(1, {"deltax": deltax, "xH": xH, "TS_box": TS, "delta_T": ref})
    torch.cuda.synchronize()

    lib = _lib.load()
    cp = p.to_ctypes()
    for _ in range(2):
        out = torch.full((D, D, D), float("nan"), dtype=torch.float32, device=dev)
        mean = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        rc, msg = _noalloc(lib, cp, zz[1], deltax, xH, TS if spin else None, out, mean, torch)
        assert rc == 0, msg
        torch.cuda.synchronize()
        a = ref.cpu().numpy().astype(np.float64)
        b = out.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(a - b) <= 1e-6 * np.abs(a) + 1e-30)
        m = float(mean.cpu()[0])
        assert abs(m - g["volume_ave_Tb"]) <= 1e-12 * abs(g["volume_ave_Tb"])
    ctx_step.close()


def test_noalloc_matches_reference_fixture():
    """delta_T of the reference's own run (tests/golden/full24.npz: spin
    temperature, no peculiar velocities) recomputed from its final deltax, xH
    and TS_box: per cell within the 1e-4 relative tolerance of delta_T, the
    volume average within 1e-6 relative."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cases import CASES
    from meraxes_gb300 import _lib
    from test_oracle_golden import golden_inputs, load_golden

    d, meta = load_golden("full24")
    init, per, out = golden_inputs(d, meta)
    w = CASES["full24"].workload()
    p = w.params
    assert p.flag_spin_temp and p.flag_pecvel == 0
    s = meta["snapshots"][-1]
    dev = torch.device("cuda:0")
    deltax = torch.from_numpy(np.ascontiguousarray(per[s]["deltax"])).to(dev)
    xH = torch.from_numpy(np.ascontiguousarray(out["xH"])).to(dev)
    TS = torch.from_numpy(np.ascontiguousarray(out["TS_box"])).to(dev)
    D = p.grid_dim
    lib = _lib.load()
    cp = p.to_ctypes()
    for _ in range(2):
        res = torch.full((D, D, D), float("nan"), dtype=torch.float32, device=dev)
        mean = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        rc, msg = _noalloc(lib, cp, meta["redshifts"][s], deltax, xH, TS, res, mean, torch)
        assert rc == 0, msg
        torch.cuda.synchronize()
        a = out["delta_T"].reshape(D, D, D).astype(np.float64)
        b = res.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(a - b) <= 1e-4 * np.abs(a) + 1e-30)
        want = meta["globals"][-1]["volume_ave_Tb"]
        assert abs(float(mean.cpu()[0]) - want) <= 1e-6 * abs(want)


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meraxes_gb300 import _lib
    from meraxes_gb300.params import ReionParams

    lib = _lib.load()
    cp = ReionParams(grid_dim=1024, flag_spin_temp=0).to_ctypes()
    err = ctypes.create_string_buffer(256)
    rc = lib.mx_brightness_temperature_noalloc(ctypes.byref(cp), 10.0, 16, 16, None, 16, 16, None, err, len(err))
    assert rc == -1
    assert b"at most 134217728 cells" in err.value
