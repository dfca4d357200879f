"""mx_brightness_temperature_noalloc against the context entry point (GB300).

The no-allocation entry point keeps its reduction scratch in a fixed device
array inside the library.  Two calls in a row must both agree with
mx_ComputeBrightnessTemperatureBox_device: the delta_T box per cell within
1e-6 relative, and the volume average within 1e-12 relative (the two
reductions sum the same doubles in different fixed orders).
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


@pytest.mark.parametrize("spin", [1, 0])
def test_noalloc_matches_context_entry_point_twice(spin):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meraxes_gb300 import _lib
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.params import ReionParams

    D = 64
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
