"""Gradients of the 21 cm power-spectrum loss (autograd.py, mx_adjoint_device)
against central finite differences of the CUDA forward, relative step 1e-3.

The loss is the squared error of the delta_T power spectrum in 20 log-spaced
bins against a target made at L_X = 2e40; gradients w.r.t. L_X, E0, the escape
fraction (a multiplier of the stars grid find_HII_bubbles reads) and the SFR
grid (along a random direction).  The backward holds the ionisation flags
fixed; the finite differences see the forward as it is.  Tolerances: 1% for
the parameters, 2% for the SFR directions (the finite difference of a 1e-3
step carries the FP32 noise of the forward).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_STEP = 1e-3


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.autograd import log_bins
    from meraxes_gb300.params import workload

    w = workload("diff_256", 48)
    step = ReionGridStep(w.params, w.redshifts)
    gen = syn.FieldGenerator(w)
    st = syn.initial_state(w.params, w.redshifts[0])
    st.update(gen.inputs(1, step.n_sfr_histories))
    D = w.params.grid_dim
    st.setdefault("delta_T", np.zeros((D, D, D), np.float32))
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in st.items()}
    edges = log_bins(step, 20)
    return w, step, dev, edges


def _loss(case, sfr, stars, lx, e0, target):
    import torch

    from meraxes_gb300.autograd import DeltaT21, PSLoss21

    w, step, dev, edges = case
    state = {k: v for k, v in dev.items() if k not in ("sfr", "stars")}
    dT = DeltaT21.apply(sfr, stars, lx, e0, step, 1, state)
    return PSLoss21.apply(dT, step, edges, target)


def test_adjoint_matches_finite_differences(case):
    import torch

    w, step, dev, edges = case
    p = w.params
    lx0, e00 = p.lx_gal, p.nu_xray_gal_threshold
    sfr0, stars0 = dev["sfr"], dev["stars"]
    # target: the power spectrum at L_X = 2e40
    state = {k: v for k, v in dev.items() if k not in ("sfr", "stars")}
    from meraxes_gb300.autograd import DeltaT21

    dT_t = DeltaT21.apply(sfr0, stars0, torch.tensor(2e40, dtype=torch.float64), torch.tensor(e00), step, 1, state)
    _, target, _ = step.ps_loss(dT_t, edges, [0.0] * 20, grad=False)
    assert sum(target) > 0

    sfr = sfr0.clone().requires_grad_(True)
    fesc = torch.tensor(1.0, dtype=torch.float32, device="cuda", requires_grad=True)
    lx = torch.tensor(lx0, dtype=torch.float64, requires_grad=True)
    e0 = torch.tensor(e00, dtype=torch.float64, requires_grad=True)
    L = _loss(case, sfr, stars0 * fesc, lx, e0, target)
    L.backward()
    assert L.item() > 0

    def fd(f, x0):
        h = REL_STEP * x0
        return (f(x0 + h) - f(x0 - h)) / (2 * h)

    def L_of(**kw):
        a = dict(sfr=sfr0, stars=stars0, lx=torch.tensor(lx0, dtype=torch.float64),
                 e0=torch.tensor(e00, dtype=torch.float64))
        a.update(kw)
        with torch.no_grad():
            return _loss(case, a["sfr"], a["stars"], a["lx"], a["e0"], target).item()

    g_lx = fd(lambda x: L_of(lx=torch.tensor(x, dtype=torch.float64)), lx0)
    g_e0 = fd(lambda x: L_of(e0=torch.tensor(x, dtype=torch.float64)), e00)
    g_fesc = fd(lambda x: L_of(stars=stars0 * x), 1.0)
    # SFR directions: a uniform relative change, one confined to the half of
    # the padded array the SFR-history scalings act on, and a randomly
    # modulated one.  (A zero-mean random direction has a derivative below the
    # FP32 noise of the forward, about 1e-7 of the loss.)
    D = w.params.grid_dim
    half = torch.zeros_like(sfr0)
    half[: D // 2] = 1
    gen = torch.Generator(device="cuda").manual_seed(5)
    dirs = {"uniform": sfr0, "first_half": sfr0 * half,
            "modulated": sfr0 * (0.5 + torch.rand(sfr0.shape, generator=gen, device="cuda"))}
    checks = [("L_X", lx.grad.item(), g_lx, 0.01), ("E0", e0.grad.item(), g_e0, 0.01),
              ("fesc", fesc.grad.item(), g_fesc, 0.01)]
    for name, v in dirs.items():
        fdv = (L_of(sfr=sfr0 + REL_STEP * v) - L_of(sfr=sfr0 - REL_STEP * v)) / (2 * REL_STEP)
        checks.append(("sfr." + name, float((sfr.grad * v).sum()), fdv, 0.02))
    print("L", L.item())
    for name, a, f, tol in checks:
        print(f"{name:16s} adjoint {a: .6e} fd {f: .6e}")
    for name, a, f, tol in checks:
        assert abs(a - f) <= tol * abs(f), (name, a, f)


def ps_numpy(dT, p, edges):
    """P per bin of mx_ps_loss_device in numpy: f = dT V / N, the half
    spectrum in double, |k| per mode in the float32 operations of the CUDA
    binning."""
    D = dT.shape[0]
    box = p.box_size / p.hubble_h
    V = np.float32(box ** 3)
    dk = np.float32(2.0 * np.pi / box)
    f = dT.astype(np.float32) * np.float32(float(V) / D ** 3)
    X = np.fft.rfftn(f.astype(np.float64))
    n = np.arange(D)
    kc = np.where(n > D // 2, (n - D).astype(np.float32) * dk, n.astype(np.float32) * dk).astype(np.float32)
    kz = (np.arange(D // 2 + 1).astype(np.float32) * dk).astype(np.float32)
    kx2 = (kc * kc).astype(np.float32)
    kz2 = (kz * kz).astype(np.float32)
    k2 = (kx2[:, None, None] + kx2[None, :, None]).astype(np.float32)
    k2 = (k2 + kz2[None, None, :]).astype(np.float32)
    kmag = np.sqrt(k2).astype(np.float32)
    e = np.asarray(edges, np.float32)
    b = np.searchsorted(e, kmag, side="right") - 1  # bin b: e[b] <= k < e[b+1]
    k = kmag.astype(np.float64)
    pw = k ** 3 * np.abs(X) ** 2 / (2 * np.pi ** 2 * float(V))
    return [pw[b == i].sum() / max(int((b == i).sum()), 1) for i in range(len(e) - 1)]


def ps_loss_numpy(dT, p, edges, target):
    return sum((P - t) ** 2 for P, t in zip(ps_numpy(dT, p, edges), target))


def test_adjoint_matches_fp64_cpu_gradient(case, tables_dir):
    """Against central differences of the oracle (the C restatement, per-cell
    physics in double) with the loss in numpy, at 32^3."""
    import dataclasses

    import torch

    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.autograd import DeltaT21, PSLoss21, log_bins
    from meraxes_gb300.params import workload
    from oracle import OracleBackend

    w = workload("diff_256", 32)
    p = w.params
    gen = syn.FieldGenerator(w)
    step = ReionGridStep(p, w.redshifts)
    st0 = syn.initial_state(p, w.redshifts[0])
    st0.update(gen.inputs(1, step.n_sfr_histories))
    D = p.grid_dim
    st0.setdefault("delta_T", np.zeros((D, D, D), np.float32))
    edges = log_bins(step, 20)

    def oracle_dT(lx=p.lx_gal, e0=p.nu_xray_gal_threshold, fesc=1.0, sfr_scale=1.0):
        q = dataclasses.replace(p, lx_gal=lx, nu_xray_gal_threshold=e0)
        orc = OracleBackend(q, w.redshifts, tables_dir)
        st = {k: v.copy() for k, v in st0.items()}
        st["stars"] = (st["stars"] * np.float32(fesc)).astype(np.float32)
        st["sfr"] = (st["sfr"] * np.float32(sfr_scale)).astype(np.float32)
        orc.step(1, st)
        return st["delta_T"]

    target = ps_numpy(oracle_dT(lx=2e40), p, edges)
    assert sum(target) > 0

    # CUDA adjoint at the same inputs and target
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in st0.items()}
    state = {k: v for k, v in dev.items() if k not in ("sfr", "stars")}
    sfr = dev["sfr"].clone().requires_grad_(True)
    fesc = torch.tensor(1.0, device="cuda", requires_grad=True)
    lx = torch.tensor(p.lx_gal, dtype=torch.float64, requires_grad=True)
    e0 = torch.tensor(p.nu_xray_gal_threshold, dtype=torch.float64, requires_grad=True)
    L = PSLoss21.apply(DeltaT21.apply(sfr, dev["stars"] * fesc, lx, e0, step, 1, state), step, edges, target)
    L.backward()

    def fd(fn):
        return (fn(1 + REL_STEP) - fn(1 - REL_STEP)) / (2 * REL_STEP)

    L0 = ps_loss_numpy(oracle_dT(), p, edges, target)
    g_lx = fd(lambda s: ps_loss_numpy(oracle_dT(lx=p.lx_gal * s), p, edges, target)) / p.lx_gal
    g_e0 = fd(lambda s: ps_loss_numpy(oracle_dT(e0=p.nu_xray_gal_threshold * s), p, edges, target)) / \
        p.nu_xray_gal_threshold
    g_fesc = fd(lambda s: ps_loss_numpy(oracle_dT(fesc=s), p, edges, target))
    g_sfr = fd(lambda s: ps_loss_numpy(oracle_dT(sfr_scale=s), p, edges, target))
    a_sfr = float((sfr.grad * dev["sfr"]).sum())
    checks = [("L_X", lx.grad.item(), g_lx), ("E0", e0.grad.item(), g_e0), ("fesc", fesc.grad.item(), g_fesc),
              ("sfr.uniform", a_sfr, g_sfr)]
    print("loss CUDA", L.item(), "oracle", L0)
    for name, a, f in checks:
        print(f"{name:12s} CUDA adjoint {a: .6e}  oracle FD {f: .6e}")
    assert abs(L.item() - L0) <= 0.02 * L0
    for name, a, f in checks:
        assert abs(a - f) <= 0.05 * abs(f), (name, a, f)
