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
