"""The differentiable form (torch.autograd.Function over the device adjoint)
on a 5,000-atom GBSW globule: its gradients against the host adjoint of the
same context, against the FP64 oracle's analytic adjoint, and against FP64
central finite differences of the oracle energy on 200 randomly chosen
entries (h = 1e-4 A for positions, 1e-5 for charges, radii and
coefficients)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from openmmcustomgbintegralforce_gb300.autograd import GBEnergy, gb_energy  # noqa: E402
from openmmcustomgbintegralforce_gb300.globule import make_globule  # noqa: E402
from openmmcustomgbintegralforce_gb300.spec import GBModel  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def case():
    g = make_globule(5000, seed=41)
    m = GBModel.charmm_gbsw()
    mod = GBEnergy(m, g.n)
    dev = torch.device("cuda:0")
    x = torch.tensor(g.positions, dtype=torch.float64, device=dev, requires_grad=True)
    q = torch.tensor(g.charge, dtype=torch.float64, device=dev, requires_grad=True)
    R = torch.tensor(g.radius, dtype=torch.float64, device=dev, requires_grad=True)
    a = torch.tensor([m.alpha0, m.alpha1], dtype=torch.float64, device=dev, requires_grad=True)
    E = mod(x, q, R, a)
    E.backward()
    grads = {"forces": -x.grad.cpu().numpy(), "dEdq": q.grad.cpu().numpy(), "dEdR": R.grad.cpu().numpy(),
             "dEdalpha": a.grad.cpu().numpy()}
    return g, m, mod, float(E.item()), grads


def test_matches_host_adjoint(case):
    g, _, mod, E, grads = case
    host = mod.gb.adjoint(g.positions)
    assert E == pytest.approx(host["energy"], rel=1e-12)
    for k in ("forces", "dEdq", "dEdR", "dEdalpha"):
        assert np.allclose(grads[k], host[k], rtol=1e-12, atol=1e-9), k


def test_against_oracle_adjoint(case):
    g, m, _, E, grads = case
    ref = O.Oracle(m).energy_forces(g.positions, g.charge, g.radius, adjoint=True)
    assert abs(E / ref["energy"] - 1) < 2e-5
    assert rel_rms(grads["forces"], ref["forces"]) < 1e-4
    assert rel_rms(grads["dEdq"], ref["dEdq"]) < 1e-4
    assert rel_rms(grads["dEdR"], ref["dEdR"]) < 1e-4
    assert np.abs(grads["dEdalpha"] / ref["dEdalpha"] - 1).max() < 1e-4


def test_against_fp64_finite_differences(case):
    """200 randomly chosen entries: 120 position components, 39 charges, 39
    radii and the two coefficients."""
    g, m, _, _, grads = case
    orc = O.Oracle(m)
    rng = np.random.default_rng(9)

    def E(pos=g.positions, q=g.charge, R=g.radius, model=None):
        o = orc if model is None else O.Oracle(model)
        return o.energy_forces(pos, q, R)["energy"]

    def close(fd, an, scale, what):
        assert abs(fd - an) <= 2e-3 * scale + 2e-3 * abs(an), f"{what}: fd {fd} vs gpu {an}"

    F = grads["forces"]
    fs = float(np.sqrt((F ** 2).mean()))
    h = 1e-5  # nm (1e-4 A)
    checked = 0
    for flat in rng.choice(3 * g.n, size=120, replace=False):
        i, d = int(flat) // 3, int(flat) % 3
        xp, xm = g.positions.copy(), g.positions.copy()
        xp[i, d] += h
        xm[i, d] -= h
        close(-(E(pos=xp) - E(pos=xm)) / (2 * h), F[i, d], fs, f"F[{i},{d}]")
        checked += 1
    h = 1e-5
    for key, which in (("dEdq", "q"), ("dEdR", "R")):
        an = grads[key]
        sc = float(np.sqrt((an ** 2).mean()))
        for i in rng.choice(g.n, size=39, replace=False):
            i = int(i)
            p = (g.charge if which == "q" else g.radius).astype(np.float64).copy()
            p[i] += h
            ep = E(q=p) if which == "q" else E(R=p)
            p[i] -= 2 * h
            em = E(q=p) if which == "q" else E(R=p)
            close((ep - em) / (2 * h), an[i], sc, f"{key}[{i}]")
            checked += 1
    for k, name in enumerate(("alpha0", "alpha1")):
        base = getattr(m, name)
        ep = E(model=m.replace(**{name: base + h}))
        em = E(model=m.replace(**{name: base - h}))
        close((ep - em) / (2 * h), grads["dEdalpha"][k], abs(grads["dEdalpha"][k]), name)
        checked += 1
    assert checked == 200


def test_fitting_step_moves_charges(case):
    """One gradient step on the charges through the functional form."""
    g, m, mod, E0, _ = case
    dev = torch.device("cuda:0")
    x = torch.tensor(g.positions, dtype=torch.float64, device=dev)
    q = torch.tensor(g.charge, dtype=torch.float64, device=dev, requires_grad=True)
    R = torch.tensor(g.radius, dtype=torch.float64, device=dev)
    a = torch.tensor([m.alpha0, m.alpha1], dtype=torch.float64, device=dev)
    E = gb_energy(x, q, R, a, mod.gb)
    (gq,) = torch.autograd.grad(E, q)
    with torch.no_grad():
        q2 = q - 1e-4 * gq / gq.norm()
    E2 = gb_energy(x, q2, R, a, mod.gb)
    assert float(E2.detach()) < float(E.detach())
