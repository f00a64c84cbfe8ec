"""The hand-written adjoint of the guest-framework energy: central finite
differences (h = 1e-4) of the energy against the analytic gradients, an
independent FP64 numpy reference of the Lennard-Jones part (charges scaled
to zero), torch.autograd through the Function, and charge-scale linearity."""
import math

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def setup(fmc_lib, inputs_dir):
    from fastmc_gb300.adjoint import Adjoint
    spec = syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=6)
    d = inputs_dir(spec, "adj_small")
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 3}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=16)
    x, n = b.coords(0)
    assert n == 6
    xyz = torch.tensor(x[:9 * n].reshape(n, 3, 3), dtype=torch.float64, device="cuda")
    adj = Adjoint(sysm)
    return spec, adj, xyz


def test_adjoint_finite_differences(setup):
    _, adj, xyz = setup
    p0 = adj.base_params()
    assert p0.shape == (4, 3) and np.all(p0[:, 2] == 1.0)
    e0, gx, gp = adj.evaluate(xyz, p0)
    h = 1e-4
    rng = np.random.default_rng(1)
    for _ in range(8):  # coordinates
        m, s, d = int(rng.integers(6)), int(rng.integers(3)), int(rng.integers(3))
        xp, xm = xyz.clone(), xyz.clone()
        xp[m, s, d] += h
        xm[m, s, d] -= h
        fd = (adj.evaluate(xp, p0)[0] - adj.evaluate(xm, p0)[0]) / (2 * h)
        an = float(gx[m, s, d])
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1.0), (m, s, d, fd, an)
    for t in range(4):  # every parameter of every framework type
        for q in range(3):
            pp, pm = p0.copy(), p0.copy()
            pp[t, q] += h
            pm[t, q] -= h
            fd = (adj.evaluate(xyz, pp)[0] - adj.evaluate(xyz, pm)[0]) / (2 * h)
            assert abs(fd - gp[t, q]) <= 1e-5 * max(abs(gp[t, q]), 1.0), (t, q, fd, gp[t, q])


def test_adjoint_lj_numpy_reference(setup):
    """With every charge scale at zero, E is the Lennard-Jones sum alone;
    an FP64 numpy restatement (minimum image, cutoff, Lorentz-Berthelot)
    gives E, dE/dxyz and dE/d(eps, sigma)."""
    spec, adj, xyz = setup
    uc = syn.make_unit_cell(spec.fw_seed)
    n, L = spec.ntile, spec.box
    offs = np.array([[i, j, k] for i in range(n) for j in range(n) for k in range(n)], float) * syn.UNIT_CELL
    fw = (uc.xyz[None, :, :] + offs[:, None, :]).reshape(-1, 3)
    # the adjoint numbers framework types in their order of first appearance
    order = list(dict.fromkeys(int(t) for t in uc.types))
    ft = np.tile(np.array([order.index(int(t)) for t in uc.types]), n ** 3)
    eps_t, sig_t = uc.eps[order], uc.sigma[order]
    p0 = adj.base_params()
    assert np.allclose(p0[:, 0], eps_t) and np.allclose(p0[:, 1], sig_t)
    p = p0.copy()
    p[:, 2] = 0.0
    e, gx, gp = adj.evaluate(xyz, p)
    site = [syn.GUEST_LJ["Cg"], syn.GUEST_LJ["Og"], syn.GUEST_LJ["Og"]]
    rc2 = spec.cutoff ** 2
    x = xyz.cpu().numpy()
    e_ref, g_ref, gp_ref = 0.0, np.zeros_like(x), np.zeros((4, 2))
    for m in range(x.shape[0]):
        for s in range(3):
            ea, sa = site[s]
            dv = x[m, s] - fw
            dv -= L * np.rint(dv / L)
            r2 = (dv ** 2).sum(axis=1)
            sel = r2 < rc2
            r = np.sqrt(r2[sel])
            t = ft[sel]
            eps = np.sqrt(ea * eps_t[t])
            sig = 0.5 * (sa + sig_t[t])
            sr6 = (sig / r) ** 6
            elj = 4 * eps * sr6 * (sr6 - 1)
            e_ref += elj.sum()
            dedr = 4 * eps * (6 * sr6 - 12 * sr6 ** 2) / r
            g_ref[m, s] = (dedr[:, None] * dv[sel] / r[:, None]).sum(axis=0)
            np.add.at(gp_ref[:, 0], t, elj / (2 * eps_t[t]))
            np.add.at(gp_ref[:, 1], t, 0.5 * (24 * eps / sig) * (2 * sr6 ** 2 - sr6))
    assert math.isclose(e, e_ref, rel_tol=1e-10, abs_tol=1e-10)
    assert np.allclose(gx.cpu().numpy(), g_ref, rtol=1e-9, atol=1e-9)
    assert np.allclose(gp[:, :2], gp_ref, rtol=1e-9, atol=1e-9)


def test_adjoint_charge_linearity(setup):
    """E is linear in each charge scale, with slope dE/dlambda_t."""
    _, adj, xyz = setup
    p0 = adj.base_params()
    e1, _, gp = adj.evaluate(xyz, p0)
    pz = p0.copy()
    pz[:, 2] = 0.0
    e0 = adj.evaluate(xyz, pz)[0]
    assert math.isclose(e1 - e0, gp[:, 2].sum(), rel_tol=1e-10, abs_tol=1e-9)
    p2 = p0.copy()
    p2[1, 2] = 3.0
    e2 = adj.evaluate(xyz, p2)[0]
    assert math.isclose(e2 - e1, 2.0 * gp[1, 2], rel_tol=1e-10, abs_tol=1e-9)


def test_adjoint_autograd(setup):
    from fastmc_gb300.adjoint import guest_framework_energy
    _, adj, xyz = setup
    x = xyz[:2].clone().requires_grad_(True)
    p = torch.tensor(adj.base_params(), dtype=torch.float64, requires_grad=True)
    e = guest_framework_energy(adj, x, p)
    e.backward()
    _, gx, gp = adj.evaluate(x.detach(), p.detach().numpy())
    assert torch.allclose(x.grad, gx) and np.allclose(p.grad.numpy(), gp)
    assert torch.autograd.gradcheck(lambda a, b: guest_framework_energy(adj, a, b),
                                    (x.detach().clone().requires_grad_(True),
                                     p.detach().clone().requires_grad_(True)),
                                    eps=1e-6, atol=1e-4, rtol=1e-4)
