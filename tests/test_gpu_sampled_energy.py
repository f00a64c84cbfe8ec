"""The batched adjoint of the energy the chains sample
(fmc_adjoint_eval_batch): tabulated real-space terms against the framework
and the other molecules, the reciprocal sum without each molecule's own
term, the guest-framework Lennard-Jones tail.  Checked against the oracle's
move energies (differences between trial positions and between deletions,
where the terms that depend only on the molecule count cancel), central
finite differences, FP32 against FP64, batch against single snapshots, and
the reweighting estimator on a device chain's own snapshots."""
import math

import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _system(fmc_lib, tmp_path, box_tiles, create):
    spec = syn.small_test_spec(seed=4, kmax=6, ntile=box_tiles, pressure_bar=5.0, create=create)
    d = str(tmp_path / f"se{box_tiles}")
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=48))
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 3}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=256)
    x, n = b.coords(0)
    assert n == create
    return d, sysm, x[:9 * n].reshape(n, 3, 3)


def _free(o, n, seed, box):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(50000):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        xyz = np.outer([0.0, 1.16, -1.16], ax) + rng.uniform(0, box, 3)
        if not o.insertion_energy(1, xyz)["overlap"]:
            out.append(xyz)
            if len(out) == n:
                break
    return out


@pytest.mark.parametrize("tiles", [2, 4])
def test_energy_differences_match_oracle(fmc_lib, oracle_lib, tmp_path, tiles):
    """U(S + A) - U(S + B) equals the oracle's insertion estep(A) -
    estep(B), and U(S - m1) - U(S - m2) its deletion estep(m2) - estep(m1)
    (FP64 to 1e-9 of the energies involved), on a 25.6 A box (every
    framework atom scanned) and a 51.2 A box (neighbour cells)."""
    from fastmc_gb300.adjoint import Adjoint
    d, sysm, mols = _system(fmc_lib, tmp_path, tiles, 12)
    adj = Adjoint(sysm)
    p0 = adj.base_params()
    o = oracle_lib.Oracle(d)
    for m in mols:
        o.apply_move(1, 1, 0, m, True)
    box = 12.8 * tiles
    pos = _free(o, 6, 5, box)
    assert len(pos) == 6
    snaps = [np.concatenate([mols, p[None]]) for p in pos]
    x = torch.tensor(np.concatenate(snaps), dtype=torch.float64, device="cuda")
    e, _, _ = adj.evaluate_batch(x, [13] * 6, p0, "fp64")
    ref = np.array([o.insertion_energy(1, p)["estep"] for p in pos])
    for i in range(1, 6):
        scale = max(abs(ref[i]), abs(ref[0]), 1.0)
        assert abs((e[i] - e[0]) - (ref[i] - ref[0])) <= 1e-9 * scale, (i, e[i] - e[0], ref[i] - ref[0])
    # deletions of each molecule
    dels = [np.delete(mols, k, axis=0) for k in range(12)]
    x = torch.tensor(np.concatenate(dels), dtype=torch.float64, device="cuda")
    e, _, _ = adj.evaluate_batch(x, [11] * 12, p0, "fp64")
    ref = np.array([o.deletion_energy(1, k + 1)["estep"] for k in range(12)])
    for k in range(1, 12):
        scale = max(abs(ref[k]), abs(ref[0]), 1.0)
        assert abs((e[k] - e[0]) - (ref[0] - ref[k])) <= 1e-9 * scale, (k, e[k] - e[0], ref[0] - ref[k])


@pytest.fixture(scope="module")
def batch(fmc_lib, tmp_path_factory):
    from fastmc_gb300.adjoint import Adjoint
    d, sysm, mols = _system(fmc_lib, tmp_path_factory.mktemp("se"), 4, 20)
    adj = Adjoint(sysm)
    # three snapshots: 20, 12 and 7 molecules
    sets = [mols, mols[3:15], mols[10:17]]
    nm = [len(s) for s in sets]
    x = torch.tensor(np.concatenate(sets), dtype=torch.float64, device="cuda")
    return adj, x, nm


def test_finite_differences(batch):
    """Central differences (h = 1e-4) of the FP64 energies against the
    adjoint's site and parameter gradients."""
    adj, x, nm = batch
    p0 = adj.base_params()
    e, gx, gp = adj.evaluate_batch(x, nm, p0, "fp64")
    snap_of = np.repeat(np.arange(len(nm)), nm)
    # h small against the table spacing: the 3-point interpolation's slope
    # steps at the table's nodes, and a stencil across one differs by the step
    h = 1e-5
    rng = np.random.default_rng(2)
    gxf = gx.cpu().numpy().astype(np.float64)
    for _ in range(10):
        m, s, dd = int(rng.integers(x.shape[0])), int(rng.integers(3)), int(rng.integers(3))
        xp, xm = x.clone(), x.clone()
        xp[m, s, dd] += h
        xm[m, s, dd] -= h
        q = snap_of[m]
        fd = (adj.evaluate_batch(xp, nm, p0, "fp64")[0][q] - adj.evaluate_batch(xm, nm, p0, "fp64")[0][q]) / (2 * h)
        an = gxf[m, s, dd]
        assert abs(fd - an) <= 2e-5 * max(abs(an), 1.0), (m, s, dd, fd, an)
    for t in range(p0.shape[0]):
        for q in range(3):
            hp = 1e-5 * max(1.0, abs(p0[t, q]))
            pp, pm = p0.copy(), p0.copy()
            pp[t, q] += hp
            pm[t, q] -= hp
            fd = (adj.evaluate_batch(x, nm, pp, "fp64")[0] - adj.evaluate_batch(x, nm, pm, "fp64")[0]) / (2 * hp)
            assert np.allclose(fd, gp[:, t, q], rtol=1e-5, atol=1e-6), (t, q, fd, gp[:, t, q])


def test_fp32_against_fp64_and_single_snapshots(batch):
    """FP32 pair terms and phases (FP64 sums) against the FP64 reference
    gradient; a batch equals its snapshots evaluated one at a time."""
    adj, x, nm = batch
    p0 = adj.base_params()
    e64, g64, p64 = adj.evaluate_batch(x, nm, p0, "fp64")
    e32, g32, p32 = adj.evaluate_batch(x, nm, p0, "fp32")
    assert np.allclose(e32, e64, rtol=2e-6, atol=1e-4)
    g64n, g32n = g64.cpu().numpy(), g32.cpu().numpy()
    assert np.abs(g32n - g64n).max() <= 1e-4 * np.abs(g64n).max()
    assert np.allclose(p32, p64, rtol=1e-5, atol=1e-4 * np.abs(p64).max())
    o = 0
    for q, n in enumerate(nm):
        e1, g1, pp1 = adj.evaluate_batch(x[o:o + n], [n], p0, "fp64")
        assert math.isclose(e1[0], e64[q], rel_tol=1e-12, abs_tol=1e-9)
        assert torch.allclose(g1, g64[o:o + n])
        assert np.allclose(pp1[0], p64[q], rtol=1e-10, atol=1e-10 * np.abs(p64[q]).max())
        o += n
    # empty snapshots: nothing but zeros, also between others
    e0, g0, pz = adj.evaluate_batch(x[:0], [0, 0], p0, "fp64")
    assert np.all(e0 == 0.0) and np.all(pz == 0.0) and g0.numel() == 0
    e2, g2, p2 = adj.evaluate_batch(x[:nm[0]], [0, nm[0], 0], p0, "fp64")
    assert e2[0] == 0.0 and e2[2] == 0.0 and math.isclose(e2[1], e64[0], rel_tol=1e-12, abs_tol=1e-9)
    assert torch.allclose(g2, g64[:nm[0]])


def test_autograd_over_a_batch(batch):
    from fastmc_gb300.adjoint import sampled_energy
    adj, x, nm = batch
    xx = x.clone().requires_grad_(True)
    p = torch.tensor(adj.base_params(), dtype=torch.float64, requires_grad=True)
    e = sampled_energy(adj, xx, nm, p, "fp64")
    w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64, device=e.device)
    (w * e).sum().backward()
    _, gx, gp = adj.evaluate_batch(x, nm, p.detach().numpy(), "fp64")
    snap = torch.as_tensor(np.repeat(np.arange(3), nm), device=x.device)
    wc = w.to(x.device)
    assert torch.allclose(xx.grad, wc[snap].view(-1, 1, 1) * gx.to(torch.float64))
    assert np.allclose(p.grad.cpu().numpy(), (w.cpu().numpy()[:, None, None] * gp).sum(axis=0))


def test_uptake_sensitivity_from_chain_snapshots(fmc_lib, tmp_path):
    """The reweighting estimator on a device chain's own snapshots: d<N>/dtheta
    from -beta (<N dU/dtheta> - <N><dU/dtheta>) with the adjoint's dU/dtheta
    equals the slope of the reweighted <N> (weights exp(-beta (U(theta +-
    h) - U(theta))) of the same snapshots) for every parameter."""
    from fastmc_gb300.adjoint import Adjoint, uptake_sensitivity
    spec = syn.small_test_spec(seed=4, kmax=6, ntile=2, pressure_bar=5.0, create=10,
                               move_mix=(("insert", 0.3), ("delete", 0.3), ("displace", 0.4)))
    spec.overlap = 1.5
    d = str(tmp_path / "rw")
    syn.write_inputs(d, spec, uc=syn.make_unit_cell(4, natoms=48))
    sysm = fmc_lib.System.load(d)
    b = fmc_lib.Batch([sysm], [{"seed": 8}], precision=fmc_lib.FMC_PREC_FP32, guest_capacity=256)
    snaps, ns = [], []
    for _ in range(120):
        b.run(50)
        x, n = b.coords(0)
        snaps.append(x[:9 * n].reshape(n, 3, 3))
        ns.append(n)
    assert np.std(ns) > 0.5
    adj = Adjoint(sysm)
    p0 = adj.base_params()
    x = torch.tensor(np.concatenate(snaps), dtype=torch.float64, device="cuda")
    e0, _, gp = adj.evaluate_batch(x, ns, p0, "fp64")
    beta = 1.0 / (1.9872041e-3 * 293.0)
    sens = uptake_sensitivity(ns, gp.reshape(len(ns), -1), beta).reshape(p0.shape)
    n = np.asarray(ns, dtype=float)
    for t in range(p0.shape[0]):
        for q in range(3):
            h = 1e-4 * max(1.0, abs(p0[t, q]))
            avg = []
            for sgn in (1, -1):
                p = p0.copy()
                p[t, q] += sgn * h
                e = adj.evaluate_batch(x, ns, p, "fp64")[0]
                w = np.exp(-beta * (e - e0) - np.max(-beta * (e - e0)))
                avg.append((w * n).sum() / w.sum())
            fd = (avg[0] - avg[1]) / (2 * h)
            assert abs(fd - sens[t, q]) <= 1e-3 * max(abs(sens[t, q]), 1e-3), (t, q, fd, sens[t, q])
