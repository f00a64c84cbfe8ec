"""Chains on thread-block clusters: every CTA of a chain's cluster takes a
share of the framework atoms, guests and k-vectors.  Only the order of the
final sums changes, so an FP64 chain on a cluster still follows the oracle
move by move, and FP32 chains on clusters of 1, 2 and 4 CTAs make the same
moves with the same energies to FP32-sum accuracy.
"""
import numpy as np
import pytest

from fastmc_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL = 1e-9


def close(a, b, rel, scale=1e-6):
    return abs(a - b) <= rel * max(abs(a), abs(b), scale)


@pytest.fixture(scope="module")
def small(inputs_dir):
    return inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "cl_small")


@pytest.mark.parametrize("csize", [2, 4])
def test_cluster_fp64_chain_matches_oracle(fmc_lib, oracle_lib, small, csize):
    n = 400
    o = oracle_lib.Oracle(small)
    o.seed(77)
    o.create_molecules(1, 10)
    ref = o.run(n)
    sysm = fmc_lib.System.load(small)
    b = fmc_lib.Batch([sysm], [{"seed": 77}], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=64)
    b.set_cluster([csize])
    assert b.cluster() == [csize]
    b.set_log(n)
    b.run(n)
    got = b.log(0, n)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert (g.move, g.choice, g.overlap, g.accepted) == (r.move, r.choice, r.overlap, r.accepted), i
        if not r.overlap:
            assert close(g.estep, r.estep, REL), (i, g.estep, r.estep)
    st = b.stats()[0]
    assert st.nummols == o.nummols(o.locguest(1))
    assert st.status == 0


def test_cluster_fp32_matches_single_cta(fmc_lib, inputs_dir):
    """Two systems, chains on clusters of 1, 2 and 4 CTAs in one batch
    (separate launches in one graph): same moves, same energies."""
    d1 = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "cl_a")
    d2 = inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=40), "cl_b")
    systems = [fmc_lib.System.load(d1), fmc_lib.System.load(d2)]
    specs = [{"system": s, "seed": 11 + i} for i, s in enumerate([0, 0, 1, 1])]
    n = 300
    logs = {}
    for sizes in ([1, 1], [2, 4], [4, 2]):
        b = fmc_lib.Batch(systems, specs, precision=fmc_lib.FMC_PREC_FP32, guest_capacity=256)
        b.set_cluster(sizes)
        b.set_log(n)
        b.run(n)
        assert all(s.status == 0 for s in b.stats())
        logs[tuple(sizes)] = [b.log(c, n) for c in range(len(specs))]
    base = logs[(1, 1)]
    for key, lg in logs.items():
        for c in range(len(specs)):
            for i, (g, r) in enumerate(zip(lg[c], base[c])):
                assert (g.move, g.choice, g.overlap) == (r.move, r.choice, r.overlap), (key, c, i)
                if r.overlap:
                    continue
                assert close(g.estep, r.estep, 1e-6, scale=1.0), (key, c, i, g.estep, r.estep)
                if g.accepted != r.accepted:
                    break  # a decision at the threshold; the chains part here


def test_autotune_leaves_chain_state(fmc_lib, inputs_dir):
    """The autotuner's trial cycles start from a copy of the chains' state,
    which is restored: the chains then run exactly like a fresh batch with
    the chosen cluster sizes."""
    d1 = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "cl_a")
    d2 = inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=40), "cl_b")
    systems = [fmc_lib.System.load(d1), fmc_lib.System.load(d2)]
    specs = [{"system": s, "seed": 21 + i} for i, s in enumerate([0, 1, 1])]
    a = fmc_lib.Batch(systems, specs, precision=fmc_lib.FMC_PREC_FP32, guest_capacity=256)
    sizes = a.autotune(64)
    assert len(sizes) == 2 and all(1 <= v <= 8 for v in sizes)
    assert a.cluster() == sizes
    per_chain = a.chain_cluster()
    assert len(per_chain) == len(specs) and all(1 <= v <= 8 for v in per_chain)
    assert sizes == [max(v for v, s in zip(per_chain, specs) if s["system"] == i) for i in range(2)]
    b = fmc_lib.Batch(systems, specs, precision=fmc_lib.FMC_PREC_FP32, guest_capacity=256)
    b.set_chain_cluster(per_chain)
    for x in (a, b):
        x.set_log(150)
        x.run(150)
    for c in range(len(specs)):
        la, lb = a.log(c, 150), b.log(c, 150)
        assert len(la) == len(lb) == 150
        for i, (u, v) in enumerate(zip(la, lb)):
            assert (u.move, u.choice, u.overlap, u.accepted, u.estep) == \
                   (v.move, v.choice, v.overlap, v.accepted, v.estep), (c, i)


def test_resident_guests_match_global(fmc_lib, inputs_dir):
    """FP32 batches keep the guests in shared memory when capacity x sites
    fits (3072 sites); a larger capacity keeps them in global memory.  Both
    visit the molecules in the same order, so the moves and energies are
    identical, and so are the coordinates written back."""
    d = inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=40), "cl_b")
    sysm = fmc_lib.System.load(d)
    specs = [{"seed": 31}, {"seed": 32}]
    n = 300
    out = []
    for cap in (256, 2048):  # 768 sites: resident; 6144 sites: global
        b = fmc_lib.Batch([sysm], specs, precision=fmc_lib.FMC_PREC_FP32, guest_capacity=cap)
        b.set_log(n)
        b.run(n // 2)
        b.run(n - n // 2)  # two launches: write-back and reload in between
        out.append((b, [b.log(c, n) for c in range(2)], b.stats()))
    (b1, l1, s1), (b2, l2, s2) = out
    for c in range(2):
        assert s1[c].nummols == s2[c].nummols and s1[c].energy == s2[c].energy
        for i, (u, v) in enumerate(zip(l1[c], l2[c])):
            assert (u.move, u.choice, u.overlap, u.accepted, u.estep) == \
                   (v.move, v.choice, v.overlap, v.accepted, v.estep), (c, i)
        x1, n1 = b1.coords(c)
        x2, n2 = b2.coords(c)
        assert n1 == n2 and np.array_equal(x1[:9 * n1], x2[:9 * n2])  # 3 sites x 3


def test_checkpoint_resume_exact(fmc_lib, inputs_dir, tmp_path):
    """A batch resumed from a checkpoint continues bit for bit like the
    batch that wrote it."""
    d1 = inputs_dir(syn.small_test_spec(seed=4, kmax=6, pressure_bar=5.0, create=10), "cl_a")
    d2 = inputs_dir(syn.small_test_spec(seed=5, kmax=8, ntile=3, pressure_bar=5.0, create=40), "cl_b")
    systems = [fmc_lib.System.load(d1), fmc_lib.System.load(d2)]
    specs = [{"system": s, "seed": 41 + i} for i, s in enumerate([0, 1, 1])]
    path = str(tmp_path / "chains.ckpt")
    for prec in (fmc_lib.FMC_PREC_FP32, fmc_lib.FMC_PREC_FP64):
        a = fmc_lib.Batch(systems, specs, precision=prec, guest_capacity=256)
        a.set_cluster([1, 2])
        a.run(150)
        a.save(path)
        a.set_log(150)
        a.run(150)
        b = fmc_lib.Batch(systems, specs, precision=prec, guest_capacity=256)
        b.set_cluster([1, 2])
        b.load(path)
        b.set_log(150)
        b.run(150)
        sa, sb = a.stats(), b.stats()
        for c in range(len(specs)):
            assert (sa[c].nummols, sa[c].energy, sa[c].moves) == (sb[c].nummols, sb[c].energy, sb[c].moves)
            la, lb = a.log(c, 150), b.log(c, 150)
            for i, (u, v) in enumerate(zip(la, lb)):
                assert (u.move, u.choice, u.accepted, u.estep) == (v.move, v.choice, v.accepted, v.estep), (c, i)
    other = fmc_lib.Batch(systems, specs[:2], precision=fmc_lib.FMC_PREC_FP64, guest_capacity=256)
    with pytest.raises(fmc_lib.FmcError):
        other.load(path)
