"""CIPSI selection with the second-order energy on the device
(qpgpu_select_pt2) against the oracle's restatement of
plugins/Full_CI_ZMQ/selection.irp.f (qpo_select_pt2).

The oracle is pinned by tests/test_selection_oracle.py against dense sums on
the full-CI golden spaces.  Here, the device must match it on the same
wave functions, on seeded sets with N_int = 1 and N_int = 2, and with
several generators whose externals overlap:
* pt2 of every state within 1e-12 relative;
* the number of external determinants with a non-zero numerator exactly;
* the buffer values (ascending) within 1e-12;
* the buffer determinants the same.  Where values tie within 1e-12, the
  comparison is of the set of determinants.
The generator / selector counts follow generators.irp.f:3-22 and
selectors.irp.f:3-25.
"""
import numpy as np
import pytest

from golden_util import load
from oracle import Oracle
from quantum_package_gb300 import ezfio
from quantum_package_gb300 import generate as G
from quantum_package_gb300 import select as S


def test_generator_and_selector_counts():
    contrib = np.array([0.9, 0.05, 0.03, 0.015, 0.004, 0.001])
    assert S.n_det_generators(contrib, 0.99) == 4
    assert S.n_det_generators(contrib, 0.5) == 1
    assert S.n_det_selectors(contrib, 4, 0.999, 0.99) == 5
    assert S.n_det_selectors(contrib, 4, 0.5, 0.99) == 4
    assert S.n_det_selectors(contrib, 1, 0.5, 1.0) == len(contrib)


def _subspace_wave_function(H, n_psi, n_st):
    idx = np.argsort(np.diag(H), kind="stable")[:n_psi]
    w, V = np.linalg.eigh(H[np.ix_(idx, idx)])
    coef = V[:, :n_st]  # (n_psi, n_st)
    order = ezfio.sorted_order(coef)
    return idx[order], np.ascontiguousarray(coef[order].T), w[:n_st]


def _compare(dev, ora, rel=1e-12):
    pt2, bd, bv, n_ext = dev
    pt2o, bdo, bvo, n_exto = ora
    scale = max(np.abs(pt2o).max(), 1e-3)
    np.testing.assert_allclose(pt2, pt2o, rtol=0, atol=rel * scale)
    assert n_ext == n_exto
    assert len(bv) == len(bvo)
    np.testing.assert_allclose(bv, bvo, rtol=0, atol=rel * max(abs(bvo[0]) if len(bvo) else 1.0, 1e-3))
    # determinants: equal where the values are separated, as sets within tie groups
    k = len(bv)
    i = 0
    while i < k:
        j = i + 1
        while j < k and abs(bvo[j] - bvo[i]) <= rel * max(abs(bvo[i]), 1e-3):
            j += 1
        got = {bytes(x.tobytes()) for x in bd[i:j]}
        want = {bytes(x.tobytes()) for x in bdo[i:j]}
        if j < k:
            assert got == want, (i, j)
        else:  # the last tie group may be cut by the buffer size
            assert len(got) == j - i
        i = j


@pytest.mark.gpu
@pytest.mark.parametrize("name,n_psi,n_st,thresholds,buf", [
    ("fci_s2", 12, 1, (0.99, 0.999), 50),
    ("fci_s2", 20, 2, (0.9, 0.99), 40),
    ("fci_cs", 16, 1, (1.0, 1.0), 30),
    ("fci_cs", 30, 3, (0.95, 0.999), 100),
])
def test_select_matches_oracle_on_golden_spaces(name, n_psi, n_st, thresholds, buf):
    from quantum_package_gb300.sigma import Wavefunction
    d = load(name)
    idx, coef, e0 = _subspace_wave_function(d["H"], n_psi, n_st)
    contrib = ezfio.average_norm_contrib(coef.T)  # coef rows are already in sorted order
    tg, ts = thresholds
    n_gen = S.n_det_generators(contrib, tg)
    n_sel = S.n_det_selectors(contrib, n_gen, ts, tg)
    dets = d["dets"][idx]
    o = Oracle(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri, dets)
    wf = Wavefunction(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri, dets)
    _compare(wf.select_pt2(coef, e0, n_gen, n_sel, buf), o.select_pt2(coef, e0, n_gen, n_sel, buf))
    wf.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n_mo,ne,n_psi,n_st,n_gen", [
    (30, 5, 160, 2, 12),   # N_int = 1
    (70, 4, 90, 1, 6),     # N_int = 2, orbitals on both sides of the word boundary
])
def test_select_matches_oracle_on_seeded_sets(n_mo, ne, n_psi, n_st, n_gen):
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=n_psi, n_mo=n_mo, n_alpha=ne, n_beta=ne)
    o0 = Oracle.from_problem(p)
    H, _ = o0.dense(with_s2=False)
    idx, coef, e0 = _subspace_wave_function(H, n_psi, n_st)
    dets = p.dets[idx]
    o = Oracle(p.n_mo, ne, ne, p.ints.h, p.ints.eri, dets)
    wf = Wavefunction(p.n_mo, ne, ne, p.ints.h, p.ints.eri, dets)
    n_sel = n_psi // 2
    _compare(wf.select_pt2(coef, e0, n_gen, n_sel, 200), o.select_pt2(coef, e0, n_gen, n_sel, 200))
    # buffer size 0: the same pt2, no entries
    pt2, bd, bv, n_ext = wf.select_pt2(coef, e0, n_gen, n_sel, 0)
    assert len(bv) == 0 and n_ext > 0
    wf.close()


@pytest.mark.gpu
def test_select_end_to_end_and_refusals():
    from quantum_package_gb300 import QPGPUError
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=120, n_mo=24, n_alpha=4, n_beta=4)
    H, _ = Oracle.from_problem(p).dense(with_s2=False)
    w, V = np.linalg.eigh(H)
    coefs = V[:, :2]
    make = lambda dd: Wavefunction(p.n_mo, 4, 4, p.ints.h, p.ints.eri, dd)
    r = S.select(make, p.dets, coefs, w[:2], 64, threshold_generators=0.9, threshold_selectors=0.99)
    o = Oracle(p.n_mo, 4, 4, p.ints.h, p.ints.eri, p.dets[r["order"]])
    ref = o.select_pt2(np.ascontiguousarray(coefs[r["order"]].T), w[:2], r["n_gen"], r["n_sel"], 64)
    _compare((r["pt2"], r["dets"], r["vals"], r["n_ext"]), ref)
    assert np.all(r["pt2"] < 0.0)
    wf = make(p.dets)
    with pytest.raises(QPGPUError):
        wf.select_pt2(np.ascontiguousarray(coefs.T), w[:2], 5, 4, 10)
    wf.close()


@pytest.mark.gpu
def test_select_many_generators_per_item():
    # 10,000 generators: work items of late generators are reached by more
    # earlier generators than the kernel's shared list holds (2,048), so the
    # bans read the global list; the result must still equal the oracle's
    from quantum_package_gb300.sigma import Wavefunction
    n_mo, ne, nd = 10, 3, 10000
    ints = G.make_integrals(n_mo, 29)
    full = G.full_ci_dets(n_mo, ne, ne)
    rng = np.random.default_rng(2)
    dets = full[np.sort(rng.choice(len(full), nd, replace=False))]
    c = rng.normal(size=(1, nd)) * np.exp(-np.arange(nd) / 5000.0)
    # the overflow is reached: count, for the last generator's first alpha-beta
    # hole pair, the earlier generators that lack at most 2 of its electrons
    g = dets[-1]
    occ_a = [o for o in range(n_mo) if (int(g[0, 0]) >> o) & 1]
    occ_b = [o for o in range(n_mo) if (int(g[1, 0]) >> o) & 1]
    mask = g.copy()
    mask[0, 0] = np.uint64(int(mask[0, 0]) & ~(1 << occ_a[0]))
    mask[1, 0] = np.uint64(int(mask[1, 0]) & ~(1 << occ_b[0]))
    lack = [bin(int(mask[0, 0]) & ~int(d[0, 0])).count("1") + bin(int(mask[1, 0]) & ~int(d[1, 0])).count("1")
            for d in dets[:-1]]
    assert sum(1 for k in lack if k <= 2) > 2048
    o = Oracle(n_mo, ne, ne, ints.h, ints.eri, dets)
    wf = Wavefunction(n_mo, ne, ne, ints.h, ints.eri, dets)
    e0 = np.array([-10.0])  # below every H_aa of this space: all denominators of one sign
    _compare(wf.select_pt2(c, e0, nd, nd, 300), o.select_pt2(c, e0, nd, nd, 300))
    wf.close()
