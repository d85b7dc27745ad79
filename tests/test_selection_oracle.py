"""CIPSI selection with the second-order energy: the oracle's restatement of
plugins/Full_CI_ZMQ/selection.irp.f (oracle/qp_oracle.cpp, qpo_select_pt2)
against a dense evaluation on the full-CI golden spaces, whose Hamiltonian
comes from the second-quantisation evaluator (oracle/secondq.py, no Slater
rules).

The dense side takes a wave function Psi of the lowest-diagonal
determinants with its own eigenvectors and energies as E0, then, for every
determinant a of the full space outside Psi and within a double excitation
of a generator: v = c . H[selectors, a], H_aa from the golden diagonal, and
the reference's two-level contribution e = (sign(d) sqrt(d^2 + 4 v^2) - d) / 2
with d = E0 - H_aa (fill_buffer_double, selection.irp.f:582-645).  Bars:
pt2 and the buffer values within 1e-12 of the dense sums, every external
determinant counted once, generator / selector counts by the reference's
threshold rules (generators.irp.f:3-22, selectors.irp.f:3-25).
"""
import numpy as np
import pytest

from golden_util import load
from oracle import Oracle, n_generators, n_selectors, sort_by_weight


def _degree(a, b):
    return sum(bin(int(w)).count("1") for w in np.bitwise_xor(a, b).ravel()) // 2


def _wave_function(d, n_psi, n_st):
    H, dets = d["H"], d["dets"]
    idx = np.argsort(np.diag(H), kind="stable")[:n_psi]
    w, V = np.linalg.eigh(H[np.ix_(idx, idx)])
    coef = V[:, :n_st].T
    order, contrib = sort_by_weight(coef)
    return idx[order], coef[:, order], w[:n_st], contrib


def _dense(d, idx, coef, e0, n_gen, n_sel):
    H, dets = d["H"], d["dets"]
    inpsi = np.zeros(len(dets), bool)
    inpsi[idx] = True
    gens, sels = idx[:n_gen], idx[:n_sel]
    pt2 = np.zeros(len(e0))
    vals = []
    for a in range(len(dets)):
        if inpsi[a] or min(_degree(dets[a], dets[g]) for g in gens) > 2:
            continue
        v = coef[:, :n_sel] @ H[sels, a]
        if np.abs(v).sum() == 0.0:
            continue
        delta = e0 - H[a, a]
        tmp = np.sqrt(delta * delta + 4.0 * v * v)
        tmp = np.where(delta < 0.0, -tmp, tmp)
        e = 0.5 * (tmp - delta)
        pt2 += e
        vals.append(min(e.min(), 0.0))
    return pt2, np.sort(np.array(vals))


def _oracle(d, dets):
    return Oracle(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri, dets)


@pytest.mark.parametrize("name,n_psi,n_st,thresholds", [
    ("fci_s2", 12, 1, (0.99, 0.999)),
    ("fci_s2", 20, 2, (0.9, 0.99)),
    ("fci_cs", 16, 1, (1.0, 1.0)),
    ("fci_cs", 30, 3, (0.95, 0.999)),
])
def test_selection_pt2_matches_dense(name, n_psi, n_st, thresholds):
    d = load(name)
    idx, coef, e0, contrib = _wave_function(d, n_psi, n_st)
    tg, ts = thresholds
    n_gen = n_generators(contrib, tg)
    n_sel = n_selectors(contrib, n_gen, ts, tg)
    assert 1 <= n_gen <= n_sel <= n_psi
    o = _oracle(d, d["dets"][idx])
    buf = 50
    pt2, bdets, bvals, n_ext = o.select_pt2(coef, e0, n_gen, n_sel, buf)
    pt2_d, vals_d = _dense(d, idx, coef, e0, n_gen, n_sel)
    scale = np.abs(pt2_d).max()
    np.testing.assert_allclose(pt2, pt2_d, rtol=0, atol=1e-12 * max(scale, 1e-3))
    assert n_ext == len(vals_d)
    k = min(buf, len(vals_d))
    assert len(bvals) == k
    np.testing.assert_allclose(bvals, vals_d[:k], rtol=0, atol=1e-12 * max(abs(vals_d[0]), 1e-3))
    # the buffer holds determinants outside Psi, each once, in ascending value order
    keys = {bytes(x.tobytes()) for x in bdets}
    assert len(keys) == k
    assert not keys & {bytes(x.tobytes()) for x in d["dets"][idx]}
    assert np.all(np.diff(bvals) >= 0.0)


def test_selection_counts_every_external_once():
    # all determinants as generators: an external reached from several
    # generators still contributes once (spot_isinwf / past_d1 / past_d2)
    d = load("fci_cs")
    idx, coef, e0, _ = _wave_function(d, 24, 1)
    o = _oracle(d, d["dets"][idx])
    pt2, _, _, n_ext = o.select_pt2(coef, e0, 24, 24, 0)
    pt2_d, vals_d = _dense(d, idx, coef, e0, 24, 24)
    assert n_ext == len(vals_d)
    np.testing.assert_allclose(pt2, pt2_d, rtol=0, atol=1e-12 * abs(pt2_d).max())
    # counting every (generator, external) pair instead would give a larger sum
    assert len(vals_d) < sum(1 for g in idx for a in range(len(d["dets"]))
                             if a not in set(idx) and 1 <= _degree(d["dets"][a], d["dets"][g]) <= 2)


def test_generator_and_selector_counts():
    contrib = np.array([0.9, 0.05, 0.03, 0.015, 0.004, 0.001])
    assert n_generators(contrib, 0.99) == 4
    assert n_generators(contrib, 0.5) == 1
    assert n_selectors(contrib, 4, 0.999, 0.99) == 5
    assert n_selectors(contrib, 4, 0.5, 0.99) == 4          # at least the generators
    assert n_selectors(contrib, 1, 0.5, 1.0) == len(contrib)  # threshold_generators = 1: every determinant


def test_selection_rejects_bad_arguments():
    d = load("fci_s2")
    idx, coef, e0, _ = _wave_function(d, 10, 1)
    o = _oracle(d, d["dets"][idx])
    with pytest.raises(ValueError):
        o.select_pt2(coef, e0, 5, 4, 10)   # more generators than selectors
    with pytest.raises(ValueError):
        o.select_pt2(coef, e0, 1, 11, 10)  # more selectors than determinants
