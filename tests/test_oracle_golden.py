"""The CPU oracle against golden vectors from second quantisation (oracle/secondq.py).

These pin the restatement of src/Determinants/slater_rules.irp.f,
src/Determinants/s2.irp.f and src/Davidson/u0Hu0.irp.f to an evaluator that
shares none of their phase/excitation formulas.
"""
import numpy as np
import pytest

from golden_util import load
from oracle import Oracle

SZ2SZ = lambda na, nb: 0.5 * (na - nb) * (0.5 * (na - nb) - 1.0)  # noqa: E731


def _oracle(d, dets=None):
    return Oracle(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri,
                  d["dets"] if dets is None else dets)


@pytest.mark.parametrize("name", ["fci_s2", "fci_cs"])
def test_full_ci_dense_matrices(name):
    d = load(name)
    o = _oracle(d)
    H, S = o.dense()
    # i_H_j generic path == second quantisation, elementwise; both operators Hermitian
    np.testing.assert_allclose(H, d["H"], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(S, d["S"])
    np.testing.assert_allclose(H, H.T, rtol=0, atol=1e-13 * np.abs(H).max())
    np.testing.assert_array_equal(S, S.T)
    # sigma path (u0Hu0.irp.f) == dense H
    u = np.random.default_rng(1).normal(size=(3, len(d["dets"])))
    v, s = o.h_s2_u0(u)
    np.testing.assert_allclose(v, u @ d["H"], rtol=0, atol=1e-12 * np.abs(u @ np.abs(d["H"])).max())
    np.testing.assert_allclose(s, u @ d["S"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", ["fci_s2", "fci_cs"])
def test_full_ci_spin_spectrum(name):
    d = load(name)
    s2 = d["s2"]
    sz = 0.5 * (d["n_alpha"] - d["n_beta"])
    allowed = np.array([S * (S + 1) for S in np.arange(sz, 10, 1.0)])
    dist = np.abs(s2[:, None] - allowed[None, :]).min(axis=1)
    assert dist.max() < 1e-8


@pytest.mark.parametrize("name", ["sci_n1", "sci_n2"])
def test_sigma_selected_space(name):
    d = load(name)
    o = _oracle(d)
    v, s = o.h_s2_u0(d["u"])
    scale = np.abs(d["sigma"]).max()
    np.testing.assert_allclose(v, d["sigma"], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(s, d["s2sigma"], rtol=0, atol=1e-12)
    hd, _ = o.diag()
    np.testing.assert_allclose(hd, d["hdiag"], rtol=0, atol=1e-12 * np.abs(d["hdiag"]).max())
    if "n_pairs" in d:
        I, J, cls = o.connected_pairs()
        assert len(I) == int(d["n_pairs"])


def test_sampled_pairs_word_boundary():
    d = load("pairs_n2")
    o = Oracle(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri)
    for di, dj, hij, sij in zip(d["I"], d["J"], d["hij"], d["sij"]):
        assert abs(o.i_h_j(di, dj) - hij) <= 1e-12 * max(1.0, abs(hij))
        assert o.get_s2(di, dj) == sij


def test_sampled_pairs_spin_routines():
    """The spin-specific routines used by sigma (get_*_excitation_spin) on the same pairs."""
    d = load("pairs_n2")
    na, nb = d["n_alpha"], d["n_beta"]
    dets = np.concatenate([d["I"], d["J"]])
    # unique dets only
    v = dets.reshape(len(dets), -1)
    _, first = np.unique(v, axis=0, return_index=True)
    o = Oracle(d["n_mo"], na, nb, d["ints"].h, d["ints"].eri, dets[np.sort(first)])
    pos = {dets[i].tobytes(): k for k, i in enumerate(np.sort(first))}
    for di, dj, hij, sij, k in zip(d["I"], d["J"], d["hij"], d["sij"], d["kind"]):
        ph, exc, h2, s2 = o.pair_excitation(pos[di.tobytes()], pos[dj.tobytes()], int(k))
        assert abs(h2 - hij) <= 1e-12 * max(1.0, abs(hij))
        assert s2 == sij


@pytest.mark.parametrize("name", ["fci_s2", "fci_cs"])
def test_oracle_davidson_matches_dense_eigenvalues(name):
    """The oracle's restatement of davidson_diag_hjj_sjj (s2_eig on, spin-complete space)
    against the eigenvalues of the second-quantisation matrix with the target S^2."""
    d = load(name)
    o = _oracle(d)
    n = len(d["dets"])
    rng = np.random.default_rng(5)
    u = rng.normal(size=(4, n))
    u[0] = 0.0
    u[0, 0] = 1.0
    e, s2, _, n_sigma, res = o.davidson(u, 2, threshold=1e-14, s2_eig=True, max_sigma=300)
    sz = 0.5 * (d["n_alpha"] - d["n_beta"])
    good = np.abs(d["s2"] - sz * (sz + 1)) < 0.6
    ref = d["eigvals"][good][:2]
    assert 0 < n_sigma < 300 and max(res) < 1e-14
    np.testing.assert_allclose(e[:2], ref, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s2[:2], sz * (sz + 1), rtol=0, atol=1e-6)
