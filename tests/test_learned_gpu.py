"""Learned Davidson preconditioner end to end on the GPU.

CIPSI-style growth (the first 1e4 determinants of a seeded 14a+14b / 80-MO
draw, then the first 6e4): training pairs are captured from the converged
smaller stage, the CUDA kernels train the MLP, and the larger stage is solved
with and without it to a squared residual of 1e-12.  The converged energies
must agree to 1e-9 Ha (the network only changes the search directions); the
iteration counts of both runs are reported.  A network with wild weights must be caught by the
fallback and still reach the same energies.
"""
import numpy as np
import pytest

from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu

NST, NSD = 4, 8


def _guess(n, seed=1):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(NSD, n))
    u[0] = 0.0
    u[0, 0] = 1.0
    return u


@pytest.fixture(scope="module")
def staged():
    from quantum_package_gb300.sigma import Wavefunction
    full = G.make_problem(4, n_det=60_000)
    wf = Wavefunction(full.n_mo, full.n_alpha, full.n_beta, full.ints.h, full.ints.eri, full.dets[:10_000])
    wf.mlp_init(seed=3)
    r = wf.davidson_diag_hs2(_guess(10_000), n_states=NST, threshold=1e-10, s2_eig=False, collect_every=1,
                             collect_max=16, max_iter=400)
    assert r["converged"] and r["n_samples"] > 0
    loss = wf.mlp_train(epochs=20, batch=4096, lr=2e-3, seed=4)
    assert np.isfinite(loss)
    wf.set_dets(full.dets)
    return wf


def test_learned_preconditioner_gain_and_same_energies(staged, capsys):
    wf = staged
    u = _guess(wf.n_det)
    kw = dict(n_states=NST, threshold=1e-12, s2_eig=False, max_iter=500)
    diag = wf.davidson_diag_hs2(u, **kw)
    learned = wf.davidson_diag_hs2(u, preconditioner=1, **kw)
    extra = wf.davidson_diag_hs2(u, preconditioner=2, **kw)
    assert diag["converged"] and learned["converged"] and extra["converged"]
    np.testing.assert_allclose(learned["energies"][:NST], diag["energies"][:NST], rtol=0, atol=1e-9)
    np.testing.assert_allclose(extra["energies"][:NST], diag["energies"][:NST], rtol=0, atol=1e-9)
    with capsys.disabled():
        print(f"\n[learned preconditioner] sigma applications: diagonal {diag['n_sigma']}, "
              f"learned in place {learned['n_sigma']} (fallbacks {learned['n_fallback']}), "
              f"learned as extra direction {extra['n_sigma']}")
    # no more than a modest regression allowed, whatever the draw
    assert learned["n_sigma"] <= 1.25 * diag["n_sigma"]
    assert extra["n_sigma"] <= 1.15 * diag["n_sigma"]


def test_bad_network_falls_back(staged):
    wf = staged
    good = wf.mlp_weights()
    rng = np.random.default_rng(0)
    wf.mlp_set_weights((rng.normal(size=good.size) * 3.0).astype(np.float32))
    try:
        u = _guess(wf.n_det)
        kw = dict(n_states=NST, threshold=1e-12, s2_eig=False, max_iter=800)
        diag = wf.davidson_diag_hs2(u, **kw)
        bad = wf.davidson_diag_hs2(u, preconditioner=1, **kw)
        assert bad["converged"] and bad["n_fallback"] >= 1
        np.testing.assert_allclose(bad["energies"][:NST], diag["energies"][:NST], rtol=0, atol=1e-9)
    finally:
        wf.mlp_set_weights(good)
