"""Batched CI problems (qpgpu_batch_davidson) against one-problem-at-a-time runs.

Problems of uneven size (seeded: 30-60 MOs, 8-16 electrons per spin,
1e3-4e3 determinants, 1-3 states) go through one persistent sigma launch per
iteration; every problem's eigenvalues must match those of its own
qpgpu_davidson_hs2 run: 1e-9 Ha in FP64, 1e-6 Ha in mixed precision.
"""
import numpy as np
import pytest

from quantum_package_gb300 import FP32, FP64
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu
NSD = 4


def _guess(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(NSD, n))
    u[0] = 0.0
    u[0, 0] = 1.0
    return u


@pytest.fixture(scope="module")
def problems():
    from quantum_package_gb300.sigma import Wavefunction
    probs = G.batched_problems(6, n_det_min=1000, n_det_max=4000)
    wfs = [Wavefunction.from_problem(p) for p in probs]
    return probs, wfs


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-9), (FP32, 1e-6)])
def test_batch_matches_single_problem_runs(problems, prec, tol):
    from quantum_package_gb300.batch import Batch
    probs, wfs = problems
    guesses = [_guess(p.n_det, 7 + i) for i, p in enumerate(probs)]
    nst = [p.n_states for p in probs]
    b = Batch(wfs)
    r = b.davidson(guesses, nst, threshold=1e-10, precision=prec, max_iter=400)
    assert r["stats"]["n_converged"] == len(probs)
    assert r["stats"]["tuned_warps"] in (4, 8)
    for i, (p, wf) in enumerate(zip(probs, wfs)):
        single = wf.davidson_diag_hs2(guesses[i], n_states=p.n_states, threshold=1e-10, s2_eig=False,
                                      precision=FP64, max_iter=400)
        assert single["converged"]
        np.testing.assert_allclose(r["energies"][i, :p.n_states], single["energies"][:p.n_states], rtol=0, atol=tol)
    b.close()
