"""Device Davidson (qpgpu_davidson_hs2) against the CPU oracle's restatement of
davidson_diag_hjj_sjj and against dense eigen-solves of golden matrices.

Bars: FP64 eigenvalues within 1e-9 Ha of the oracle / of the dense
eigenvalues; mixed precision (FP32 sigma, FP64 sigma at each restart) within
1e-6 Ha of the FP64 device run at threshold 1e-10 and within 1e-9 Ha at
1e-12 (both restart sigmas).  The seeded selected spaces are not spin
complete, so their runs use s2_eig = False (lowest eigenvalues of H in the
space); the full-CI golden spaces keep s2_eig = True.  Every run is capped.
"""
import numpy as np
import pytest

from golden_util import load
from oracle import Oracle
from quantum_package_gb300 import FP32, FP64
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _guess(n, nsd, seed):
    """Unit vector on the reference + seeded Gaussian extra guesses (diagonalization_hs2.irp.f:188-200)."""
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(nsd, n))
    u[0] = 0.0
    u[0, 0] = 1.0
    return u


def test_davidson_fp64_matches_oracle():
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=3000)
    wf = Wavefunction.from_problem(p)
    o = Oracle.from_problem(p)
    u = _guess(p.n_det, 4, 11)
    r = wf.davidson_diag_hs2(u, n_states=2, threshold=1e-12, s2_eig=False, max_iter=300)
    eo, s2o, _, nso, reso = o.davidson(u, 2, threshold=1e-12, s2_eig=False, max_sigma=300)
    assert r["converged"] and max(reso) < 1e-12
    np.testing.assert_allclose(r["energies"][:2], eo[:2], rtol=0, atol=1e-9)
    np.testing.assert_allclose(r["s2"][:2], s2o[:2], rtol=0, atol=1e-6)


@pytest.mark.parametrize("name", ["fci_s2", "fci_cs"])
def test_davidson_vs_dense_golden(name):
    from quantum_package_gb300.sigma import Wavefunction
    d = load(name)
    wf = Wavefunction(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"].h, d["ints"].eri, d["dets"])
    u = _guess(len(d["dets"]), 4, 5)
    r = wf.davidson_diag_hs2(u, n_states=2, threshold=1e-14, max_iter=300)
    assert r["converged"]
    sz = 0.5 * (d["n_alpha"] - d["n_beta"])
    good = np.abs(d["s2"] - sz * (sz + 1)) < 0.6
    ref = d["eigvals"][good][:2]
    np.testing.assert_allclose(r["energies"][:2], ref, rtol=0, atol=1e-9)


def test_davidson_mixed_precision_within_1e6():
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(2, n_det=20_000, n_states=4)
    wf = Wavefunction.from_problem(p)
    u = _guess(p.n_det, 8, 3)
    r64 = wf.davidson_diag_hs2(u, n_states=4, threshold=1e-10, s2_eig=False, max_iter=400)
    r32 = wf.davidson_diag_hs2(u, n_states=4, threshold=1e-10, s2_eig=False, precision=FP32, max_iter=400)
    assert r64["converged"] and r32["converged"]
    assert np.abs(r32["energies"][:4] - r64["energies"][:4]).max() < 1e-6
    tr = r32["trace"]
    assert (tr["precision"] == FP32).any() and tr["precision"][-1] == FP64


@pytest.mark.parametrize("prec_name,nsd,nst", [("FF", 8, 4), ("FP32", 8, 4), ("FP32", 3, 2), ("FP32", 1, 1),
                                               ("FF", 2, 2), ("FP32", 5, 3)])
def test_davidson_mixed_tight(prec_name, nsd, nst):
    # both mixed modes (FP32 sigma, the FP64 or float-float sigma at each
    # restart; float-float Gram-Schmidt, projections and Ritz vectors):
    # converged eigenvalues as accurate as the FP64 loop's
    from quantum_package_gb300 import FF
    from quantum_package_gb300.sigma import Wavefunction
    prec = {"FF": FF, "FP32": FP32}[prec_name]
    p = G.make_problem(2, n_det=20_000, n_states=4)
    wf = Wavefunction.from_problem(p)
    u = _guess(p.n_det, nsd, 3)
    kw = dict(n_states=nst, threshold=1e-12, s2_eig=False, max_iter=500)
    r64 = wf.davidson_diag_hs2(u, **kw)
    rm = wf.davidson_diag_hs2(u, precision=prec, **kw)
    assert r64["converged"] and rm["converged"]
    np.testing.assert_allclose(rm["energies"][:nst], r64["energies"][:nst], rtol=0, atol=1e-9)
    tr = rm["trace"]
    assert (tr["precision"] == FP32).any() and tr["precision"][-1] == (FF if prec == FF else FP64)


@pytest.mark.parametrize("threshold,tol", [(1e-10, 1e-6), (1e-12, 1e-9)])
@pytest.mark.parametrize("algebra_name", ["FP64", "TC"])
def test_davidson_mixed_fp64_algebra(threshold, tol, algebra_name):
    # FP32 sigma with the FP64 sigma at each restart; projections,
    # Gram-Schmidt, step and residual norms in FP64 -- on the FP64 pipe, or
    # with the Gram blocks FP64-accurate on the tensor cores (TC)
    from quantum_package_gb300 import ALGEBRA_FP64, ALGEBRA_TC
    from quantum_package_gb300.sigma import Wavefunction
    algebra = {"FP64": ALGEBRA_FP64, "TC": ALGEBRA_TC}[algebra_name]
    p = G.make_problem(2, n_det=20_000, n_states=4)
    wf = Wavefunction.from_problem(p)
    u = _guess(p.n_det, 8, 3)
    kw = dict(n_states=4, threshold=threshold, s2_eig=False, max_iter=500)
    r64 = wf.davidson_diag_hs2(u, **kw)
    rs = wf.davidson_diag_hs2(u, precision=FP32, algebra=algebra, **kw)
    assert r64["converged"] and rs["converged"]
    np.testing.assert_allclose(rs["energies"][:4], r64["energies"][:4], rtol=0, atol=tol)
    tr = rs["trace"]
    assert (tr["precision"] == FP32).any() and tr["precision"][-1] == FP64


def test_davidson_state_following_matches_oracle():
    # state_following (src/Davidson/EZFIO.cfg:19-22): the targets keep the
    # Ritz vectors of largest overlap with the guesses
    # (diagonalization_hs2.irp.f:328-370); same guess as the oracle's run
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=3000)
    wf = Wavefunction.from_problem(p)
    o = Oracle.from_problem(p)
    u = np.random.default_rng(1).normal(size=(4, p.n_det))
    kw = dict(threshold=1e-10, s2_eig=False)
    eo, _, _, _, _ = o.davidson(u, 2, davidson_sze_max=8, state_following=True, max_sigma=300, **kw)
    eo_plain, _, _, _, _ = o.davidson(u, 2, davidson_sze_max=8, max_sigma=300, **kw)
    assert abs(eo[0] - eo_plain[0]) > 1e-3  # the flag changes which states are followed here
    r = wf.davidson_diag_hs2(u, n_states=2, davidson_sze_max=8, state_following=True, max_iter=300, **kw)
    assert r["converged"]
    np.testing.assert_allclose(r["energies"][:2], eo[:2], rtol=0, atol=1e-8)


def test_davidson_fp64_with_tensor_core_grams_matches_oracle():
    # plain FP64 sigma with the Gram blocks on the tensor cores: the same
    # energies as the oracle's CPU Davidson
    from quantum_package_gb300 import ALGEBRA_TC
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=3000)
    wf = Wavefunction.from_problem(p)
    o = Oracle.from_problem(p)
    u = _guess(p.n_det, 4, 11)
    r = wf.davidson_diag_hs2(u, n_states=2, threshold=1e-12, s2_eig=False, max_iter=300, algebra=ALGEBRA_TC)
    eo, _, _, _, _ = o.davidson(u, 2, threshold=1e-12, s2_eig=False, max_sigma=300)
    assert r["converged"]
    np.testing.assert_allclose(r["energies"][:2], eo[:2], rtol=0, atol=1e-9)
