"""The CI-state callers of sigma and the Davidson against the oracle.

find_reference (src/Davidson/find_reference.irp.f:1-41) is restated in the
test as a plain loop over the oracle's dense H:
* references start from determinant 1;
* E0 = <u|H|u> of the references' coefficients, undivided by the norm
  (u_0_H_u_0, diagonalization_hs2.irp.f:446-485);
* determinant i joins when |(H_i,ref c_ref)^2 / (E0 - H_ii)| > thresh.
The device version must return the same list.

CI_electronic_energy (src/Davidson/diagonalize_CI.irp.f:22-165) is checked
both ways:
* its Davidson and Lapack branches must give the oracle's dense eigenvalues
  to 1e-9 Ha;
* with s2_eig, the Lapack branch must keep the states whose S^2 is within
  0.5 of the expected value.
The psi_coef guess (determinants.irp.f:174-224) must read an EZFIO file
whose mo_label matches, and ignore one whose label differs.
"""
import numpy as np
import pytest

from quantum_package_gb300 import ci, ezfio
from quantum_package_gb300 import generate as G


def test_diag_algorithm_rule():
    # determinants.irp.f:3-17: Davidson above N_det_max_jacobi, Lapack below
    # it and whenever N_det < N_states
    assert ci.diag_algorithm(2001, 1) == "Davidson"
    assert ci.diag_algorithm(2000, 1) == "Lapack"
    assert ci.diag_algorithm(3, 4) == "Lapack"
    assert ci.diag_algorithm(500, 2, n_det_max_jacobi=100) == "Davidson"


def test_psi_coef_guess_reads_matching_label(tmp_path):
    n = 40
    g = ci.psi_coef_guess(n, 3)
    np.testing.assert_array_equal(g[:3, :3], np.eye(3))
    assert g.sum() == 3.0
    p = G.make_problem(1, n_det=n)
    c = np.random.default_rng(2).normal(size=(n, 2))
    d = str(tmp_path / "wf.ezfio")
    ezfio.save_wavefunction_unsorted(d, p.dets, c, mo_label="Natural")
    r = ci.psi_coef_guess(n, 3, d, read_wf=True, mo_label="Natural")
    np.testing.assert_array_equal(r[:, :2], ezfio.read_psi_coef(d))
    np.testing.assert_array_equal(r[:, 2], g[:, 2])
    np.testing.assert_array_equal(ci.psi_coef_guess(n, 3, d, read_wf=True, mo_label="Canonical"), g)
    np.testing.assert_array_equal(ci.psi_coef_guess(n, 3, d, read_wf=False), g)


def _find_reference_dense(H, c, thresh):
    refs = [0]

    def e0():
        u = c[refs]
        return float(u @ H[np.ix_(refs, refs)] @ u)

    E0 = e0()
    for i in range(1, len(c)):
        hpsi = float(H[i, refs] @ c[refs])
        if abs(hpsi ** 2 / (E0 - H[i, i])) > thresh:
            refs.append(i)
            E0 = e0()
    return refs


@pytest.mark.gpu
def test_find_reference_matches_dense_restatement():
    from oracle import Oracle
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=400)
    H, _ = Oracle.from_problem(p).dense(with_s2=False)
    w, X = np.linalg.eigh(H)
    psi = X[:, :2]
    wf = Wavefunction.from_problem(p)
    for thresh in (1e-3, 1e-5, 1e-7):
        got = ci.find_reference(wf, psi, thresh)
        ref = _find_reference_dense(H, psi[:, 0], thresh)
        assert got.tolist() == ref, thresh
    assert len(ci.find_reference(wf, psi, 1e-7)) > len(ci.find_reference(wf, psi, 1e-3))
    wf.close()


@pytest.mark.gpu
def test_ci_energy_davidson_and_lapack_branches():
    from oracle import Oracle
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=300)
    H, S2 = Oracle.from_problem(p).dense(with_s2=True)
    w = np.linalg.eigvalsh(H)
    wf = Wavefunction.from_problem(p)
    guess = ci.psi_coef_guess(p.n_det, 2)
    rd = ci.ci_electronic_energy(wf, guess, 2, n_states_diag=4, algorithm="Davidson", s2_eig=False,
                                 threshold=1e-12, max_iter=400)
    rl = ci.ci_electronic_energy(wf, guess, 2, n_states_diag=4, algorithm="Lapack", s2_eig=False)
    np.testing.assert_allclose(rd["energies"][:2], w[:2], rtol=0, atol=1e-9)
    np.testing.assert_allclose(rl["energies"], w[:4], rtol=0, atol=1e-9)
    # S^2 of the Lapack eigenvectors against the oracle's dense S^2 (+ S_z(S_z-1), as u_0_S2_u_0)
    X = rl["eigenvectors"]
    s2o = np.einsum("ij,ij->j", X, S2 @ X) / np.einsum("ij,ij->j", X, X)
    np.testing.assert_allclose(rl["s2"], s2o + ci.s_z2_sz(wf), rtol=0, atol=1e-9)
    new, res = ci.diagonalize_ci(wf, guess, 2, n_states_diag=4, algorithm="Lapack", s2_eig=False)
    np.testing.assert_allclose(np.einsum("ij,ij->j", new, H @ new), res["energies"][:2], rtol=0, atol=1e-9)
    np.testing.assert_allclose(ci.ci_energy(res, nuclear_repulsion=9.5)[:2], res["energies"][:2] + 9.5)
    wf.close()


@pytest.mark.gpu
def test_lapack_branch_keeps_states_of_the_expected_spin():
    # a spin-complete set (full CI, 3 + 3 electrons in 7 MOs): S^2 eigenvalues
    # are exact, and s2_eig keeps the lowest singlets
    from oracle import Oracle
    from quantum_package_gb300.sigma import Wavefunction
    n_mo, na, nb = 7, 3, 3
    ints = G.make_integrals(n_mo, 31)
    dets = G.full_ci_dets(n_mo, na, nb)
    o = Oracle(n_mo, na, nb, ints.h, ints.eri, dets)
    H, S2 = o.dense(with_s2=True)
    w, X = np.linalg.eigh(H)
    s2o = np.einsum("ij,ij->j", X, S2 @ X)
    singlets = w[np.abs(s2o) <= 0.5]
    wf = Wavefunction(n_mo, na, nb, ints.h, ints.eri, dets)
    guess = ci.psi_coef_guess(len(dets), 2)
    rs = ci.ci_electronic_energy(wf, guess, 2, n_states_diag=4, algorithm="Lapack", s2_eig=True)
    np.testing.assert_allclose(rs["energies"][:2], singlets[:2], rtol=0, atol=1e-9)
    assert np.all(np.abs(rs["s2"][:2]) <= 1e-8), rs["s2"]
    # the remaining slots take the other eigenvectors in order
    others = [j for j in range(len(w)) if abs(s2o[j]) > 0.5][:2]
    np.testing.assert_allclose(rs["energies"][2:], w[others], rtol=0, atol=1e-9)
    wf.close()
