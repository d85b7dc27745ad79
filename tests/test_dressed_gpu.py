"""Dressed sigma and Davidson of the MRCC / MRCEPA0 plugins against the oracle.

H_S2_u_0_mrcc_nstates (plugins/MRCC_Utils/davidson.irp.f:955-1127) adds to
the sigma of H a dressing that couples each reference determinant
i = idx_ref(ii) with each non-reference determinant j = idx_non_ref(jj) both
ways (:1084-1105: v_i += delta_ij(jj,ii) u_j, v_j += delta_ij(jj,ii) u_i, the
same with delta_ij_s2 for S^2), and its diagonal term uses H_jj dressed by
delta_ii on the references (:1120-1124 with :547-549).  The check restates
those loops in numpy on top of the oracle's sigma: the device result must
agree to 1e-12 relative.  The dressed Davidson (davidson_diag_mrcc_hs2,
:496-553) must reach the lowest eigenvalues of the dense dressed matrix to
1e-9 Ha.
"""
import numpy as np
import pytest

from oracle import Oracle
from quantum_package_gb300 import QPGPUError
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _dressing(n_det, seed, n_ref=12, n_non_ref=1800):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_det)
    ref, nref = perm[:n_ref], np.sort(perm[n_ref:n_ref + n_non_ref])
    d = rng.normal(0.0, 0.01, (n_ref, n_non_ref))
    ds = rng.normal(0.0, 0.001, (n_ref, n_non_ref))
    dii = rng.normal(0.0, 0.05, n_ref)
    return ref, nref, d, ds, dii


def _oracle_dressed(o, u, ref, nref, d, ds, dii):
    v, s = o.h_s2_u0(u)
    v = v.copy()
    s = s.copy()
    for k in range(u.shape[0]):
        v[k, ref] += d @ u[k, nref] + dii * u[k, ref]
        v[k, nref] += d.T @ u[k, ref]
        s[k, ref] += ds @ u[k, nref]
        s[k, nref] += ds.T @ u[k, ref]
    return v, s


def test_dressed_sigma_matches_oracle():
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=3000)
    wf = Wavefunction.from_problem(p)
    o = Oracle.from_problem(p)
    dr = _dressing(p.n_det, 5)
    wf.set_dressing(*dr)
    u = G.random_coefficients(p.n_det, 3, 7)
    v, s = wf.H_S2_u_0_mrcc_nstates(u)
    vo, so = _oracle_dressed(o, u, *dr)
    scale = np.abs(vo).max(axis=1, keepdims=True)
    assert np.all(np.abs(v - vo).max(axis=1, keepdims=True) <= 1e-12 * scale)
    np.testing.assert_allclose(s, so, rtol=0, atol=1e-12 * max(1.0, np.abs(so).max()))
    # the plain sigma is unchanged by a dressing
    v0, _ = wf.H_S2_u_0_nstates_openmp(u)
    np.testing.assert_allclose(v0, o.h_s2_u0(u)[0], rtol=0, atol=1e-12 * np.abs(vo).max())
    wf.clear_dressing()
    with pytest.raises(QPGPUError) as e:
        wf.H_S2_u_0_mrcc_nstates(u)
    assert e.value.code == -2


def test_dressed_davidson_matches_dense():
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=2500)
    wf = Wavefunction.from_problem(p)
    o = Oracle.from_problem(p)
    ref, nref, d, ds, dii = _dressing(p.n_det, 9, n_ref=8, n_non_ref=2000)
    wf.set_dressing(ref, nref, d, ds, dii)
    H, _ = o.dense(with_s2=False)
    Hd = H.copy()
    Hd[np.ix_(ref, nref)] += d
    Hd[np.ix_(nref, ref)] += d.T
    Hd[ref, ref] += dii
    w = np.linalg.eigvalsh(Hd)[:2]
    rng = np.random.default_rng(3)
    u = rng.normal(size=(4, p.n_det))
    r = wf.davidson_diag_hs2(u, n_states=2, threshold=1e-12, s2_eig=False, max_iter=400, dressed=True)
    assert r["converged"]
    np.testing.assert_allclose(r["energies"][:2], w, rtol=0, atol=1e-9)
    r0 = wf.davidson_diag_hs2(u, n_states=2, threshold=1e-12, s2_eig=False, max_iter=400)
    assert np.abs(r0["energies"][:2] - w).max() > 1e-6  # the dressing matters here
