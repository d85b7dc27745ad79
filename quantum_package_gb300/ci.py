"""The callers of the Davidson and of sigma: the CI-state providers of the
reference, on top of the device library.

* ``psi_coef_guess`` is the ``psi_coef`` provider
  (src/Determinants/determinants.irp.f:174-224): coefficient 1 on
  determinant i of state i, replaced by the EZFIO file's ``psi_coef`` when
  ``read_wf`` is set and the file's ``mo_label`` matches.
* ``ci_electronic_energy`` is ``CI_electronic_energy`` / ``CI_eigenvectors`` /
  ``CI_eigenvectors_s2`` (src/Davidson/diagonalize_CI.irp.f:22-165).  The
  guess is ``psi_coef`` for the first min(N_states, N_det) vectors; the
  "Davidson" branch (davidson_diag_HS2 on the device) fills the others with
  seeded normal vectors, as davidson_diag_hjj_sjj draws them
  (diagonalization_hs2.irp.f:188-200).  The "Lapack" branch diagonalises the dense H assembled from the
  device's pair elements and diagonal, and picks states by S^2 as the
  reference does when s2_eig is set.
* ``ci_energy`` adds the nuclear repulsion (:1-20).  ``diagonalize_ci``
  returns the new ``psi_coef`` (:154-167).
* ``find_reference`` (src/Davidson/find_reference.irp.f:1-41) grows the
  reference list from determinant 1.  Determinant i joins when
  (<i|H|psi_ref>)^2 / (E0 - H_ii) exceeds the threshold in magnitude.
  E0 = u_0_H_u_0 of the references at the time, which is <u|H|u>
  undivided by the norm (diagonalization_hs2.irp.f:446-485).  The device
  computes H u_ref for every determinant with one sigma call per accepted
  reference.
* ``u_0_S2_u_0`` (src/Determinants/s2.irp.f:107-130):
  <u|S^2|u>/<u|u> + S_z(S_z - 1).

Energies are electronic unless stated.
"""
from __future__ import annotations

import numpy as np

from . import ezfio as _ezfio

MAX_SIGMA_STATES = 8  # states per sigma call of the device library


def psi_coef_guess(n_det, n_states, ezfio_dir=None, read_wf=False, mo_label=None):
    """(n_det, n_states) guess of the psi_coef provider."""
    c = np.zeros((n_det, n_states))
    for i in range(min(n_states, n_det)):
        c[i, i] = 1.0
    if read_wf and ezfio_dir is not None and _ezfio.has(ezfio_dir, "psi_coef"):
        exists = True
        if _ezfio.has(ezfio_dir, "mo_label"):
            exists = mo_label is None or _ezfio.read_scalar(ezfio_dir, "mo_label", str) == mo_label
        if exists:
            r = _ezfio.read_psi_coef(ezfio_dir)
            if r.shape[0] != n_det:
                raise ValueError(f"psi_coef of {ezfio_dir} has {r.shape[0]} determinants, not {n_det}")
            k = min(n_states, r.shape[1])
            c[:, :k] = r[:, :k]
    return c


def _sigma_batches(wf, U):
    """(H U, S^2 U) for U (k, N), at most MAX_SIGMA_STATES vectors per call."""
    V = np.empty_like(U)
    S = np.empty_like(U)
    for a in range(0, U.shape[0], MAX_SIGMA_STATES):
        v, s = wf.H_S2_u_0_nstates_openmp(U[a:a + MAX_SIGMA_STATES])
        V[a:a + MAX_SIGMA_STATES] = v
        S[a:a + MAX_SIGMA_STATES] = s
    return V, S


def s_z2_sz(wf):
    sz = 0.5 * (wf.n_alpha - wf.n_beta)
    return sz * (sz - 1.0)


def u_0_S2_u_0(wf, U):
    """<u|S^2|u>/<u|u> + S_z(S_z - 1) for each row u of U (k, N)."""
    U = np.ascontiguousarray(np.atleast_2d(U), dtype=np.float64)
    _, S = _sigma_batches(wf, U)
    return np.einsum("ij,ij->i", S, U) / np.einsum("ij,ij->i", U, U) + s_z2_sz(wf)


def dense_h(wf):
    """The dense H of the determinant set from the device's pair elements and
    diagonal (the reference's H_matrix_all_dets, for small sets)."""
    n = wf.n_det
    H = np.zeros((n, n))
    p = wf.connected_pairs()
    H[p["I"], p["J"]] = p["hij"]
    H[p["J"], p["I"]] = p["hij"]
    H[np.arange(n), np.arange(n)] = wf.diag()[0]
    return H


N_DET_MAX_JACOBI = 2000  # src/Determinants/EZFIO.cfg default


def diag_algorithm(n_det, n_states, n_det_max_jacobi=N_DET_MAX_JACOBI):
    """The diag_algorithm provider (src/Determinants/determinants.irp.f:3-17):
    Davidson above N_det_max_jacobi determinants, else Lapack, and Lapack
    when N_det < N_states."""
    alg = "Davidson" if n_det > n_det_max_jacobi else "Lapack"
    return "Lapack" if n_det < n_states else alg


def ci_electronic_energy(wf, psi_coef, n_states, n_states_diag=None, algorithm=None, s2_eig=True,
                         expected_s2=None, threshold=1e-12, davidson_sze_max=8, seed=0,
                         n_det_max_jacobi=N_DET_MAX_JACOBI, **davidson_kw):
    """CI_electronic_energy, CI_eigenvectors (N_det, N_states_diag) and
    CI_eigenvectors_s2; ``algorithm`` None follows diag_algorithm."""
    n = wf.n_det
    if algorithm is None:
        algorithm = diag_algorithm(n, n_states, n_det_max_jacobi)
    nsd = n_states if n_states_diag is None else n_states_diag
    if expected_s2 is None:
        sz = 0.5 * (wf.n_alpha - wf.n_beta)
        expected_s2 = sz * (sz + 1.0)
    guess = np.zeros((n, nsd))
    k = min(n_states, n)
    guess[:, :k] = np.asarray(psi_coef)[:, :k]
    if algorithm == "Davidson":
        # davidson_diag_hjj_sjj draws the guesses beyond N_states from a
        # normal distribution (diagonalization_hs2.irp.f:188-200); seeded here
        rng = np.random.default_rng(seed)
        for c in range(k, min(n, nsd)):
            guess[:, c] = rng.normal(size=n)
        r = wf.davidson_diag_hs2(np.ascontiguousarray(guess[:, :min(n, nsd)].T), min(n, n_states),
                                 davidson_sze_max=davidson_sze_max, threshold=threshold, s2_eig=s2_eig,
                                 **davidson_kw)
        e = np.zeros(nsd)
        s2 = np.zeros(nsd)
        vec = np.zeros((n, nsd))
        m = min(n, nsd)
        e[:m] = r["energies"][:m]
        s2[:m] = r["s2"][:m]
        vec[:, :m] = r["vectors"][:m].T
        return dict(energies=e, eigenvectors=vec, s2=s2, converged=r["converged"], n_sigma=r["n_sigma"])
    if algorithm != "Lapack":
        raise ValueError(f"diag_algorithm {algorithm!r}: Davidson or Lapack")
    w, X = np.linalg.eigh(dense_h(wf))
    e = np.zeros(nsd)
    s2 = np.zeros(nsd)
    vec = guess.copy()
    if s2_eig:
        s2v = u_0_S2_u_0(wf, X.T)
        good = [j for j in range(n) if abs(s2v[j] - expected_s2) <= 0.5][:n_states]
        if good:
            for a, j in enumerate(good):
                vec[:, a] = X[:, j]
                e[a] = w[j]
                s2[a] = s2v[j]
            other = 0
            for j in range(n):
                if j in good:
                    continue
                other += 1
                if len(good) + other > nsd:
                    break
                vec[:, len(good) + other - 1] = X[:, j]
                e[len(good) + other - 1] = w[j]
                # the reference takes this S^2 from the position, not from j
                # (diagonalize_CI.irp.f:117); restated as written
                s2[len(good) + other - 1] = s2v[len(good) + other - 1]
        else:
            for j in range(min(nsd, n)):
                vec[:, j] = X[:, j]
                e[j] = w[j]
                s2[j] = s2v[j]
    else:
        m = min(n, nsd)
        s2[:m] = u_0_S2_u_0(wf, X[:, :m].T)
        vec[:, :m] = X[:, :m]
        e[:m] = w[:m]
    return dict(energies=e, eigenvectors=vec, s2=s2, converged=True, n_sigma=0)


def ci_energy(res, nuclear_repulsion=0.0, n_det=None):
    """CI_energy = CI_electronic_energy + nuclear_repulsion."""
    e = np.asarray(res["energies"])
    m = len(e) if n_det is None else min(n_det, len(e))
    return e[:m] + nuclear_repulsion


def diagonalize_ci(wf, psi_coef, n_states, **kw):
    """diagonalize_CI: the new psi_coef (N_det, N_states) and the CI result."""
    res = ci_electronic_energy(wf, psi_coef, n_states, **kw)
    return np.ascontiguousarray(res["eigenvectors"][:, :n_states]), res


def find_reference(wf, psi_coef, thresh, istate=0):
    """find_reference(thresh): 0-based indices of the reference determinants."""
    c = np.asarray(psi_coef, dtype=np.float64)[:, istate]
    n = wf.n_det
    hii = wf.diag()[0]
    refs = [0]
    u = np.zeros((1, n))
    u[0, 0] = c[0]

    def refresh():
        v, _ = wf.H_S2_u_0_nstates_openmp(u)
        e0 = float(np.dot(v[0], u[0])) if np.dot(u[0], u[0]) != 0.0 else 0.0
        return v[0], e0

    hpsi, e0 = refresh()
    for i in range(1, n):
        de = hpsi[i] ** 2 / (e0 - hii[i])
        if abs(de) > thresh:
            refs.append(i)
            u[0, i] = c[i]
            hpsi, e0 = refresh()
    return np.asarray(refs, dtype=np.int64)
