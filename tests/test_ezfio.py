"""EZFIO wave-function I/O of the determinants group against the reference's
save/read routines (src/Determinants/determinants.irp.f:399-540).

save_wavefunction_general writes n_int, bit_kind, n_det, n_states, mo_label,
psi_det as integer*8 words (n_int, 2, n_det) and psi_coef (n_det, n_states)
with every state normalised (a zero state divided by sqrt(1e-12));
save_wavefunction orders the determinants by decreasing state-averaged norm
contribution through the reference's dsort (insertion sort below 32 entries,
middle-pivot quicksort otherwise, src/Utils/sort.irp.f:1-78,241-265);
read_dets checks n_int and bit_kind.  The checks: exact round trips, the
stored layout (rank, dimensions, Fortran order, signed words), the sort
order and the refusals.  The GPU test builds the device wave function from
the file read back and compares its sigma with the oracle's on the original
determinants, bit for bit in the pairs and to 1e-12 in sigma.
"""
import gzip
import os

import numpy as np
import pytest

from quantum_package_gb300 import ezfio
from quantum_package_gb300 import generate as G


def _coefs(n, nst, seed, zero_state=None):
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(n, nst))
    if zero_state is not None:
        c[:, zero_state] = 0.0
    return c


def test_unsorted_round_trip_and_layout(tmp_path):
    p = G.make_problem(2, n_det=300)  # N_int = 2: words with the top bit set appear
    c = _coefs(p.n_det, 3, 1, zero_state=2)
    d = str(tmp_path / "wf.ezfio")
    ezfio.save_wavefunction_unsorted(d, p.dets, c, mo_label="Canonical")
    dets, coefs = ezfio.read_wavefunction(d, n_int=2)
    np.testing.assert_array_equal(dets, p.dets)
    for k in range(2):
        col = c[:, k]
        np.testing.assert_array_equal(coefs[:, k], col * (1.0 / np.sqrt(np.cumsum(col * col)[-1])))
    np.testing.assert_array_equal(coefs[:, 2], 0.0)  # a zero state stays zero (norm taken as 1e-12)
    assert ezfio.read_scalar(d, "n_det") == p.n_det
    assert ezfio.read_scalar(d, "n_states") == 3
    assert ezfio.read_scalar(d, "bit_kind") == 8
    assert ezfio.read_scalar(d, "mo_label", str) == "Canonical"
    with gzip.open(os.path.join(d, "determinants", "psi_det.gz"), "rt") as f:
        tok = f.read().split()
    assert [int(t) for t in tok[:4]] == [3, 2, 2, p.n_det]
    words = np.array([int(t) for t in tok[4:4 + 4]], dtype=np.int64)
    np.testing.assert_array_equal(words.view(np.uint64), p.dets[0].reshape(-1))  # (k, spin) fastest
    with gzip.open(os.path.join(d, "determinants", "psi_coef.gz"), "rt") as f:
        tok = f.read().split()
    assert [int(t) for t in tok[:3]] == [2, p.n_det, 3]
    assert float(tok[3 + 1]) == coefs[1, 0]  # determinant index fastest


def test_sorted_save_orders_by_norm_contribution(tmp_path):
    p = G.make_problem(1, n_det=200)
    c = _coefs(p.n_det, 2, 3)
    c[10:20] = c[5]  # ties
    d = str(tmp_path / "wf.ezfio")
    order = ezfio.save_wavefunction(d, p.dets, c)
    dets, coefs = ezfio.read_wavefunction(d)
    assert sorted(order.tolist()) == list(range(p.n_det))
    np.testing.assert_array_equal(dets, p.dets[order])
    contrib = ezfio.average_norm_contrib(c)[order]
    assert np.all(np.diff(contrib) <= 0.0)
    cn = c / np.sqrt(np.cumsum(c * c, axis=0)[-1])
    np.testing.assert_allclose(coefs, cn[order], rtol=1e-15, atol=0)


def test_dsort_insertion_is_stable_and_quicksort_sorts():
    x = [3.0, 1.0, 2.0, 1.0, 3.0, 0.5, 1.0]
    xs, order = ezfio.dsort(x)
    assert xs.tolist() == sorted(x)
    assert order.tolist() == [5, 1, 3, 6, 2, 0, 4]  # ties in their input order below 32 entries
    rng = np.random.default_rng(0)
    y = rng.integers(0, 20, size=1000).astype(float)
    ys, oy = ezfio.dsort(y)
    assert np.all(np.diff(ys) >= 0) and np.array_equal(y[oy], ys)
    assert sorted(oy.tolist()) == list(range(1000))


def test_ref_determinant_and_refusals(tmp_path):
    p = G.make_problem(2, n_det=10)
    d = str(tmp_path / "ref.ezfio")
    ezfio.save_ref_determinant(d, p.dets[0], n_states=2)
    dets, coefs = ezfio.read_wavefunction(d)
    np.testing.assert_array_equal(dets, p.dets[:1])
    np.testing.assert_array_equal(coefs, [[1.0, 0.0]])
    with pytest.raises(ValueError):
        ezfio.read_dets(d, n_int=1)
    ezfio.write_scalar(d, "bit_kind", 4)
    with pytest.raises(ValueError):
        ezfio.read_dets(d)


@pytest.mark.gpu
def test_sigma_of_read_back_wavefunction(tmp_path):
    from oracle import Oracle
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=2000)
    c = _coefs(p.n_det, 2, 9)
    d = str(tmp_path / "wf.ezfio")
    order = ezfio.save_wavefunction(d, p.dets, c)
    dets, coefs = ezfio.read_wavefunction(d)
    wf = Wavefunction(p.n_mo, p.n_alpha, p.n_beta, p.ints.h, p.ints.eri, dets)
    v, s = wf.H_S2_u_0_nstates_openmp(np.ascontiguousarray(coefs.T))
    vo, so = Oracle.from_problem(p).h_s2_u0(np.ascontiguousarray(coefs.T[:, np.argsort(order)]))
    vo, so = vo[:, order], so[:, order]
    scale = np.abs(vo).max(axis=1, keepdims=True)
    assert np.all(np.abs(v - vo).max(axis=1, keepdims=True) <= 1e-12 * scale)
    np.testing.assert_allclose(s, so, rtol=0, atol=1e-12 * max(1.0, np.abs(so).max()))
    wf.close()
