"""Direct sigma (QPGPU_SIGMA_DIRECT): no stored pairs, every call enumerates them.

For determinant sets whose connected pairs do not fit in device memory (2e7
determinants in 120 MOs hold 5.3e10 pairs), sigma walks the bilinear index
and evaluates the Slater rules at each call, as the reference does
(u0Hu0.irp.f:177-444).  Bars: FP64 sigma and S^2 sigma within 1e-12 relative
of the stored-pair path and of the oracle, the range variant selects the same
rows, Davidson eigenvalues within 1e-9 Ha of the stored-pair run, and the
entry points that need stored pairs refuse the direct set cleanly.
"""
import numpy as np
import pytest

from oracle import Oracle
from quantum_package_gb300 import FP32, FP64, SIGMA_DIRECT, SIGMA_STORED, QPGPUError
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu

REL64 = 1e-12


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module", params=[(1, 3000), (2, 5000)], ids=["nint1", "nint2"])
def pair(request):
    from quantum_package_gb300.sigma import Wavefunction
    cfg, n = request.param
    p = G.make_problem(cfg, n_det=n)
    stored = Wavefunction.from_problem(p, sigma_mode=SIGMA_STORED)
    direct = Wavefunction.from_problem(p, sigma_mode=SIGMA_DIRECT)
    return p, stored, direct


def test_modes_and_counts(pair):
    p, stored, direct = pair
    i_s, i_d = stored.info(), direct.info()
    assert i_s["direct_sigma"] == 0 and i_d["direct_sigma"] == 1
    assert i_d["n_pairs"] == i_s["n_pairs"] > 0
    np.testing.assert_array_equal(direct.bilinear_order(), stored.bilinear_order())


@pytest.mark.parametrize("n_st", [1, 3, 8])
def test_direct_sigma_matches_stored_and_oracle(pair, n_st):
    p, stored, direct = pair
    u = G.random_coefficients(p.n_det, n_st, p.seed + n_st)
    vd, sd = direct.H_S2_u_0_nstates_openmp(u)
    vs, ss = stored.H_S2_u_0_nstates_openmp(u)
    assert _rel(vd, vs) <= REL64 and _rel(sd, ss) <= REL64
    o = Oracle.from_problem(p)
    vo, so = o.h_s2_u0(u)
    assert _rel(vd, vo) <= REL64 and _rel(sd, so) <= REL64


def test_direct_range_variant(pair):
    p, stored, direct = pair
    u = G.random_coefficients(p.n_det, 2, p.seed)
    order = direct.bilinear_order()
    u_t = np.ascontiguousarray(u[:, order].T)
    istart, iend, ishift, istep = 11, p.n_det - 7, 2, 5
    vd, sd = direct.H_S2_u_0_nstates_openmp_work(u_t, istart, iend, ishift, istep)
    vs, ss = stored.H_S2_u_0_nstates_openmp_work(u_t, istart, iend, ishift, istep)
    rows = np.arange(istart - 1 + ishift, iend, istep)
    mask = np.zeros(p.n_det, bool)
    mask[rows] = True
    assert np.all(vd[~mask] == 0) and np.all(sd[~mask] == 0)
    assert _rel(vd[rows], vs[rows]) <= REL64 and _rel(sd[rows], ss[rows]) <= REL64


def test_direct_davidson(pair):
    p, stored, direct = pair
    rng = np.random.default_rng(3)
    u = rng.normal(size=(4, p.n_det))
    u[0] = 0.0
    u[0, 0] = 1.0
    kw = dict(n_states=2, threshold=1e-12, s2_eig=False, max_iter=400)
    rd = direct.davidson_diag_hs2(u, precision=FP64, **kw)
    rs = stored.davidson_diag_hs2(u, precision=FP64, **kw)
    assert rd["converged"] and rs["converged"]
    np.testing.assert_allclose(rd["energies"][:2], rs["energies"][:2], rtol=0, atol=1e-9)
    # the mixed-precision loop on a direct set (its FP32 sigma requests run in FP64)
    rm = direct.davidson_diag_hs2(u, precision=FP32, **kw)
    assert rm["converged"]
    np.testing.assert_allclose(rm["energies"][:2], rs["energies"][:2], rtol=0, atol=1e-6)


def test_stored_pair_entry_points_refuse_direct_sets(pair):
    p, stored, direct = pair
    with pytest.raises(QPGPUError):
        direct.connected_pairs()


def test_direct_sigma_in_many_chunks(monkeypatch):
    # the direct sigma regenerates the columns chunk by chunk; a small column
    # budget forces hundreds of chunks, with the same results
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(2, n_det=3000)
    monkeypatch.setenv("QPGPU_DIRECT_CHUNK_COLS", "7")
    direct = Wavefunction.from_problem(p, sigma_mode=SIGMA_DIRECT)
    u = G.random_coefficients(p.n_det, 3, p.seed)
    vd, sd = direct.H_S2_u_0_nstates_openmp(u)
    monkeypatch.delenv("QPGPU_DIRECT_CHUNK_COLS")
    vo, so = Oracle.from_problem(p).h_s2_u0(u)
    assert _rel(vd, vo) <= REL64 and _rel(sd, so) <= REL64
