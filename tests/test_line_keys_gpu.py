"""Deletion-key tables of heavy lines (qpgpu_set_line_keys): the pair scans
probe a line's strings by deletion keys instead of testing every string of the
line (the reference's loops, u0Hu0.irp.f:177-332, test them all).  The pairs
must be exactly those of the plain scans.

Bars: with a table on every line, the connected pairs (I, J, class, phase,
excitation, FP64 element) are bit-exact against the oracle, also with the key
hashes cut to 6 bits so that thousands of distinct keys share one group; the
direct sigma with tables matches the stored sigma without them to 1e-12; with
the default thresholds a set whose reference column holds ~2.5e4 determinants
gets tables, and its pairs equal those of the same set without tables.
"""
import numpy as np
import pytest

from oracle import Oracle
from quantum_package_gb300 import FP64, KEYS_OFF, SIGMA_DIRECT, SIGMA_STORED, QPGPUError
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu

REL64 = 1e-12


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("cfg,n,bits", [(1, 10_000, 64), (2, 20_000, 64), (1, 4_000, 6), (2, 3_000, 6)],
                         ids=["nint1", "nint2", "nint1-collide", "nint2-collide"])
def test_every_line_keyed_pairs_bit_exact(cfg, n, bits):
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(cfg, n_det=n)
    wf = Wavefunction.from_problem(p, sigma_mode=SIGMA_STORED, line_keys=(0, 0, bits))
    info = wf.info()
    assert info["n_keyed_lines"] == info["n_alpha_unique"] + info["n_beta_unique"]
    o = Oracle.from_problem(p)
    I, J, cls = o.connected_pairs()
    g = wf.connected_pairs()
    np.testing.assert_array_equal(g["I"], I)
    np.testing.assert_array_equal(g["J"], J)
    np.testing.assert_array_equal(g["cls"], cls)
    ph, exc, hij, _ = o.pair_excitations(I, J, cls)
    np.testing.assert_array_equal(g["phase"], ph)
    np.testing.assert_array_equal(g["exc"].astype(np.int32), exc)
    np.testing.assert_array_equal(g["hij"], hij)
    u = G.random_coefficients(p.n_det, 3, p.seed)
    v, s = wf.H_S2_u_0_nstates_openmp(u)
    vo, so = o.h_s2_u0(u)
    assert _rel(v, vo) <= REL64 and _rel(s, so) <= REL64


@pytest.mark.parametrize("cfg,n", [(1, 3000), (2, 5000)], ids=["nint1", "nint2"])
def test_direct_sigma_with_keys(cfg, n):
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(cfg, n_det=n)
    direct = Wavefunction.from_problem(p, sigma_mode=SIGMA_DIRECT, line_keys=(0, 0, 64))
    stored = Wavefunction.from_problem(p, sigma_mode=SIGMA_STORED, line_keys=(KEYS_OFF, KEYS_OFF, 64))
    assert direct.info()["n_keyed_lines"] > 0 and stored.info()["n_keyed_lines"] == 0
    assert direct.info()["n_pairs"] == stored.info()["n_pairs"]
    u = G.random_coefficients(p.n_det, 4, p.seed + 1)
    vd, sd = direct.H_S2_u_0_nstates_openmp(u)
    vs, ss = stored.H_S2_u_0_nstates_openmp(u)
    assert _rel(vd, vs) <= REL64 and _rel(sd, ss) <= REL64
    rng = np.random.default_rng(3)
    g = rng.normal(size=(4, p.n_det))
    kw = dict(n_states=2, threshold=1e-12, s2_eig=False, max_iter=400, precision=FP64)
    rd = direct.davidson_diag_hs2(g, **kw)
    rs = stored.davidson_diag_hs2(g, **kw)
    assert np.abs(rd["energies"][:2] - rs["energies"][:2]).max() < 1e-9


def test_default_thresholds_key_the_heavy_column():
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(2, n_det=100_000)
    keyed = Wavefunction.from_problem(p, sigma_mode=SIGMA_STORED)
    plain = Wavefunction.from_problem(p, sigma_mode=SIGMA_STORED, line_keys=(KEYS_OFF, KEYS_OFF, 64))
    ik, ip = keyed.info(), plain.info()
    assert ik["n_keyed_lines"] >= 2 and ip["n_keyed_lines"] == 0
    assert ik["n_pairs"] == ip["n_pairs"] and ik["n_s2_pairs"] == ip["n_s2_pairs"]
    # the heavy column's rows (beta = reference) and a spread of others
    ref_b = p.dets[0, 1]
    heavy = np.nonzero(np.all(p.dets[:, 1] == ref_b, axis=1))[0]
    rows = np.unique(np.concatenate([heavy[:: max(1, len(heavy) // 400)], np.arange(0, p.n_det, 997)]))
    assert len(heavy) > 16384
    a, b = keyed.connected_pairs_rows(rows), plain.connected_pairs_rows(rows)
    for k in ("I", "J", "cls", "phase", "exc", "hij"):
        np.testing.assert_array_equal(a[k], b[k])
    u = G.random_coefficients(p.n_det, 2, p.seed)
    v1, s1 = keyed.H_S2_u_0_nstates_openmp(u)
    v2, s2 = plain.H_S2_u_0_nstates_openmp(u)
    assert _rel(v1, v2) <= REL64 and _rel(s1, s2) <= REL64


def test_line_keys_argument_checks():
    from quantum_package_gb300.sigma import Wavefunction
    wf = Wavefunction(40, 10, 10)
    with pytest.raises(QPGPUError):
        wf.set_line_keys(-2, 0, 64)
    with pytest.raises(QPGPUError):
        wf.set_line_keys(0, 0, 0)
    with pytest.raises(QPGPUError):
        wf.set_line_keys(0, 0, 65)
    wf.set_line_keys(-1, -1, 64)
