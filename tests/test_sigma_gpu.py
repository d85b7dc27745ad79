"""CUDA sigma path (libqpgpu, through the C-ABI) against the CPU oracle and the golden vectors.

Bars: connected pairs, classes, excitations and phases bit-exact; FP64 matrix
elements bit-exact (the device follows the reference routines' operation
order); FP64 sigma within 1e-12 relative; FP32 (Kahan) sigma within 2e-6
relative of the row scale sum_J |H_IJ u_J|.
"""
import numpy as np
import pytest

from golden_util import load
from oracle import Oracle
from quantum_package_gb300 import FP32, QPGPUError
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu

REL64 = 1e-12
REL32 = 2e-6


def _wf(n_mo, na, nb, ints, dets):
    from quantum_package_gb300.sigma import Wavefunction
    return Wavefunction(n_mo, na, nb, ints.h, ints.eri, dets)


def _assert_sigma(v, ref, rel, what):
    scale = np.abs(ref).max(axis=1, keepdims=True)
    err = np.abs(v - ref).max(axis=1, keepdims=True)
    assert np.all(err <= rel * scale), f"{what}: max rel err {float((err / scale).max()):.3e}"
    nrm = np.linalg.norm(v - ref) / np.linalg.norm(ref)
    assert nrm <= rel, f"{what}: norm rel err {nrm:.3e}"


@pytest.mark.parametrize("name", ["sci_n1", "sci_n2", "fci_s2", "fci_cs"])
def test_golden_sigma(name):
    d = load(name)
    wf = _wf(d["n_mo"], d["n_alpha"], d["n_beta"], d["ints"], d["dets"])
    if "u" in d:
        u, sig, s2 = d["u"], d["sigma"], d["s2sigma"]
    else:
        u = np.random.default_rng(3).normal(size=(2, len(d["dets"])))
        sig, s2 = u @ d["H"], u @ d["S"]
    v, s = wf.H_S2_u_0_nstates_openmp(u)
    _assert_sigma(v, sig, REL64, name)
    np.testing.assert_allclose(s, s2, rtol=0, atol=1e-12)
    if "hdiag" in d:
        h, _ = wf.diag()
        np.testing.assert_allclose(h, d["hdiag"], rtol=0, atol=1e-12 * np.abs(d["hdiag"]).max())


def _problem(cfg, **kw):
    p = G.make_problem(cfg, **kw)
    return p, Oracle.from_problem(p), _wf(p.n_mo, p.n_alpha, p.n_beta, p.ints, p.dets)


@pytest.mark.parametrize("cfg,kw", [(1, dict(n_det=10_000)), (2, dict(n_det=20_000, n_states=4))])
def test_connectivity_bit_exact(cfg, kw):
    p, o, wf = _problem(cfg, **kw)
    I, J, cls = o.connected_pairs()
    g = wf.connected_pairs()
    assert len(g["I"]) == len(I) == wf.info()["n_pairs"]
    np.testing.assert_array_equal(g["I"], I)
    np.testing.assert_array_equal(g["J"], J)
    np.testing.assert_array_equal(g["cls"], cls)
    ph, exc, hij, _ = o.pair_excitations(I, J, cls)
    np.testing.assert_array_equal(g["phase"], ph)
    np.testing.assert_array_equal(g["exc"].astype(np.int32), exc)
    np.testing.assert_array_equal(g["hij"], hij)  # FP64 elements: same operation order
    h, s = wf.diag()
    ho, so = o.diag()
    np.testing.assert_array_equal(h, ho)
    np.testing.assert_array_equal(s, so)
    assert wf.info()["ref_energy"] == o.ref_energy


@pytest.mark.parametrize("cfg,kw", [(1, dict(n_det=10_000)), (2, dict(n_det=20_000, n_states=4))])
def test_sigma_fp64_vs_oracle(cfg, kw):
    p, o, wf = _problem(cfg, **kw)
    u = G.random_coefficients(p.n_det, p.n_states, p.seed)
    v, s = wf.H_S2_u_0_nstates_openmp(u)
    vo, so = o.h_s2_u0(u)
    _assert_sigma(v, vo, REL64, "H u")
    np.testing.assert_allclose(s, so, rtol=0, atol=1e-12 * max(1.0, np.abs(so).max()))


def test_sigma_fp32_kahan_vs_oracle():
    import torch
    p, o, wf = _problem(2, n_det=20_000, n_states=4)
    u = G.random_coefficients(p.n_det, 4, p.seed)
    vo, so = o.h_s2_u0(u)
    dev = torch.device("cuda")
    ut = torch.from_numpy(u).to(dev)
    v = torch.empty_like(ut)
    s = torch.empty_like(ut)
    wf.h_s2_u0_device(v, s, ut, precision=FP32)
    torch.cuda.synchronize()
    _assert_sigma(v.cpu().numpy(), vo, REL32, "FP32 H u")
    np.testing.assert_allclose(s.cpu().numpy(), so, rtol=0, atol=1e-6)


def test_device_fp64_matches_host_entry():
    import torch
    p, o, wf = _problem(1, n_det=5_000)
    u = G.random_coefficients(p.n_det, 3, p.seed)
    vh, sh = wf.H_S2_u_0_nstates_openmp(u)
    ut = torch.from_numpy(u).cuda()
    v = torch.empty_like(ut)
    s = torch.empty_like(ut)
    wf.h_s2_u0_device(v, s, ut)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(v.cpu().numpy(), vh)
    np.testing.assert_array_equal(s.cpu().numpy(), sh)


def test_range_variant_matches_oracle_work():
    p, o, wf = _problem(1, n_det=4_000)
    u = G.random_coefficients(p.n_det, 2, p.seed)
    order = wf.bilinear_order()
    u_t = np.ascontiguousarray(u[:, order].T)  # bilinear order, states fastest
    istart, iend, ishift, istep = 101, 3500, 3, 7
    v, s = wf.H_S2_u_0_nstates_openmp_work(u_t, istart, iend, ishift, istep)
    rows = np.arange(istart - 1 + ishift, iend, istep)
    mask = np.zeros(p.n_det, bool)
    mask[rows] = True
    assert np.all(v[~mask] == 0) and np.all(s[~mask] == 0)
    vfull, _ = wf.H_S2_u_0_nstates_openmp(u)
    np.testing.assert_array_equal(v[rows], vfull[:, order[rows]].T)


def test_edge_cases():
    # single determinant: no pairs, sigma = H_II u
    ints = G.make_integrals(12, 5)
    ref = G.reference_det(12, 3, 3)[None]
    wf = _wf(12, 3, 3, ints, ref)
    assert wf.info()["n_pairs"] == 0
    o = Oracle(12, 3, 3, ints.h, ints.eri, ref)
    v, s = wf.H_S2_u_0_nstates_openmp(np.ones((1, 1)))
    assert v[0, 0] == o.diag()[0][0]
    # one beta string only (a single column), open shell
    d = G.full_ci_dets(8, 3, 1)
    d = d[d[:, 1, 0] == d[0, 1, 0]]
    ints8 = G.make_integrals(8, 6)
    wf = _wf(8, 3, 1, ints8, d)
    o = Oracle(8, 3, 1, ints8.h, ints8.eri, d)
    u = np.random.default_rng(0).normal(size=(1, len(d)))
    _assert_sigma(wf.H_S2_u_0_nstates_openmp(u)[0], o.h_s2_u0(u)[0], REL64, "single column")
    # n_mo = 64 (one full word), 65 (second word with a single bit) and 128
    # (the largest supported space: both words full)
    for n in (64, 65, 128):
        p = G.make_problem(1, n_det=3000, n_mo=n, n_alpha=6, n_beta=5)
        wf = _wf(p.n_mo, 6, 5, p.ints, p.dets)
        o = Oracle.from_problem(p)
        u = G.random_coefficients(p.n_det, 2, 1)
        _assert_sigma(wf.H_S2_u_0_nstates_openmp(u)[0], o.h_s2_u0(u)[0], REL64, f"n_mo={n}")
        g = wf.connected_pairs()
        I, J, cls = o.connected_pairs()
        np.testing.assert_array_equal(g["J"], J)


def test_invalid_inputs_raise():
    ints = G.make_integrals(10, 2)
    from quantum_package_gb300.sigma import Wavefunction
    wf = Wavefunction(10, 3, 3, ints.h, ints.eri)
    bad = G.reference_det(10, 3, 3)[None].copy()
    bad[0, 0, 0] |= np.uint64(1 << 9)  # 4 alpha electrons
    with pytest.raises(QPGPUError):
        wf.set_dets(bad)
    with pytest.raises(QPGPUError):
        wf.H_S2_u_0_nstates_openmp(np.ones((1, 1)))  # no determinants yet
    bad = G.reference_det(10, 3, 3)[None].copy()
    bad[0, 1, 0] = np.uint64((1 << 12) | 3)  # orbital 13 > n_mo
    with pytest.raises(QPGPUError):
        wf.set_dets(bad)
    with pytest.raises(QPGPUError):  # empty determinant set
        wf.set_dets(np.zeros((0, 2, 1), np.uint64))


def test_u0_h_u0_matches_oracle():
    # u_0_H_u_0 (diagonalization_hs2.irp.f:446-484): <u|H|u> per column, not
    # divided by <u|u>; a zero column gives 0
    p, o, wf = _problem(2, n_det=5_000)
    u = G.random_coefficients(p.n_det, 3, p.seed)
    u[1] = 0.0
    e = wf.u_0_H_u_0(u)
    v, _ = o.h_s2_u0(u)
    ref = np.einsum("ij,ij->i", u, v)
    assert e[1] == 0.0
    np.testing.assert_allclose(e[[0, 2]], ref[[0, 2]], rtol=REL64, atol=0)


def test_sigma_float_float_vs_fp64():
    # QPGPU_FF: float-float elements, coefficients and sums on the FP32 pipes
    import torch
    from quantum_package_gb300 import FF, FP64
    p, o, wf = _problem(2, n_det=20_000, n_states=4)
    for n_st in (1, 2, 3, 5, 8):
        u = G.random_coefficients(p.n_det, n_st, p.seed + n_st)
        order = wf.bilinear_order()
        ut = torch.from_numpy(np.ascontiguousarray(u[:, order].T)).cuda()
        v64, s64, vff, sff = (torch.empty_like(ut) for _ in range(4))
        wf.sigma_bilinear(v64, s64, ut, None, FP64)
        wf.sigma_bilinear(vff, sff, ut, None, FF)
        torch.cuda.synchronize()
        a, b = v64.cpu().numpy(), vff.cpu().numpy()
        _assert_sigma(b.T, a.T, REL64, f"FF n_st={n_st}")
        _assert_sigma(sff.cpu().numpy().T, s64.cpu().numpy().T, REL64, f"FF S2 n_st={n_st}")


def test_nonfinite_inputs_give_numeric_error():
    # NaN / Inf in a host input vector: QPGPU_ERR_NUMERIC (-7) from every
    # host-array entry point, and the context stays usable afterwards
    p, o, wf = _problem(1, n_det=2_000)
    u = G.random_coefficients(p.n_det, 2, p.seed)
    bad = u.copy()
    bad[1, 17] = np.nan
    inf = u.copy()
    inf[0, 3] = np.inf
    for x in (bad, inf):
        with pytest.raises(QPGPUError) as e:
            wf.H_S2_u_0_nstates_openmp(x)
        assert e.value.code == -7
        with pytest.raises(QPGPUError) as e:
            wf.u_0_H_u_0(x)
        assert e.value.code == -7
        order = wf.bilinear_order()
        with pytest.raises(QPGPUError) as e:
            wf.H_S2_u_0_nstates_openmp_work(np.ascontiguousarray(x[:, order].T), 1, p.n_det)
        assert e.value.code == -7
    g = np.random.default_rng(0).normal(size=(4, p.n_det))
    g[2, 5] = np.nan
    with pytest.raises(QPGPUError) as e:
        wf.davidson_diag_hs2(g, n_states=1, s2_eig=False)
    assert e.value.code == -7
    v, _ = wf.H_S2_u_0_nstates_openmp(u)
    _assert_sigma(v, o.h_s2_u0(u)[0], REL64, "after the refused calls")
