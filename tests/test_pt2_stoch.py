"""Stochastic second-order energy: the comb estimator of
plugins/Full_CI_ZMQ/pt2_stoch_routines.irp.f, restated in
quantum_package_gb300/pt2.py, over the device's per-generator contributions
(qpgpu_pt2_generators).

CPU (synthetic per-generator contributions, exact sum known):
* the vectorised pt2_find equals the scalar restatement of the reference's
  bisection (:352-378);
* the comb set-up follows the pt2_weight provider: the deterministic set,
  the teeth, the first weight normalised as written;
* the work list reaches every generator once;
* the estimate is unbiased over seeds, and its error bar matches the spread.
GPU:
* the per-generator contributions add up to qpgpu_select_pt2's sum and to
  the oracle's (1e-12);
* the device-driven comb estimate lies within 4 error bars of that exact
  sum.
"""
import numpy as np
import pytest

from quantum_package_gb300 import pt2 as P


def _synthetic(n, seed, decay):
    rng = np.random.default_rng(seed)
    c = np.sort(np.abs(rng.normal(size=n)) * np.exp(-np.arange(n) / decay))[::-1]
    c = c / np.linalg.norm(c) * 0.97
    detail = -(c ** 2) * np.abs(1 + 0.5 * rng.normal(size=n)) * 0.3
    return c, detail


def test_pt2_find_vectorised_equals_scalar():
    rng = np.random.default_rng(5)
    w = np.concatenate([[0.0], np.sort(rng.random(4000))])
    w[-1] = 1.0
    v = rng.random(5000)
    lo = rng.integers(1, 2000, size=5000)
    hi = lo + rng.integers(1, 2000, size=5000)
    b = np.array([P.pt2_find(v[i], w, lo[i], hi[i]) for i in range(5000)])
    np.testing.assert_array_equal(P.pt2_find_many(v, w, lo, hi), b)


def test_comb_setup_and_work_list():
    c, _ = _synthetic(2000, 1, 200)
    comb = P.Comb(c)
    assert comb.first_det_of_comb >= 2
    fdt = comb.first_det_of_teeth
    assert fdt[1] == comb.first_det_of_comb and fdt[comb.teeth + 1] == comb.n + 1
    assert np.all(np.diff(fdt[1:]) >= 0)
    assert np.all(np.diff(comb.cw[1:comb.n + 1]) >= 0) and comb.cw[comb.n] == 1.0
    # only the first weight is normalised (the loop divides by cw(1) = 1 afterwards)
    np.testing.assert_allclose(comb.w[1], c[0] ** 2 / np.sum(c ** 2), rtol=1e-14)
    np.testing.assert_array_equal(comb.w[2:], c[1:] * c[1:])
    _, teeth, tbc = comb.workbatch(np.random.default_rng(0))
    assert sorted(tbc) == list(range(1, comb.n + 1))  # every generator, once
    assert tbc[:comb.first_det_of_comb - 1] == list(range(1, comb.first_det_of_comb))
    # every tooth's generator lies in its tooth
    for j in (1, 50, comb.teeth):
        assert np.all((teeth[:, j] >= fdt[j]) & (teeth[:, j] <= fdt[j + 1]))


def test_estimator_unbiased_with_calibrated_errors():
    c, detail = _synthetic(3000, 2, 300)
    exact = detail.sum()
    comp = lambda g: detail[g][:, None]
    runs = [P.pt2_stochastic(comp, c, relative_error=1e-3, seed=s) for s in range(60)]
    avg = np.array([r["pt2"][0] for r in runs])
    err = np.array([r["error"][0] for r in runs])
    z = (avg.mean() - exact) / (avg.std() / np.sqrt(len(avg)))
    assert abs(z) < 3.0, z
    assert 0.5 < avg.std() / err.mean() < 2.0
    assert np.mean([r["n_computed"] for r in runs]) < 0.5 * len(c)  # sampling, not the full sum
    # relative_error = 0: every comb used; the error bar is the smallest
    full = P.pt2_stochastic(comp, c, relative_error=0.0, seed=7)
    assert full["n_computed"] == len(c) and abs(full["pt2"][0] - exact) < 4 * full["error"][0]


def test_small_sets_are_exact():
    c, detail = _synthetic(8, 3, 2)
    r = P.pt2_stochastic(lambda g: detail[g][:, None], c, n_det=8)
    assert r["error"][0] == 0.0 and r["pt2"][0] == pytest.approx(detail.sum(), abs=1e-15)


@pytest.mark.gpu
def test_device_pt2_generators_and_comb_estimate():
    from oracle import Oracle
    from quantum_package_gb300 import ezfio, select as S
    from quantum_package_gb300.sigma import Wavefunction
    p = __import__("quantum_package_gb300.generate", fromlist=["x"]).make_problem(1, n_det=400, n_mo=26, n_alpha=5,
                                                                                   n_beta=5)
    H, _ = Oracle.from_problem(p).dense(with_s2=False)
    w, V = np.linalg.eigh(H)
    coefs = V[:, :1]
    order = ezfio.sorted_order(coefs)
    dets = np.ascontiguousarray(p.dets[order])
    cs = np.ascontiguousarray(coefs[order].T)
    n_gen = n_sel = 400  # every determinant a generator and a selector
    wf = Wavefunction(p.n_mo, 5, 5, p.ints.h, p.ints.eri, dets)
    detail = wf.pt2_generators(cs, w[:1], n_sel, np.arange(n_gen))
    pt2, _, _, _ = wf.select_pt2(cs, w[:1], n_gen, n_sel, 0)
    o = Oracle(p.n_mo, 5, 5, p.ints.h, p.ints.eri, dets)
    pt2o, _, _, _ = o.select_pt2(cs, w[:1], n_gen, n_sel, 0)
    np.testing.assert_allclose(detail.sum(axis=0), pt2, rtol=0, atol=1e-12 * abs(pt2[0]))
    np.testing.assert_allclose(pt2, pt2o, rtol=0, atol=1e-12 * abs(pt2o[0]))
    # a subset, in any order: the same per-generator values
    sub = np.array([399, 3, 250, 17])
    np.testing.assert_allclose(wf.pt2_generators(cs, w[:1], n_sel, sub), detail[sub], rtol=0,
                               atol=1e-13 * abs(pt2[0]))
    wf.close()
    make = lambda dd: Wavefunction(p.n_mo, 5, 5, p.ints.h, p.ints.eri, dd)
    # a flat coefficient vector (not an eigenvector), so that the comb samples
    rng = np.random.default_rng(11)
    flat = (np.exp(-np.arange(400) / 150.0) * rng.choice([-1.0, 1.0], 400))[:, None]
    flat /= np.linalg.norm(flat)
    o2 = np.argsort(-flat[:, 0] ** 2, kind="stable")
    d2 = np.ascontiguousarray(p.dets[o2])
    exact = Oracle(p.n_mo, 5, 5, p.ints.h, p.ints.eri, d2).select_pt2(np.ascontiguousarray(flat[o2].T), w[:1],
                                                                        400, 400, 0)[0][0]
    r = S.pt2_stochastic(make, p.dets, flat, w[:1], relative_error=5e-3, seed=3, batch=32,
                         threshold_generators=1.0, threshold_selectors=1.0)
    assert r["n_gen"][0] == 400 and r["n_combs"][0] >= 5
    assert r["error"][0] > 0.0
    assert abs(r["pt2"][0] - exact) < 4 * r["error"][0] + 1e-11 * abs(exact), (r["pt2"][0], exact, r["error"][0])
