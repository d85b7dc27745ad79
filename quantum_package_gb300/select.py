"""CIPSI selection on the device: the generator / selector counts and one
selection step over a wave function.

* ``n_det_generators`` (plugins/Generators_full/generators.irp.f:3-22): the
  first i whose running sum of psi_average_norm_contrib_sorted reaches
  threshold_generators (>=), at least 1.
* ``n_det_selectors`` (plugins/Selectors_full/selectors.irp.f:3-25): the
  first i whose running sum exceeds threshold_selectors (>), at least
  N_det_generators.  It is every determinant when threshold_generators >= 1.
* ``select`` sorts the wave function (psi_det_sorted, the reference's
  dsort), counts generators and selectors, and runs qpgpu_select_pt2 on the
  device.  It returns the second-order energy of every state and the most
  negative buffer entries: the determinants a CIPSI iteration adds
  (selection_buffer.irp.f, Full_CI_ZMQ).
"""
from __future__ import annotations

import numpy as np

from . import ezfio as _ezfio


def _running_sum(x):
    # the reference's loop: norm = norm + contrib(i), in order
    return np.cumsum(np.asarray(x, dtype=np.float64))


def n_det_generators(contrib_sorted, threshold_generators=0.99):
    c = _running_sum(contrib_sorted)
    hit = np.nonzero(c >= threshold_generators)[0]
    n = int(hit[0]) + 1 if len(hit) else len(c)
    return max(n, 1)


def n_det_selectors(contrib_sorted, n_gen, threshold_selectors=0.999, threshold_generators=0.99):
    n = len(contrib_sorted)
    if threshold_generators < 1.0:
        c = _running_sum(contrib_sorted)
        hit = np.nonzero(c > threshold_selectors)[0]
        if len(hit):
            n = int(hit[0]) + 1
        n = max(n, n_gen)
    return n


def select(make_wf, dets, coefs, e0, buf_size, threshold_generators=0.99, threshold_selectors=0.999,
           weights=None):
    """One selection over the wave function (dets [N][2][N_int], coefs
    [N][n_st]).  ``make_wf(sorted_dets)`` builds the device wave function
    (a Wavefunction over those determinants).  Returns dict(pt2, dets, vals,
    n_ext, n_gen, n_sel, order)."""
    coefs = np.asarray(coefs, dtype=np.float64).reshape(len(dets), -1)
    order = _ezfio.sorted_order(coefs, weights)
    contrib = _ezfio.average_norm_contrib(coefs, weights)[order]
    n_gen = n_det_generators(contrib, threshold_generators)
    n_sel = n_det_selectors(contrib, n_gen, threshold_selectors, threshold_generators)
    wf = make_wf(np.ascontiguousarray(np.asarray(dets)[order]))
    try:
        pt2, bd, bv, n_ext = wf.select_pt2(np.ascontiguousarray(coefs[order].T), e0, n_gen, n_sel, buf_size)
    finally:
        wf.close()
    return dict(pt2=pt2, dets=bd, vals=bv, n_ext=n_ext, n_gen=n_gen, n_sel=n_sel, order=order)


def pt2_stochastic(make_wf, dets, coefs, e0, relative_error=1e-3, absolute_error=0.0, seed=0, batch=256,
                   threshold_generators=0.99, threshold_selectors=0.999):
    """ZMQ_pt2 over the wave function (dets, coefs [N][n_st]): the comb
    estimate of every state's second-order energy with its error.  As the
    reference, each state gets its own psi_det_sorted (state_average_weight
    set to that state alone), hence its own generators and selectors.
    Below max(10, n_st) determinants the full selection gives the exact sum.
    The per-generator contributions are computed on the device in batches.
    Returns dict(pt2, error, n_computed, n_combs, n_gen, n_sel) with
    per-state lists."""
    from . import pt2 as _pt2
    coefs = np.asarray(coefs, dtype=np.float64).reshape(len(dets), -1)
    n_st = coefs.shape[1]
    e0 = np.asarray(e0, dtype=np.float64)
    if len(dets) < max(10, n_st):
        r = select(make_wf, dets, coefs, e0, 0, threshold_generators, threshold_selectors)
        return dict(pt2=r["pt2"], error=np.zeros(n_st), n_computed=[r["n_gen"]] * n_st, n_combs=[0] * n_st,
                    n_gen=[r["n_gen"]] * n_st, n_sel=[r["n_sel"]] * n_st)
    out = dict(pt2=np.zeros(n_st), error=np.zeros(n_st), n_computed=[], n_combs=[], n_gen=[], n_sel=[])
    for st in range(n_st):
        w = np.zeros(n_st)
        w[st] = 1.0
        order = _ezfio.sorted_order(coefs, w)
        contrib = _ezfio.average_norm_contrib(coefs, w)[order]
        n_gen = n_det_generators(contrib, threshold_generators)
        n_sel = n_det_selectors(contrib, n_gen, threshold_selectors, threshold_generators)
        cs = np.ascontiguousarray(coefs[order])
        wf = make_wf(np.ascontiguousarray(np.asarray(dets)[order]))
        try:
            r = _pt2.pt2_stochastic(lambda g: wf.pt2_generators(cs.T, e0, n_sel, g)[:, st:st + 1],
                                    cs[:n_gen, st], n_det=len(dets), relative_error=relative_error,
                                    absolute_error=absolute_error, seed=seed + st, batch=batch)
        finally:
            wf.close()
        out["pt2"][st] = r["pt2"][0]
        out["error"][st] = r["error"][0]
        for k in ("n_computed", "n_combs"):
            out[k].append(r[k])
        out["n_gen"].append(n_gen)
        out["n_sel"].append(n_sel)
    return out
