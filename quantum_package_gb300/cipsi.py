"""The CIPSI loop of the Full_CI program (plugins/Full_CI_ZMQ/fci_zmq.irp.f)
over the device library: diagonalise, select, grow, until N_det_max or a
small enough second-order energy.

* ``run`` restates fci_zmq:
  * diagonalize_CI of the starting wave function;
  * then, while N_det < N_det_max and max_st |pt2| > pt2_max, each
    iteration does the following:
    * optionally the stochastic PT2 with every determinant a generator
      and a selector (``do_pt2``), as the loop computes it;
    * a selection of to_select = N_det determinants (N_det / 2 + 1 with
      s2_eig), at most N_det_max - N_det. The denominator is psi_energy,
      i.e. pt2_E0_denominator (Full_CI_ZMQ/energy.irp.f);
    * the new determinants appended with zero coefficients
      (fill_H_apply_buffer_no_selection / copy_H_apply_buffer_to_wf);
    * a spin completion with s2_eig or several states
      (make_s2_eigenfunction);
    * diagonalize_CI from the previous coefficients.
  * The PT2 of an iteration is the selection's own (the reference's
    "(approx)") unless ``do_pt2`` asks for the stochastic one.
* ``make_s2_eigenfunction`` (src/Determinants/occ_pattern.irp.f:251-300)
  adds, for every occupation pattern of the wave function, the
  determinants of that pattern with N_alpha electrons that are missing: the
  alpha / beta assignments of the singly occupied orbitals.

The device work is sigma / the Davidson (through ``ci``) and the selection
(through ``select``). This module is host logic over them.
"""
from __future__ import annotations

from itertools import combinations

import numpy as np

from . import ci as _ci
from . import select as _select


def make_s2_eigenfunction(dets, n_alpha):
    """The determinants of every occupation pattern of ``dets`` (N, 2, N_int)
    with n_alpha alpha electrons, the missing ones appended after the given
    ones in pattern order.  Returns (all determinants, number added)."""
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    nint = dets.shape[2]
    have = {d.tobytes() for d in dets}
    seen = set()
    new = []
    for d in dets:
        a = [int(x) for x in d[0]]
        b = [int(x) for x in d[1]]
        docc = [a[w] & b[w] for w in range(nint)]
        socc = [a[w] ^ b[w] for w in range(nint)]
        key = tuple(docc + socc)
        if key in seen:
            continue
        seen.add(key)
        opens = [64 * w + o for w in range(nint) for o in range(64) if (socc[w] >> o) & 1]
        n_docc = sum(bin(x).count("1") for x in docc)
        k = n_alpha - n_docc
        if k < 0 or k > len(opens):
            continue
        for up in combinations(opens, k):
            aw = list(docc)
            bw = list(docc)
            ups = set(up)
            for o in opens:
                if o in ups:
                    aw[o >> 6] |= 1 << (o & 63)
                else:
                    bw[o >> 6] |= 1 << (o & 63)
            x = np.array([aw, bw], dtype=np.uint64)
            kb = x.tobytes()
            if kb not in have:
                have.add(kb)
                new.append(x)
    if not new:
        return dets, 0
    return np.concatenate([dets, np.stack(new)], axis=0), len(new)


def run(make_wf, dets0, n_states, n_det_max, pt2_max=1e-4, n_states_diag=None, s2_eig=False, do_pt2=False,
        threshold_davidson=1e-12, threshold_generators=0.99, threshold_selectors=0.999, pt2_relative_error=1e-3,
        davidson_sze_max=8, max_iterations=100, seed=0, log=None):
    """fci_zmq over the device library.  ``make_wf(dets)`` builds the device
    wave function (a Wavefunction) of a determinant set.  Returns dict(dets,
    coefs (N, n_states), energies (electronic), pt2, pt2_error, history)
    where history lists (N_det, energies, pt2, pt2_error) per iteration."""
    nst = n_states
    nsd = max(nst, n_states_diag or nst)

    def diagonalize(dets, coefs):
        wf = make_wf(dets)
        try:
            new, res = _ci.diagonalize_ci(wf, coefs, nst, n_states_diag=min(nsd, len(dets)), s2_eig=s2_eig,
                                          threshold=threshold_davidson, davidson_sze_max=davidson_sze_max,
                                          seed=seed)
        finally:
            wf.close()
        return new, np.asarray(res["energies"][:nst])

    dets = np.ascontiguousarray(dets0, dtype=np.uint64)
    coefs = _ci.psi_coef_guess(len(dets), nst)
    coefs, e = diagonalize(dets, coefs)
    pt2 = np.full(nst, -np.inf)
    err = np.zeros(nst)
    history = []
    it = 0
    while len(dets) < n_det_max and np.max(np.abs(pt2)) > pt2_max and it < max_iterations:
        it += 1
        if do_pt2:
            r = _select.pt2_stochastic(make_wf, dets, coefs, e, relative_error=pt2_relative_error, seed=seed + it,
                                       threshold_generators=1.0, threshold_selectors=1.0)
            pt2, err = np.asarray(r["pt2"]), np.asarray(r["error"])
        n_before = len(dets)
        to_select = (n_before // 2 + 1) if s2_eig else n_before
        to_select = min(to_select, n_det_max - n_before)
        sel = _select.select(make_wf, dets, coefs, e, to_select, threshold_generators, threshold_selectors)
        if not do_pt2:
            pt2, err = np.asarray(sel["pt2"]), np.zeros(nst)
        history.append(dict(n_det=n_before, energies=e.copy(), pt2=pt2.copy(), pt2_error=err.copy(),
                            n_gen=sel["n_gen"], n_sel=sel["n_sel"], n_ext=sel["n_ext"]))
        if log:
            log(history[-1])
        if len(sel["dets"]) == 0:
            break
        dets = np.concatenate([dets, sel["dets"]], axis=0)
        coefs = np.concatenate([coefs, np.zeros((len(sel["dets"]), nst))], axis=0)
        if s2_eig or nst > 1:
            n_alpha = sum(bin(int(w)).count("1") for w in dets[0, 0])
            dets, added = make_s2_eigenfunction(dets, n_alpha)
            if added:
                coefs = np.concatenate([coefs, np.zeros((added, nst))], axis=0)
        coefs, e = diagonalize(dets, coefs)
    return dict(dets=dets, coefs=coefs, energies=e, pt2=pt2, pt2_error=err, history=history)
