"""Stochastic second-order energy (the comb estimator of
plugins/Full_CI_ZMQ/pt2_stoch_routines.irp.f) over the device selection.

The exact PT2 of a state is the sum over generators of pt2_detail(g): the
second-order contributions of the external determinants first reached by
generator g.  qpgpu_pt2_generators computes pt2_detail for a list of
generators on the device.  The reference samples generators instead of
computing all of them:

* weights (the pt2_weight provider, :459-510): w_i = c_i^2 of the state's
  generator coefficients, cumulative weights taken backwards.  The
  normalisation loop divides by pt2_cweight(1), which is already 1 after
  its first pass, so only the first weight is normalised.  This is restated
  as written; the comb positions use the cumulative weights
  1 - cw(i + 1), which stay consistent.
* deterministic set (:486-497): the leading generators whose weight is at
  least half a comb step of the norm left (at least one generator).  The
  comb step then shrinks to the weight of the rest, and tooth j starts at
  first_det_of_teeth(j) (pt2_find, :352-378, restated with its bisection as
  written);
* combs (get_carlo_workbatch / get_comb / add_comb, :422-479): a uniform
  offset in [0, comb_step) picks one generator per tooth.  The work list
  gets the new generators of each comb plus the next generator in order not
  yet computed;
* estimator (do_carlo :157-180, pt2_collector :199-350): each comb
  accumulates pt2_detail(d) / w_d * comb_step from the last tooth down, into
  sums per starting tooth.  The estimate is the exact sum over the
  generators before the first incomplete tooth, plus that tooth's share, plus
  the mean of the comb sums from that tooth; the error is the standard error
  of that mean.  It stops when |error / estimate| < relative_error or
  |error| < absolute_error, or when every comb is done;
* states (ZMQ_pt2, :6-155): one comb run per state, with that state's
  weights.  Below max(10, N_states) determinants the sum is exact.

The device computes the work list in batches of generators.  The stopping
rule is checked after each batch, where the reference checks every 10 s.
The uniform offsets come from numpy's generator with a seed, where the
reference calls Fortran's RANDOM_NUMBER.
"""
from __future__ import annotations

import numpy as np

COMB_TEETH = 100


def pt2_find(v, w, imin, imax):
    """pt2_find (pt2_stoch_routines.irp.f:352-378), 1-based indices into w
    (w[0] unused): bisection while the range is >= 64 wide, then the first i
    in [l, h] with w(i) >= v, else h + 1."""
    block = 64
    l, h = imin, imax - 1
    while h - l >= block:
        i = (h + l) >> 1
        if w[i + 1] > v:
            h = i - 1
        else:
            l = i + 1
    for i in range(l, h + 1):
        if w[i] >= v:
            return i
    return h + 1


def pt2_find_many(v, w, imin, imax):
    """pt2_find for arrays v, imin, imax (same bisection per element).  w is
    non-decreasing (cumulative weights), so the linear tail's first
    w(i) >= v in [l, h] is a sorted search clipped to [l, h + 1]."""
    v = np.asarray(v, dtype=np.float64)
    l = np.broadcast_to(np.asarray(imin, dtype=np.int64), v.shape).copy()
    h = np.broadcast_to(np.asarray(imax, dtype=np.int64), v.shape).copy() - 1
    while True:
        m = (h - l) >= 64
        if not m.any():
            break
        i = (h + l) >> 1
        up = w[np.where(m, i + 1, 0)] > v
        h = np.where(m & up, i - 1, h)
        l = np.where(m & ~up, i + 1, l)
    k = np.searchsorted(w[1:], v, side="left") + 1  # first 1-based index with w >= v
    return np.clip(k, l, h + 1)


class Comb:
    """The pt2_weight provider for one state: weights, cumulative weights,
    the deterministic set and the teeth (1-based arrays, index 0 unused)."""

    def __init__(self, coef_gen, teeth=COMB_TEETH):
        c = np.asarray(coef_gen, dtype=np.float64)
        n = len(c)
        self.n, self.teeth = n, teeth
        w = np.zeros(n + 1)
        cw = np.zeros(n + 2)
        for i in range(1, n + 1):
            w[i] = c[i - 1] * c[i - 1]  # Fortran x**2 is x*x
        cw[n] = w[n]
        for i in range(n - 1, 0, -1):
            cw[i] = w[i] + cw[i + 1]
        for i in range(1, n + 1):  # as written: cw(1) is 1 from the second pass on
            w[i] = w[i] / cw[1]
            cw[i] = cw[i] / cw[1]
        for i in range(1, n):
            cw[i] = 1.0 - cw[i + 1]
        cw[n] = 1.0
        norm_left = 1.0
        step = 1.0 / teeth
        fdc = 1
        for i in range(1, n + 1):
            if w[i] / norm_left < 0.5 * step:
                fdc = i
                break
            norm_left -= w[i]
        fdc = max(2, fdc)
        step = (1.0 - cw[fdc - 1]) * step
        fdt = np.zeros(teeth + 2, dtype=np.int64)
        stato = 1.0 - step
        iloc = n
        for i in range(teeth, 0, -1):
            iloc = pt2_find(stato, cw, 1, iloc)
            fdt[i] = iloc
            stato -= step
        fdt[teeth + 1] = n + 1
        fdt[1] = fdc
        self.w, self.cw, self.step, self.first_det_of_comb, self.first_det_of_teeth = w, cw, step, fdc, fdt
        with np.errstate(divide="ignore"):
            self.w_inv = np.where(w != 0.0, 1.0 / np.where(w != 0.0, w, 1.0), np.inf)

    def get_comb(self, stato):
        """get_comb: the generator of every tooth (1-based), index by tooth."""
        dets = np.zeros(self.teeth + 1, dtype=np.int64)
        curs = 1.0 - stato
        for j in range(self.teeth, 0, -1):
            dets[j] = pt2_find(curs, self.cw, self.first_det_of_teeth[j], self.first_det_of_teeth[j + 1])
            curs -= self.step
        return dets

    def get_combs(self, stato):
        """get_comb of many offsets at once: (len(stato), teeth + 1)."""
        st = np.asarray(stato, dtype=np.float64)
        t = self.teeth
        # curs of tooth j: 1 - stato - (teeth - j) comb_step, formed as the
        # reference's repeated subtraction
        curs = np.empty((len(st), t + 1))
        cur = 1.0 - st
        for j in range(t, 0, -1):
            curs[:, j] = cur
            cur = cur - self.step
        dets = np.zeros((len(st), t + 1), dtype=np.int64)
        for j in range(1, t + 1):
            dets[:, j] = pt2_find_many(curs[:, j], self.cw, self.first_det_of_teeth[j], self.first_det_of_teeth[j + 1])
        return dets

    def workbatch(self, rng):
        """get_carlo_workbatch: (comb offsets, their teeth, work list tbc of
        1-based generators in order).  The deterministic set comes first."""
        n = self.n
        computed = np.zeros(n + 2, dtype=bool)
        tbc = list(range(1, self.first_det_of_comb))
        computed[1:self.first_det_of_comb] = True
        comb = rng.random(n) * self.step
        teeth = self.get_combs(comb)
        ncomb = 0
        l = self.first_det_of_comb
        for i in range(n):
            d = teeth[i, 1:]
            new = d[~computed[d]]
            if len(new):
                # in tooth order, each generator once
                _, first = np.unique(new, return_index=True)
                new = new[np.sort(first)]
                tbc.extend(int(x) for x in new)
                computed[new] = True
            ncomb = i + 1
            if len(tbc) == n:
                break
            while computed[l]:
                l += 1
            tbc.append(l)
            computed[l] = True
        return comb[:ncomb], teeth[:ncomb], tbc


class Estimator:
    """do_carlo and the estimate / error of pt2_collector for one state."""

    def __init__(self, comb: Comb, teeth_of_combs):
        self.c = comb
        self.dets = teeth_of_combs  # (n_comb, teeth + 1) from Comb.get_combs
        self.first = 0  # first comb not yet accumulated
        t = comb.teeth
        self.sumabove = np.zeros(t + 1)
        self.sum2above = np.zeros(t + 1)
        self.nabove = np.zeros(t + 1)

    def do_carlo(self, detail, computed):
        """The combs from the first not yet counted up to the first with a
        generator not computed: myVal from the last tooth down, into the sums
        of every tooth."""
        c = self.c
        rest = self.dets[self.first:, 1:]
        if len(rest) == 0:
            return
        ok = computed[rest].all(axis=1)
        k = len(ok) if ok.all() else int(np.argmin(ok))
        if k == 0:
            return
        d = rest[:k]
        contrib = detail[d] * c.w_inv[d] * c.step  # (k, teeth), tooth j at column j - 1
        my = np.cumsum(contrib[:, ::-1], axis=1)[:, ::-1]  # my[:, j - 1]: teeth j..teeth
        self.sumabove[1:] += my.sum(axis=0)
        self.sum2above[1:] += (my * my).sum(axis=0)
        self.nabove[1:] += k
        self.first += k

    def first_tooth(self, computed):
        c = self.c
        first_det = 1
        for i in range(c.first_det_of_comb, c.n + 1):
            if not computed[i]:
                first_det = i
                break
        tooth = 1
        for i in range(c.teeth, 0, -1):
            if c.first_det_of_teeth[i] < first_det:
                tooth = i
                break
        return tooth

    def estimate(self, detail, computed):
        """(average, error) as pt2_collector forms them."""
        c = self.c
        tooth = self.first_tooth(computed)
        f = c.first_det_of_teeth[tooth]
        e0 = float(np.sum(detail[1:f]))
        if tooth <= c.teeth:
            prop = ((1.0 - float(c.teeth - tooth + 1) * c.step) - c.cw[f - 1]) * c.w_inv[f]
            e0 += detail[f] * prop
            n = self.nabove[tooth]
            avg = e0 + self.sumabove[tooth] / n
            err = np.sqrt(1.0 / (n - 1) * abs(self.sum2above[tooth] / n - (self.sumabove[tooth] / n) ** 2)) if n > 1 \
                else np.inf
        else:
            avg, err = e0, 0.0
        return avg, err


def pt2_stochastic(compute, coef_gen, n_det=None, relative_error=1e-3, absolute_error=0.0, seed=0, batch=256,
                   teeth=COMB_TEETH):
    """ZMQ_pt2: the second-order energy of every state and its error.

    ``compute(gens)`` returns pt2_detail (len(gens), n_st) for 0-based
    generator indices (qpgpu_pt2_generators through Wavefunction.pt2_generators).
    ``coef_gen`` (n_gen, n_st) are the generators' coefficients
    (psi_coef_generators); ``n_det`` the size of the wave function (below
    max(10, n_st) the sum is exact).  Returns dict(pt2, error, n_computed,
    n_combs)."""
    cg = np.asarray(coef_gen, dtype=np.float64)
    if cg.ndim == 1:
        cg = cg[:, None]
    n_gen, n_st = cg.shape
    nst = n_st

    rng = np.random.default_rng(seed)
    detail = np.zeros((n_gen + 1, n_st))  # 1-based generator index
    computed = np.zeros(n_gen + 2, dtype=bool)

    def run(gens1):
        todo = [g for g in gens1 if not computed[g]]
        for a in range(0, len(todo), batch):
            part = todo[a:a + batch]
            d = np.asarray(compute([g - 1 for g in part]), dtype=np.float64).reshape(len(part), n_st)
            detail[part] = d
            computed[part] = True

    if (n_gen if n_det is None else n_det) < max(10, nst):
        run(list(range(1, n_gen + 1)))
        return dict(pt2=detail[1:].sum(axis=0)[:nst], error=np.zeros(nst), n_computed=n_gen, n_combs=0)
    pt2 = np.zeros(nst)
    err = np.zeros(nst)
    ncombs = 0
    for st in range(nst):
        comb = Comb(cg[:, st], teeth)
        _, comb_teeth, tbc = comb.workbatch(rng)
        est = Estimator(comb, comb_teeth)
        det_set = list(range(1, comb.first_det_of_comb))
        done = False
        for a in range(0, len(tbc), batch):
            run(tbc[a:a + batch])
            if not computed[det_set].all():
                continue
            est.do_carlo(detail[:, st], computed)
            if est.nabove[1] < 5:
                continue
            avg, e = est.estimate(detail[:, st], computed)
            if abs(e / avg) < relative_error or abs(e) < absolute_error:
                pt2[st], err[st] = avg, e
                done = True
                break
        if not done:
            est.do_carlo(detail[:, st], computed)
            pt2[st], err[st] = est.estimate(detail[:, st], computed)
        ncombs += est.first
    return dict(pt2=pt2, error=err, n_computed=int(computed.sum()), n_combs=ncombs)
