"""Second-quantisation matrix elements (test infrastructure only).

An evaluator that shares no code and no formula with the Slater-Condon rules of
``src/Determinants/slater_rules.irp.f``: it applies the fermionic operators of

    H   = sum_{pq,s} h_pq a+_{ps} a_{qs}
        + 1/2 sum_{pqrs,st} (pq|rs) a+_{ps} a+_{rt} a_{st} a_{qs}
    S+S- = sum_{pq} a+_{p,alpha} a_{p,beta} a+_{q,beta} a_{q,alpha}

to occupation lists and counts signs by the number of occupied spin-orbitals
that each operator passes.  Spin-orbital order is alpha 1..n then beta 1..n,
i.e. a determinant is prod_{alpha, ascending} a+ prod_{beta, ascending} a+ |0>,
which is the convention under which the reference's phases are derived.
``S+S-`` is the operator whose matrix QP's ``get_s2`` / ``diag_S_mat_elem``
(``src/Determinants/s2.irp.f:1-63``) return; QP adds ``S_z(S_z-1)`` on top.

Pure-Python loops: meant for small spaces and sampled pairs only.
"""
from __future__ import annotations

import numpy as np


def modes(det: np.ndarray, n_mo: int) -> list[int]:
    """det (2, n_int) uint64 -> ascending spin-orbital indices (alpha first)."""
    out = []
    for s in range(2):
        for w, word in enumerate(det[s]):
            x = int(word)
            while x:
                b = (x & -x).bit_length() - 1
                x &= x - 1
                out.append(s * n_mo + 64 * w + b)
    return out


def _annihilate(occ: list[int], k: int):
    if k not in occ:
        return None, 0
    i = occ.index(k)
    return occ[:i] + occ[i + 1:], (-1) ** i


def _create(occ: list[int], k: int):
    if k in occ:
        return None, 0
    i = 0
    while i < len(occ) and occ[i] < k:
        i += 1
    return occ[:i] + [k] + occ[i:], (-1) ** i


def _apply(occ, ops):
    """ops: list of ('c'|'a', mode), applied right-to-left as written."""
    sign = 1
    for kind, k in reversed(ops):
        if kind == "a":
            occ, s = _annihilate(occ, k)
        else:
            occ, s = _create(occ, k)
        if occ is None:
            return None, 0
        sign *= s
    return occ, sign


class SecondQuantized:
    def __init__(self, n_mo: int, h: np.ndarray, eri_chem):
        """eri_chem(p, q, r, s) -> chemist (pq|rs), 1-based spatial orbitals."""
        self.n = n_mo
        self.h = h
        self.eri = eri_chem

    def h_elem(self, det_i: np.ndarray, det_j: np.ndarray) -> float:
        n = self.n
        oi, oj = modes(det_i, n), modes(det_j, n)
        si, sj = set(oi), set(oj)
        removed = sj - si
        if len(removed) > 2:
            return 0.0
        total = 0.0
        # one-body
        for q in oj:
            rest = sj - {q}
            if not rest <= si:
                continue
            cand = list(si - rest)
            if len(cand) != 1:
                continue
            p = cand[0]
            if p // n != q // n:
                continue
            occ, sg = _apply(oj, [("c", p), ("a", q)])
            if occ is not None and occ == oi:
                total += sg * self.h[p % n, q % n]
        # two-body
        for q in oj:
            for s_ in oj:
                if s_ == q:
                    continue
                rest = sj - {q, s_}
                if not rest <= si:
                    continue
                add = list(si - rest)
                if len(add) != 2:
                    continue
                for p, r in ((add[0], add[1]), (add[1], add[0])):
                    if p // n != q // n or r // n != s_ // n:
                        continue
                    occ, sg = _apply(oj, [("c", p), ("c", r), ("a", s_), ("a", q)])
                    if occ is not None and occ == oi:
                        total += 0.5 * sg * self.eri(p % n + 1, q % n + 1, r % n + 1, s_ % n + 1)
        return total

    def s2_elem(self, det_i: np.ndarray, det_j: np.ndarray) -> float:
        """<I| S+ S- |J>."""
        n = self.n
        oi, oj = modes(det_i, n), modes(det_j, n)
        if len(set(oj) ^ set(oi)) > 4:
            return 0.0
        total = 0.0
        for q in range(n):
            occ1, s1 = _apply(oj, [("c", n + q), ("a", q)])
            if occ1 is None:
                continue
            for p in range(n):
                occ2, s2 = _apply(occ1, [("c", p), ("a", n + p)])
                if occ2 is not None and occ2 == oi:
                    total += s1 * s2
        return float(total)
