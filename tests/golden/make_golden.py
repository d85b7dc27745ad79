"""Generate the golden fixtures in this folder (run once; the .npz files are committed).

    python tests/golden/make_golden.py

Every expected value comes from ``oracle/secondq.py``: fermionic operator
algebra applied to occupation lists, sharing no code or formula with the
Slater-Condon rules of ``src/Determinants/slater_rules.irp.f``.  The fixtures
are small enough for pure-Python loops.

Sets
----
fci_s2   n=6, 3a/2b, full CI (300 dets): dense H and S+S-, lowest eigenvalues
fci_cs   n=6, 3a/3b, full CI (400 dets): same, closed shell
sci_n1   n=12, 4a/4b, 500 seeded dets (N_int=1): sigma and S^2-sigma of 2 vectors
sci_n2   n=70, 9a/8b, 400 dets whose electrons live on orbitals 1..9 and
         56..70 (N_int=2, excitations cross the 64-bit word boundary):
         sigma and S^2-sigma of 2 vectors
pairs_n2 n=70, 9a/8b: 400 sampled connected pairs (random occupations over
         both words) with <I|H|J>, <I|S+S-|J>

Integrals of the n=70 sets are drawn for 24 "active" orbitals and embedded in
the 70-orbital space (other entries zero; their h_pp large so they stay
virtual); the fixtures store only the active block.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from quantum_package_gb300 import generate as G  # noqa: E402
from secondq import SecondQuantized  # noqa: E402

SEED = 777


def embed(n_full: int, active: np.ndarray, small: G.Integrals) -> G.Integrals:
    """Place the integrals of len(active) orbitals on orbitals `active` (1-based) of n_full."""
    h = np.zeros((n_full, n_full))
    np.fill_diagonal(h, 50.0)
    a0 = active - 1
    h[np.ix_(a0, a0)] = small.h
    eri = np.zeros(G.packed_size(n_full))
    na = len(active)
    idx = np.arange(1, na + 1)
    p, q, r, s = np.meshgrid(idx, idx, idx, idx, indexing="ij")
    p, q, r, s = (x.ravel() for x in (p, q, r, s))
    sel = (p <= q) & (r <= s) & (G.pair_index(p, q) >= G.pair_index(r, s))
    p, q, r, s = p[sel], q[sel], r[sel], s[sel]
    vals = small.eri[G.eri_key(p, q, r, s) - 1]
    eri[G.eri_key(active[p - 1], active[q - 1], active[r - 1], active[s - 1]) - 1] = vals
    return G.Integrals(n_mo=n_full, h=h, eri=eri)


def n70_integrals():
    active = np.array(list(range(1, 10)) + list(range(56, 71)), dtype=np.int64)
    small = G.make_integrals(len(active), SEED + 70)
    return active, small, embed(70, active, small)


def sq_for(ints: G.Integrals) -> SecondQuantized:
    return SecondQuantized(ints.n_mo, ints.h, lambda p, q, r, s: float(ints.chem(p, q, r, s)))


def dense(sq, dets):
    n = len(dets)
    H = np.zeros((n, n))
    S = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            H[i, j] = H[j, i] = sq.h_elem(dets[i], dets[j])
            S[i, j] = S[j, i] = sq.s2_elem(dets[i], dets[j])
    return H, S


def random_occupation_dets(rng, n_mo, na, nb, orbitals, count):
    """Determinants whose electrons are drawn among `orbitals` (1-based), aufbau ref first."""
    n_int = G.n_int_for(n_mo)
    out = [G.reference_det(n_mo, na, nb)]
    seen = {out[0].tobytes()}
    while len(out) < count:
        d = np.zeros((2, n_int), dtype=np.uint64)
        for s, ne in enumerate((na, nb)):
            occ = rng.choice(orbitals, ne, replace=False) - 1
            for p in occ:
                d[s, p // 64] |= np.uint64(1) << np.uint64(p % 64)
        if d.tobytes() not in seen:
            seen.add(d.tobytes())
            out.append(d)
    return np.ascontiguousarray(np.stack(out))


def excite(rng, det, n_mo, spin, k):
    """Move k electrons of `spin` to random empty orbitals (anywhere in 1..n_mo)."""
    d = det.copy()
    occ = [p for p in range(n_mo) if (int(d[spin, p // 64]) >> (p % 64)) & 1]
    emp = [p for p in range(n_mo) if not (int(d[spin, p // 64]) >> (p % 64)) & 1]
    for p in rng.choice(occ, k, replace=False):
        d[spin, p // 64] ^= np.uint64(1) << np.uint64(p % 64)
    for p in rng.choice(emp, k, replace=False):
        d[spin, p // 64] ^= np.uint64(1) << np.uint64(p % 64)
    return d


def main():
    rng = np.random.default_rng(SEED)
    out = {}

    for name, (n, na, nb) in {"fci_s2": (6, 3, 2), "fci_cs": (6, 3, 3)}.items():
        ints = G.make_integrals(n, SEED + n + na + nb)
        dets = G.full_ci_dets(n, na, nb)
        H, S = dense(sq_for(ints), dets)
        sz = 0.5 * (na - nb)
        w, v = np.linalg.eigh(H)
        s2 = np.einsum("ik,ij,jk->k", v, S, v) + sz * (sz - 1.0)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n_mo=n, n_alpha=na, n_beta=nb,
                            h=ints.h, eri=ints.eri, dets=dets, H=H, S=S, eigvals=w, s2=s2)
        out[name] = len(dets)

    # sci_n1: N_int = 1 selected space
    n, na, nb = 12, 4, 4
    ints = G.make_integrals(n, SEED + 12)
    dets = G.make_dets(n, na, nb, 500, SEED + 12)
    H, S = dense(sq_for(ints), dets)
    u = rng.normal(size=(2, len(dets)))
    np.savez_compressed(os.path.join(HERE, "sci_n1.npz"), n_mo=n, n_alpha=na, n_beta=nb,
                        h=ints.h, eri=ints.eri, dets=dets, u=u, sigma=u @ H, s2sigma=u @ S,
                        hdiag=np.diag(H).copy())
    out["sci_n1"] = len(dets)

    # sci_n2: N_int = 2, word-boundary crossing
    active, small, ints70 = n70_integrals()
    na, nb = 9, 8
    dets = random_occupation_dets(rng, 70, na, nb, active, 400)
    H, S = dense(sq_for(ints70), dets)
    u = rng.normal(size=(2, len(dets)))
    np.savez_compressed(os.path.join(HERE, "sci_n2.npz"), n_mo=70, n_alpha=na, n_beta=nb,
                        active=active, h_active=small.h, eri_active=small.eri, dets=dets, u=u,
                        sigma=u @ H, s2sigma=u @ S, hdiag=np.diag(H).copy(),
                        n_pairs=int(np.count_nonzero(H - np.diag(np.diag(H)))))
    out["sci_n2"] = len(dets)

    # pairs_n2: sampled connected pairs with electrons anywhere in 1..70
    allorb = np.arange(1, 71)
    base = random_occupation_dets(rng, 70, na, nb, allorb, 120)[1:]
    sq70 = SecondQuantized(70, ints70.h, lambda p, q, r, s: float(ints70.chem(p, q, r, s)))
    I, J, hij, sij, kind = [], [], [], [], []
    for t in range(400):
        di = base[t % len(base)]
        k = t % 5  # 0: a-single 1: b-single 2: aa 3: bb 4: ab
        if k == 0:
            dj = excite(rng, di, 70, 0, 1)
        elif k == 1:
            dj = excite(rng, di, 70, 1, 1)
        elif k == 2:
            dj = excite(rng, di, 70, 0, 2)
        elif k == 3:
            dj = excite(rng, di, 70, 1, 2)
        else:
            dj = excite(rng, excite(rng, di, 70, 0, 1), 70, 1, 1)
        I.append(di)
        J.append(dj)
        hij.append(sq70.h_elem(di, dj))
        sij.append(sq70.s2_elem(di, dj))
        kind.append(k + 1)
    np.savez_compressed(os.path.join(HERE, "pairs_n2.npz"), n_mo=70, n_alpha=na, n_beta=nb,
                        active=active, h_active=small.h, eri_active=small.eri,
                        I=np.stack(I), J=np.stack(J), hij=np.array(hij), sij=np.array(sij),
                        kind=np.array(kind, np.int8))
    out["pairs_n2"] = len(I)
    print(out)


if __name__ == "__main__":
    main()
