"""Load the committed golden fixtures (tests/golden/*.npz) as problems."""
import os

import numpy as np

from quantum_package_gb300 import generate as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    n = int(d["n_mo"])
    if "active" in d:
        small = G.Integrals(n_mo=len(d["active"]), h=d["h_active"], eri=d["eri_active"])
        ints = embed(n, d["active"], small)
    else:
        ints = G.Integrals(n_mo=n, h=d["h"], eri=d["eri"])
    d["ints"] = ints
    d["n_mo"], d["n_alpha"], d["n_beta"] = n, int(d["n_alpha"]), int(d["n_beta"])
    return d


def embed(n_full, active, small):
    h = np.zeros((n_full, n_full))
    np.fill_diagonal(h, 50.0)
    a0 = np.asarray(active) - 1
    h[np.ix_(a0, a0)] = small.h
    eri = np.zeros(G.packed_size(n_full))
    na = len(active)
    idx = np.arange(1, na + 1)
    p, q, r, s = (x.ravel() for x in np.meshgrid(idx, idx, idx, idx, indexing="ij"))
    sel = (p <= q) & (r <= s) & (G.pair_index(p, q) >= G.pair_index(r, s))
    p, q, r, s = p[sel], q[sel], r[sel], s[sel]
    active = np.asarray(active)
    eri[G.eri_key(active[p - 1], active[q - 1], active[r - 1], active[s - 1]) - 1] = \
        small.eri[G.eri_key(p, q, r, s) - 1]
    return G.Integrals(n_mo=n_full, h=h, eri=eri)
