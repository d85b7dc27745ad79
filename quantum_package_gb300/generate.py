"""Seeded synthetic inputs for the Davidson sigma path.

Quantum Package reads MO integrals through ``plugins/read_integral``
(``read_integrals_mo.irp.f:1-116``) and determinants from EZFIO ``psi_det``
(``src/Determinants/EZFIO.cfg:81-85``).  No molecule, basis or SCF is involved
here: every input is drawn from a numpy PCG64 stream so that the CPU oracle,
the CUDA path and (on a machine with gfortran/irpf90) the reference itself can
be fed identical data.

Conventions (the same as the reference):

* orbitals are 1-based in every exported list; orbital ``p`` is bit ``(p-1) % 64``
  of word ``(p-1) // 64`` (``src/Bitmask/bitmasks_module.f90:1-11``);
* determinants are ``psi_det(N_int, 2, N)`` in Fortran order, i.e. a C array
  ``dets[N][2][N_int]`` of uint64 (spin 0 = alpha, spin 1 = beta);
* two-electron integrals are chemist ``(pq|rs)`` stored 8-fold packed at
  ``key - 1`` where ``key`` is ``bielec_integrals_index``
  (``src/Integrals_Bielec/map_integrals.irp.f:19-34``):
  ``key = P(P(p,q), P(r,s))`` with ``P(i,j) = max*(max-1)/2 + min``;
* the aufbau reference (orbitals 1..N_alpha / 1..N_beta) equals QP's
  ``HF_bitmask`` (``src/Bitmask/bitmasks.irp.f:71-87``) because the orbital
  energies are sorted ascending.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np

BASE_SEED = 20261203
N_CHOLESKY = 120


def n_int_for(n_mo: int) -> int:
    return (n_mo - 1) // 64 + 1


def pair_index(i, j):
    """1-based symmetric pair index ``P(i,j)`` of ``bielec_integrals_index``."""
    i = np.asarray(i, dtype=np.int64)
    j = np.asarray(j, dtype=np.int64)
    lo = np.minimum(i, j)
    hi = np.maximum(i, j)
    return lo + (hi * hi - hi) // 2


def eri_key(p, q, r, s):
    """1-based 8-fold key of chemist ``(pq|rs)``; physicist ``<ij|kl>`` is ``(ik|jl)``."""
    return pair_index(pair_index(p, q), pair_index(r, s))


def packed_size(n_mo: int) -> int:
    p2 = n_mo * (n_mo + 1) // 2
    return p2 * (p2 + 1) // 2


@dataclass
class Integrals:
    n_mo: int
    h: np.ndarray            # (n, n) float64, symmetric one-electron h_pq
    eri: np.ndarray          # (packed_size,) float64, chemist (pq|rs) at key-1

    def chem(self, p, q, r, s):
        return self.eri[eri_key(p, q, r, s) - 1]


def make_integrals(n_mo: int, seed: int, n_chol: int = N_CHOLESKY) -> Integrals:
    """h_pp = eps_p ~ U[-2,2] sorted, h_pq ~ N(0,0.02); (pq|rs) = sum_k L^k_pq L^k_rs, L ~ N(0,0.05)."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 0]))
    eps = np.sort(rng.uniform(-2.0, 2.0, n_mo))
    h = np.zeros((n_mo, n_mo))
    iu = np.triu_indices(n_mo, 1)
    h[iu] = rng.normal(0.0, 0.02, len(iu[0]))
    h = h + h.T
    h[np.diag_indices(n_mo)] = eps
    p2 = n_mo * (n_mo + 1) // 2
    # L[k, P(p,q)-1] for p <= q: pair P(p,q) = p + q(q-1)/2 (1-based)
    L = rng.normal(0.0, 0.05, (n_chol, p2))
    full = L.T @ L                      # (P2, P2) symmetric, PSD
    rows, cols = np.tril_indices(p2)    # rows >= cols ; key = cols+1 + rows(rows+1)/2
    keys = (cols + 1) + (rows * (rows + 1)) // 2
    eri = np.empty(p2 * (p2 + 1) // 2)
    eri[keys - 1] = full[rows, cols]
    return Integrals(n_mo=n_mo, h=h, eri=eri)


def _bits_from_positions(pos: np.ndarray, n_int: int) -> np.ndarray:
    """pos: (M, k) int array of 0-based orbitals (or -1 for none) -> (M, n_int) uint64 OR of bits."""
    m = pos.shape[0]
    out = np.zeros((m, n_int), dtype=np.uint64)
    valid = pos >= 0
    word = np.where(valid, pos // 64, 0)
    bit = np.where(valid, pos % 64, 0).astype(np.uint64)
    val = np.where(valid, np.left_shift(np.uint64(1), bit), np.uint64(0))
    for w in range(n_int):
        out[:, w] = np.bitwise_or.reduce(np.where(word == w, val, np.uint64(0)), axis=1)
    return out


def reference_det(n_mo: int, n_alpha: int, n_beta: int) -> np.ndarray:
    n_int = n_int_for(n_mo)
    det = np.zeros((2, n_int), dtype=np.uint64)
    for s, ne in enumerate((n_alpha, n_beta)):
        pos = np.arange(ne)[None, :]
        det[s] = _bits_from_positions(pos, n_int)[0]
    return det


def _random_excitations(rng, m, n_mo, n_el, rank, n_int):
    """rank: (m,) number of electrons moved; returns (m, n_int) XOR masks."""
    n_vir = n_mo - n_el
    kmax = int(rank.max()) if m else 0
    if kmax == 0:
        return np.zeros((m, n_int), dtype=np.uint64)
    occ_perm = np.argsort(rng.random((m, n_el)), axis=1)[:, :kmax]
    vir_perm = np.argsort(rng.random((m, n_vir)), axis=1)[:, :kmax] + n_el
    use = np.arange(kmax)[None, :] < rank[:, None]
    holes = np.where(use, occ_perm, -1)
    parts = np.where(use, vir_perm, -1)
    return _bits_from_positions(holes, n_int) ^ _bits_from_positions(parts, n_int)


def make_dets(n_mo: int, n_alpha: int, n_beta: int, n_det: int, seed: int,
              max_rank: int = 4, chunk: int = 1 << 18) -> np.ndarray:
    """Aufbau reference + random rank-r (r uniform in 1..max_rank) excitations.

    The alpha/beta split r_alpha is uniform in 0..r; holes are drawn uniformly
    from the occupied orbitals of that spin and particles from the virtuals.
    Candidates are deduplicated (first occurrence kept, reference first) until
    ``n_det`` unique determinants exist.  Returns ``dets[N][2][N_int]`` uint64.
    """
    n_int = n_int_for(n_mo)
    rng = np.random.default_rng(np.random.SeedSequence([seed, 1]))
    ref = reference_det(n_mo, n_alpha, n_beta)
    max_a = min(n_alpha, n_mo - n_alpha)
    max_b = min(n_beta, n_mo - n_beta)
    found = [ref.reshape(1, 2 * n_int)]
    seen = {ref.tobytes()}
    total = 1
    while total < n_det:
        m = chunk
        r = rng.integers(1, max_rank + 1, m)
        ra = rng.integers(0, r + 1)
        ra = np.minimum(ra, max_a)
        rb = np.minimum(r - ra, max_b)
        xa = _random_excitations(rng, m, n_mo, n_alpha, ra, n_int)
        xb = _random_excitations(rng, m, n_mo, n_beta, rb, n_int)
        cand = np.concatenate([xa ^ ref[0][None, :], xb ^ ref[1][None, :]], axis=1)
        # dedup inside the chunk, keep first occurrences in draw order
        v = np.ascontiguousarray(cand).view(np.dtype((np.void, cand.dtype.itemsize * cand.shape[1]))).ravel()
        _, first = np.unique(v, return_index=True)
        first.sort()
        keep = []
        for idx in first:
            b = v[idx].tobytes()
            if b not in seen:
                seen.add(b)
                keep.append(idx)
                if total + len(keep) >= n_det:
                    break
        if keep:
            found.append(cand[np.asarray(keep)])
            total += len(keep)
    dets = np.concatenate(found, axis=0)[:n_det]
    return np.ascontiguousarray(dets.reshape(n_det, 2, n_int))


def random_coefficients(n_det: int, n_states: int, seed: int) -> np.ndarray:
    """C ~ N(0,1), columns normalised; returned as u0[N_st][N] (column-major u_0(sze,N_st))."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 2]))
    u = rng.normal(0.0, 1.0, (n_states, n_det))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return u


@dataclass
class Problem:
    name: str
    n_mo: int
    n_alpha: int
    n_beta: int
    n_det: int
    n_states: int
    seed: int
    ints: Integrals
    dets: np.ndarray

    @property
    def n_int(self) -> int:
        return n_int_for(self.n_mo)


# Configurations quoted by the sigma/Davidson workload (sizes only; the
# generator above defines the distributions).
CONFIGS = {
    1: dict(name="c1_n40_10a10b_1e4_1st", n_mo=40, n_alpha=10, n_beta=10, n_det=10_000, n_states=1),
    2: dict(name="c2_n80_14a14b_1e6_4st", n_mo=80, n_alpha=14, n_beta=14, n_det=1_000_000, n_states=4),
    4: dict(name="c4_n80_14a14b_cipsi_4st", n_mo=80, n_alpha=14, n_beta=14, n_det=1_000_000, n_states=4),
    5: dict(name="c5_n120_16a16b_2e7_2st", n_mo=120, n_alpha=16, n_beta=16, n_det=20_000_000, n_states=2),
}


def make_problem(cfg: int, n_det: int | None = None, n_mo: int | None = None,
                 n_alpha: int | None = None, n_beta: int | None = None,
                 n_states: int | None = None, seed: int | None = None) -> Problem:
    c = dict(CONFIGS[cfg])
    if n_det is not None:
        c["n_det"] = n_det
    if n_mo is not None:
        c["n_mo"] = n_mo
    if n_alpha is not None:
        c["n_alpha"] = n_alpha
    if n_beta is not None:
        c["n_beta"] = n_beta
    if n_states is not None:
        c["n_states"] = n_states
    s = BASE_SEED + cfg if seed is None else seed
    ints = make_integrals(c["n_mo"], s)
    dets = make_dets(c["n_mo"], c["n_alpha"], c["n_beta"], c["n_det"], s)
    return Problem(c["name"], c["n_mo"], c["n_alpha"], c["n_beta"], c["n_det"],
                   c["n_states"], s, ints, dets)


def batched_problems(n_problems: int = 64, seed: int = BASE_SEED + 3,
                     n_det_min: float = 1e3, n_det_max: float = 1e5):
    """Independent CI problems of uneven size: n ~ U{30..60}, N_a = N_b ~ U{8..16},
    N_det log-uniform, 1..3 states; problem j uses seed + 1000*j."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n_problems):
        n_mo = int(rng.integers(30, 61))
        ne = int(rng.integers(8, 17))
        nd = int(round(math.exp(rng.uniform(math.log(n_det_min), math.log(n_det_max)))))
        nst = int(rng.integers(1, 4))
        s = seed + 1000 * (j + 1)
        ints = make_integrals(n_mo, s)
        dets = make_dets(n_mo, ne, ne, nd, s)
        out.append(Problem(f"c3_p{j}", n_mo, ne, ne, nd, nst, s, ints, dets))
    return out


# ---------------------------------------------------------------------------
# Exchange formats (so that the reference can be run on the same data)
# ---------------------------------------------------------------------------

def write_read_integral(directory: str, ints: Integrals) -> None:
    """Files read by ``plugins/read_integral/read_integrals_mo.irp.f:58-105``.

    ``kinetic_mo`` / ``nuclear_mo`` hold ``i j value`` for every (i,j) (both
    triangles, 1-based); h_pq goes to ``kinetic_mo`` and ``nuclear_mo`` is zero.
    ``bielec_mo`` holds physicist ``<ij|kl>`` as ``i j k l value``: chemist
    ``(pq|rs)`` is written as ``p r q s`` once per 8-fold class.
    """
    os.makedirs(directory, exist_ok=True)
    n = ints.n_mo
    with open(os.path.join(directory, "kinetic_mo"), "w") as f:
        for i in range(n):
            for j in range(n):
                f.write(f"{i + 1} {j + 1} {ints.h[i, j]:.17e}\n")
    with open(os.path.join(directory, "nuclear_mo"), "w") as f:
        for i in range(n):
            for j in range(n):
                f.write(f"{i + 1} {j + 1} {0.0:.17e}\n")
    with open(os.path.join(directory, "bielec_mo"), "w") as f:
        for s in range(1, n + 1):
            for r in range(1, s + 1):
                for q in range(1, n + 1):
                    for p in range(1, q + 1):
                        if pair_index(p, q) < pair_index(r, s):
                            continue
                        v = ints.chem(p, q, r, s)
                        f.write(f"{p} {r} {q} {s} {v:.17e}\n")


def write_fcidump(path: str, ints: Integrals, n_alpha: int, n_beta: int) -> None:
    """FCIDUMP in the layout of ``plugins/FCIdump/fcidump.irp.f:9-49`` (chemist order)."""
    n = ints.n_mo
    with open(path, "w") as f:
        f.write(f" &FCI NORB={n}, NELEC={n_alpha + n_beta}, MS2={n_alpha - n_beta},\n")
        f.write(" ORBSYM=" + "1," * n + "\n ISYM=0,\n /\n")
        for s in range(1, n + 1):
            for r in range(1, s + 1):
                for q in range(1, n + 1):
                    for p in range(1, q + 1):
                        if pair_index(p, q) < pair_index(r, s):
                            continue
                        f.write(f" {ints.chem(p, q, r, s):.17e} {p} {q} {r} {s}\n")
        for j in range(1, n + 1):
            for i in range(j, n + 1):
                f.write(f" {ints.h[i - 1, j - 1]:.17e} {i} {j} 0 0\n")
        f.write(f" {0.0:.17e} 0 0 0 0\n")


def full_ci_dets(n_mo: int, n_alpha: int, n_beta: int) -> np.ndarray:
    """Every (alpha, beta) string pair of the space, aufbau reference first."""
    from itertools import combinations
    n_int = n_int_for(n_mo)

    def strings(ne):
        out = []
        for occ in combinations(range(n_mo), ne):
            w = [0] * n_int
            for p in occ:
                w[p // 64] |= 1 << (p % 64)
            out.append(w)
        return np.array(out, dtype=np.uint64).reshape(-1, n_int)

    sa, sb = strings(n_alpha), strings(n_beta)
    ia, ib = np.meshgrid(np.arange(len(sa)), np.arange(len(sb)), indexing="ij")
    dets = np.stack([sa[ia.ravel()], sb[ib.ravel()]], axis=1)
    return np.ascontiguousarray(dets)
