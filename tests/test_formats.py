"""Round trips of the integral exchange formats written by generate.py.

The files are read back the way the reference reads them, restated here:
read_integral (plugins/read_integral/read_integrals_mo.irp.f:58-105) fills
A(i,j) from `kinetic_mo` and `nuclear_mo` (mo_mono_elec_integral is their
sum) and keys each `bielec_mo` line `i j k l value` with
bielec_integrals_index(i,j,k,l) (src/Integrals_Bielec/map_integrals.irp.f:19-34),
i.e. physicist <ij|kl> = chemist (ik|jl); an FCIDUMP line `value p q r s`
(plugins/FCIdump/fcidump.irp.f:9-49) is chemist (pq|rs), `value i j 0 0` the
one-electron h_ij and `value 0 0 0 0` the core energy.  The arrays read back
must equal those the generator produced, bit for bit (17 significant digits
round-trip a double), with every 8-fold class present once.
"""
import numpy as np

from quantum_package_gb300 import generate as G


def _read_read_integral(directory, n):
    A = np.zeros((n, n))
    for name in ("kinetic_mo", "nuclear_mo"):
        B = np.zeros((n, n))
        with open(f"{directory}/{name}") as f:
            for ln in f:
                i, j, v = ln.split()
                B[int(i) - 1, int(j) - 1] = float(v)
        A += B
    eri = np.full(G.packed_size(n), np.nan)
    seen = np.zeros(G.packed_size(n), np.int64)
    with open(f"{directory}/bielec_mo") as f:
        for ln in f:
            i, j, k, l, v = ln.split()
            key = int(G.eri_key(int(i), int(k), int(j), int(l)))  # <ij|kl> = (ik|jl)
            eri[key - 1] = float(v)
            seen[key - 1] += 1
    return A, eri, seen


def _read_fcidump(path):
    with open(path) as f:
        lines = f.readlines()
    head = "".join(lines[:4])
    norb = int(head.split("NORB=")[1].split(",")[0])
    nelec = int(head.split("NELEC=")[1].split(",")[0])
    ms2 = int(head.split("MS2=")[1].split(",")[0])
    h = np.full((norb, norb), np.nan)
    eri = np.full(G.packed_size(norb), np.nan)
    seen = np.zeros(G.packed_size(norb), np.int64)
    core = None
    body = [ln for ln in lines if ln.strip() and not ln.lstrip().startswith(("&", "ORBSYM", "ISYM", "/"))]
    for ln in body:
        v, p, q, r, s = ln.split()
        p, q, r, s = int(p), int(q), int(r), int(s)
        if p == q == r == s == 0:
            core = float(v)
        elif r == 0 and s == 0:
            h[p - 1, q - 1] = h[q - 1, p - 1] = float(v)
        else:
            key = int(G.eri_key(p, q, r, s))
            eri[key - 1] = float(v)
            seen[key - 1] += 1
    return norb, nelec, ms2, h, eri, seen, core


def test_read_integral_round_trip(tmp_path):
    ints = G.make_integrals(9, 11)
    G.write_read_integral(str(tmp_path), ints)
    A, eri, seen = _read_read_integral(str(tmp_path), 9)
    np.testing.assert_array_equal(A, ints.h)
    assert np.all(seen == 1)
    np.testing.assert_array_equal(eri, ints.eri)


def test_fcidump_round_trip(tmp_path):
    ints = G.make_integrals(8, 12)
    path = str(tmp_path / "FCIDUMP")
    G.write_fcidump(path, ints, 3, 2)
    norb, nelec, ms2, h, eri, seen, core = _read_fcidump(path)
    assert (norb, nelec, ms2, core) == (8, 5, 1, 0.0)
    np.testing.assert_array_equal(h, ints.h)
    assert np.all(seen == 1)
    np.testing.assert_array_equal(eri, ints.eri)


def test_read_back_integrals_give_the_same_oracle_sigma(tmp_path):
    # the same determinant set on the integrals read back: identical sigma
    from oracle import Oracle
    p = G.make_problem(1, n_det=500, n_mo=12, n_alpha=4, n_beta=4)
    G.write_read_integral(str(tmp_path), p.ints)
    A, eri, _ = _read_read_integral(str(tmp_path), p.n_mo)
    u = G.random_coefficients(p.n_det, 2, 3)
    v0, s0 = Oracle(p.n_mo, 4, 4, p.ints.h, p.ints.eri, p.dets).h_s2_u0(u)
    v1, s1 = Oracle(p.n_mo, 4, 4, A, eri, p.dets).h_s2_u0(u)
    np.testing.assert_array_equal(v0, v1)
    np.testing.assert_array_equal(s0, s1)
