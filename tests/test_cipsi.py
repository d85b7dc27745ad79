"""The CIPSI loop of the Full_CI program (plugins/Full_CI_ZMQ/fci_zmq.irp.f)
over the device library (quantum_package_gb300/cipsi.py).

CPU: make_s2_eigenfunction (src/Determinants/occ_pattern.irp.f:251-300)
completes every occupation pattern of the wave function, i.e. every alpha /
beta assignment of its singly occupied orbitals.

GPU: on a full-CI space (3 + 3 electrons in 8 MOs, 3136 determinants,
seeded integrals), CIPSI from the aufbau determinant must behave like the
reference's loop:
* the variational energy falls at every iteration and stays above the
  full-CI energy (dense diagonalisation of the oracle's H);
* the selection's second-order energy is negative and shrinks;
* E + PT2 is closer to the full-CI energy than E in the later iterations;
* with N_det_max = the full space, the loop ends at the full-CI energy
  (1e-9 Ha).
"""
import numpy as np
import pytest

from quantum_package_gb300 import cipsi
from quantum_package_gb300 import generate as G


def _patterns(dets):
    return {tuple(int(x) for x in np.concatenate([d[0] & d[1], d[0] ^ d[1]])) for d in dets}


def test_make_s2_eigenfunction_completes_patterns():
    full = G.full_ci_dets(7, 3, 3)
    rng = np.random.default_rng(4)
    pick = full[np.sort(rng.choice(len(full), 25, replace=False))]
    out, added = cipsi.make_s2_eigenfunction(pick, 3)
    assert added == len(out) - len(pick) and np.array_equal(out[:25], pick)
    keys = {d.tobytes() for d in out}
    assert len(keys) == len(out)  # no duplicates
    # every determinant of the full space with one of the patterns is there, and nothing else
    pats = _patterns(pick)
    want = {d.tobytes() for d in full if next(iter(_patterns([d]))) in pats}
    assert keys == want
    # a closed set is left alone
    again, n2 = cipsi.make_s2_eigenfunction(out, 3)
    assert n2 == 0 and np.array_equal(again, out)


@pytest.mark.gpu
def test_cipsi_converges_to_full_ci():
    from oracle import Oracle
    from quantum_package_gb300.sigma import Wavefunction
    n_mo, na, nb = 8, 3, 3
    ints = G.make_integrals(n_mo, 17)
    full = G.full_ci_dets(n_mo, na, nb)
    H, _ = Oracle(n_mo, na, nb, ints.h, ints.eri, full).dense(with_s2=False)
    e_fci = np.linalg.eigvalsh(H)[0]
    start = full[np.argsort(np.diag(H), kind="stable")[:1]]
    make = lambda d: Wavefunction(n_mo, na, nb, ints.h, ints.eri, d)
    r = cipsi.run(make, start, 1, 400, pt2_max=1e-10, n_states_diag=4, threshold_davidson=1e-12,
                  threshold_generators=1.0, threshold_selectors=1.0)
    hist = r["history"]
    e = [h["energies"][0] for h in hist] + [r["energies"][0]]
    assert len(hist) >= 4
    assert np.all(np.diff(e) <= 1e-10), e
    assert e[-1] >= e_fci - 1e-9
    pt2 = [h["pt2"][0] for h in hist]
    assert all(p < 0 for p in pt2)
    assert abs(pt2[-1]) < abs(pt2[0])
    late = hist[len(hist) // 2:]
    assert all(abs(h["energies"][0] + h["pt2"][0] - e_fci) < abs(h["energies"][0] - e_fci) for h in late)
    # grown to the whole space: the full-CI energy
    r2 = cipsi.run(make, start, 1, len(full), pt2_max=0.0, n_states_diag=4, threshold_davidson=1e-12,
                   threshold_generators=1.0, threshold_selectors=1.0)
    assert abs(r2["energies"][0] - e_fci) < 1e-9, (r2["energies"][0], e_fci, len(r2["dets"]))
