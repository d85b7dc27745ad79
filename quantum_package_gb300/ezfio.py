"""Wave-function I/O of the EZFIO ``determinants`` group (host side).

The reference keeps the wave function in an EZFIO directory (the EZFIO
library, version 1.3.5, fetched by the reference's ``configure`` and not part
of its sources).  The routines restated here are the reference's own call
sites of that library:

* ``save_wavefunction_general`` (src/Determinants/determinants.irp.f:480-540)
  sets ``n_int``, ``bit_kind``, ``n_det``, ``n_states`` and ``mo_label``,
  stores the determinants as ``integer*8`` words, and stores the
  coefficients with every state normalised to 1.  A state of norm 0 is
  divided by sqrt(1e-12), so it stays 0;
* ``save_wavefunction`` (:456-465) saves the determinants sorted by their
  state-averaged contribution to the norm (``psi_det_sorted``, :258-292,
  with ``psi_average_norm_contrib``, :228-247, and the default state weights
  of density_matrix.irp.f:364-377);
* ``save_wavefunction_unsorted`` (:468-477) and ``save_ref_determinant``
  (:446-453) save in ``psi_det`` order, or the one reference determinant with
  coefficient 1 in state 1;
* ``read_dets`` (:399-444) reads ``psi_det`` back after checking
  ``n_int`` and ``bit_kind``.  The coefficients come back through
  ``psi_coef``.

Storage layout of an EZFIO attribute, as the library keeps it:
* a scalar is a text file ``<dir>/<group>/<name>`` holding the value;
* an array is ``<dir>/<group>/<name>.gz``, gzip-compressed text: the rank,
  then the dimensions, then one value per line in Fortran (column-major)
  order.

``psi_det`` has dimensions (n_int, 2, n_det): for determinant i, spin s and
word k the value sits at k + n_int (s + 2 i), which is exactly the
``dets[N][2][N_int]`` layout of this package flattened.  The words are
written as signed 64-bit integers, like the reference's
``transfer(psidet, 1_8)``.  ``psi_coef`` has dimensions (n_det, n_states).
The reader accepts any whitespace and Fortran ``D`` exponents.
"""
from __future__ import annotations

import gzip
import os

import numpy as np

GROUP = "determinants"
BIT_KIND = 8  # bytes per determinant word (integer*8)


# ---- attribute files -------------------------------------------------------

def _path(ezfio_dir, name):
    return os.path.join(ezfio_dir, GROUP, name)


def _fmt(v):
    if isinstance(v, (bool, np.bool_)):
        return "T" if v else "F"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):20d}"
    if isinstance(v, (float, np.floating)):
        return f"{float(v):25.16E}"
    return str(v)


def write_scalar(ezfio_dir, name, value):
    os.makedirs(os.path.join(ezfio_dir, GROUP), exist_ok=True)
    with open(_path(ezfio_dir, name), "w") as f:
        f.write(_fmt(value) + "\n")


def read_scalar(ezfio_dir, name, kind=int):
    with open(_path(ezfio_dir, name)) as f:
        s = f.read().strip()
    if kind is bool:
        return s.upper().lstrip(".").startswith("T")
    if kind is str:
        return s
    return kind(s.replace("D", "E").replace("d", "e")) if kind is float else int(s)


def write_array(ezfio_dir, name, arr, dims):
    """``arr`` flattened in Fortran order against ``dims`` (first index fastest)."""
    flat = np.asarray(arr).reshape(-1)
    assert flat.size == int(np.prod(dims)), (flat.size, dims)
    os.makedirs(os.path.join(ezfio_dir, GROUP), exist_ok=True)
    if flat.dtype.kind in "iu":
        body = "\n".join(f"{int(v):20d}" for v in flat.astype(np.int64))
    else:
        body = "\n".join(f"{float(v):25.16E}" for v in flat.astype(np.float64))  # 17 digits: exact round trip
    text = f"{len(dims):11d}\n" + "".join(f"{int(d):11d}" for d in dims) + "\n" + body + "\n"
    with gzip.open(_path(ezfio_dir, name + ".gz"), "wt") as f:
        f.write(text)


def read_array(ezfio_dir, name, dtype):
    """Returns (flat values in Fortran order, dims)."""
    with gzip.open(_path(ezfio_dir, name + ".gz"), "rt") as f:
        tok = f.read().replace("D", "E").replace("d", "e").split()
    rank = int(tok[0])
    dims = [int(t) for t in tok[1:1 + rank]]
    vals = tok[1 + rank:]
    n = int(np.prod(dims))
    if len(vals) != n:
        raise ValueError(f"{name}: {len(vals)} values for dimensions {dims}")
    if np.dtype(dtype).kind in "iu":
        out = np.array([int(v) for v in vals], dtype=np.int64)
    else:
        out = np.array([float(v) for v in vals], dtype=np.float64)
    return out, dims


def has(ezfio_dir, name):
    return os.path.exists(_path(ezfio_dir, name)) or os.path.exists(_path(ezfio_dir, name + ".gz"))


# ---- the reference's sort (dsort: insertion below 32 entries, else quicksort)

def dsort(x):
    """Ascending sort of ``x`` with the reference's ``dsort``
    (src/Utils/sort.irp.f:241-265): insertion sort below 32 entries, else a
    quicksort with the middle element as pivot (:41-78).  Equal keys keep
    the order that algorithm leaves them in.  Returns (sorted x, iorder)
    with ``iorder`` 0-based."""
    x = np.array(x, dtype=np.float64)
    n = len(x)
    order = np.arange(n)
    if n < 2:
        return x, order
    if n < 32:
        for i in range(1, n):
            xt, it = x[i], order[i]
            j = i - 1
            while j >= 0 and not (x[j] <= xt):
                x[j + 1] = x[j]
                order[j + 1] = order[j]
                j -= 1
            x[j + 1] = xt
            order[j + 1] = it
        return x, order
    stack = [(0, n - 1)]  # inclusive bounds, 0-based
    while stack:
        first, last = stack.pop()
        c = x[(first + last + 2) // 2 - 1]  # x(ishft(first+last,-1)) in 1-based indices
        i, j = first, last
        while True:
            while x[i] < c:
                i += 1
            while c < x[j]:
                j -= 1
            if i >= j:
                break
            x[i], x[j] = x[j], x[i]
            order[i], order[j] = order[j], order[i]
            i += 1
            j -= 1
        # the reference recurses into (first, i-1) first, then (j+1, last);
        # the sub-ranges are disjoint, so the visiting order does not change the result
        if j + 1 < last:
            stack.append((j + 1, last))
        if first < i - 1:
            stack.append((first, i - 1))
    return x, order


def average_norm_contrib(coefs, weights=None):
    """psi_average_norm_contrib (determinants.irp.f:228-247).  The default
    weights are 1 per state, + 1e-31, normalised (density_matrix.irp.f:364-377)."""
    c = np.asarray(coefs, dtype=np.float64)
    nst = c.shape[1]
    w = np.ones(nst) if weights is None else np.asarray(weights, dtype=np.float64)
    w = w + 1e-31
    w = w / w.sum()
    contrib = np.zeros(c.shape[0])
    for k in range(nst):
        contrib = contrib + c[:, k] * c[:, k] * w[k]
    return contrib * (1.0 / float(np.cumsum(contrib)[-1]))


def sorted_order(coefs, weights=None):
    """psi_det_sorted order: determinants by decreasing state-averaged norm
    contribution (determinants.irp.f:258-292)."""
    _, order = dsort(-average_norm_contrib(coefs, weights))
    return order


# ---- save / read -------------------------------------------------------------

def save_wavefunction_general(ezfio_dir, dets, coefs, n_states=None, mo_label=""):
    """save_wavefunction_general(ndet, nstates, psidet, dim, psicoef):
    ``dets`` [n_det][2][n_int] uint64, ``coefs`` [n_det][>= n_states]."""
    dets = np.ascontiguousarray(dets, dtype=np.uint64)
    n_det, two, n_int = dets.shape
    assert two == 2
    c = np.asarray(coefs, dtype=np.float64).reshape(n_det, -1)
    nst = c.shape[1] if n_states is None else int(n_states)
    c = c[:, :nst]
    write_scalar(ezfio_dir, "n_int", n_int)
    write_scalar(ezfio_dir, "bit_kind", BIT_KIND)
    write_scalar(ezfio_dir, "n_det", n_det)
    write_scalar(ezfio_dir, "n_states", nst)
    write_scalar(ezfio_dir, "mo_label", mo_label)
    write_array(ezfio_dir, "psi_det", dets.view(np.int64), [n_int, 2, n_det])
    save = np.empty_like(c)
    for k in range(nst):
        col = c[:, k]
        acc = float(np.cumsum(col * col)[-1]) if n_det else 0.0  # the reference's sequential sum
        if acc == 0.0:
            acc = 1.0e-12
        save[:, k] = col * (1.0 / np.sqrt(acc))
    write_array(ezfio_dir, "psi_coef", save.T, [n_det, nst])  # Fortran order: determinant index fastest


def save_wavefunction(ezfio_dir, dets, coefs, n_states=None, mo_label="", weights=None):
    """save_wavefunction: the determinants in psi_det_sorted order."""
    c = np.asarray(coefs, dtype=np.float64).reshape(len(dets), -1)
    nst = c.shape[1] if n_states is None else int(n_states)
    order = sorted_order(c[:, :nst], weights)
    save_wavefunction_general(ezfio_dir, np.asarray(dets)[order], c[order], min(nst, len(dets)), mo_label)
    return order


def save_wavefunction_unsorted(ezfio_dir, dets, coefs, n_states=None, mo_label=""):
    c = np.asarray(coefs, dtype=np.float64).reshape(len(dets), -1)
    nst = c.shape[1] if n_states is None else int(n_states)
    save_wavefunction_general(ezfio_dir, dets, c, min(nst, len(dets)), mo_label)


def save_ref_determinant(ezfio_dir, ref_det, n_states, mo_label=""):
    """save_ref_determinant: one determinant, coefficient 1 in state 1."""
    buf = np.zeros((1, n_states))
    buf[0, 0] = 1.0
    save_wavefunction_general(ezfio_dir, np.asarray(ref_det, dtype=np.uint64).reshape(1, 2, -1), buf, n_states,
                              mo_label)


def read_dets(ezfio_dir, n_int=None):
    """read_dets: [n_det][2][n_int] uint64.  ``n_int`` and ``bit_kind`` must
    match (the reference ASSERTs both)."""
    ni = read_scalar(ezfio_dir, "n_int")
    if n_int is not None and ni != n_int:
        raise ValueError(f"determinants/n_int is {ni}, expected {n_int}")
    bk = read_scalar(ezfio_dir, "bit_kind")
    if bk != BIT_KIND:
        raise ValueError(f"determinants/bit_kind is {bk}, expected {BIT_KIND}")
    flat, dims = read_array(ezfio_dir, "psi_det", np.int64)
    if dims[0] != ni * bk // 8 or dims[1] != 2:
        raise ValueError(f"psi_det dimensions {dims} do not match n_int = {ni}")
    return np.ascontiguousarray(flat.view(np.uint64).reshape(dims[2], 2, dims[0]))


def read_psi_coef(ezfio_dir):
    """psi_coef as [n_det][n_states]."""
    flat, dims = read_array(ezfio_dir, "psi_coef", np.float64)
    return np.ascontiguousarray(flat.reshape(dims[1], dims[0]).T)


def read_wavefunction(ezfio_dir, n_int=None):
    """(dets [n_det][2][n_int], coefs [n_det][n_states]) of an EZFIO directory."""
    dets = read_dets(ezfio_dir, n_int)
    coefs = read_psi_coef(ezfio_dir)
    if coefs.shape[0] != dets.shape[0] or read_scalar(ezfio_dir, "n_det") != dets.shape[0]:
        raise ValueError("psi_det, psi_coef and n_det disagree")
    return dets, coefs
