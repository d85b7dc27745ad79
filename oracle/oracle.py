"""ctypes front-end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libqporacle.so`` (built from ``qp_oracle.cpp`` by
``oracle/Makefile``).  Only the tests, the smoke check and the CPU-baseline
leg of the bench use it, as the checker; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libqporacle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "qp_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.qpo_create.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.POINTER(C.c_void_p)]
        L.qpo_destroy.argtypes = [C.c_void_p]
        L.qpo_set_dets.argtypes = [C.c_void_p, _u64p, C.c_int64]
        L.qpo_ref_energy.argtypes = [C.c_void_p]
        L.qpo_ref_energy.restype = C.c_double
        L.qpo_n_unique.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.qpo_tables.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        L.qpo_bilinear.argtypes = [C.c_void_p] + [_i32p] * 8
        L.qpo_unique_strings.argtypes = [C.c_void_p, _u64p, _u64p]
        L.qpo_h_s2_u0_work.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.qpo_h_s2_u0.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int64]
        L.qpo_connected_pairs.argtypes = [C.c_void_p, _i32p, _i32p, _i8p, C.c_int64]
        L.qpo_connected_pairs.restype = C.c_int64
        L.qpo_h_s2_u0_rows.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int64, _i32p, C.c_int64]
        L.qpo_connected_pairs_rows.argtypes = [C.c_void_p, _i32p, C.c_int64, _i32p, _i32p, _i8p, C.c_int64]
        L.qpo_connected_pairs_rows.restype = C.c_int64
        L.qpo_pair_excitation.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, _i32p,
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.qpo_pair_excitations.argtypes = [C.c_void_p, C.c_int64, _i32p, _i32p, _i8p, _i8p, _i32p, _dp, _dp]
        L.qpo_diag.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.qpo_i_h_j.argtypes = [C.c_void_p, _u64p, _u64p]
        L.qpo_i_h_j.restype = C.c_double
        L.qpo_get_s2.argtypes = [C.c_void_p, _u64p, _u64p]
        L.qpo_get_s2.restype = C.c_double
        L.qpo_dense.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.qpo_davidson.argtypes = [C.c_void_p, _dp, C.c_int64, _dp, _dp, C.c_int, C.c_int, C.c_int,
                                   C.c_double, C.c_int, C.c_int, _dp, C.c_int]
        L.qpo_num_threads.restype = C.c_int
        L.qpo_select_pt2.argtypes = [C.c_void_p, _dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp, _u64p, _dp,
                                     C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    """FP64 restatement of the reference's sigma / Slater rules / Davidson."""

    def __init__(self, n_mo, n_alpha, n_beta, h, eri, dets=None):
        L = lib()
        self.n_mo, self.n_alpha, self.n_beta = n_mo, n_alpha, n_beta
        self.n_int = (n_mo - 1) // 64 + 1
        hf = np.ascontiguousarray(np.asarray(h, dtype=np.float64).T)  # col-major
        self._h = C.c_void_p()
        rc = L.qpo_create(n_mo, n_alpha, n_beta, hf.ravel(), np.ascontiguousarray(eri, dtype=np.float64),
                          C.byref(self._h))
        if rc != 0:
            raise ValueError(f"qpo_create failed ({rc})")
        self.n_det = 0
        if dets is not None:
            self.set_dets(dets)

    @classmethod
    def from_problem(cls, prob):
        return cls(prob.n_mo, prob.n_alpha, prob.n_beta, prob.ints.h, prob.ints.eri, prob.dets)

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.qpo_destroy(self._h)
            self._h = None

    def set_dets(self, dets):
        dets = np.ascontiguousarray(dets, dtype=np.uint64)
        self.dets = dets
        self.n_det = dets.shape[0]
        rc = lib().qpo_set_dets(self._h, dets.ravel(), self.n_det)
        if rc != 0:
            raise ValueError(f"qpo_set_dets failed ({rc})")

    @property
    def ref_energy(self):
        return lib().qpo_ref_energy(self._h)

    def n_unique(self):
        a, b = C.c_int(), C.c_int()
        lib().qpo_n_unique(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def tables(self):
        n = self.n_mo
        f, jj, kk = (np.empty((n, n)) for _ in range(3))
        bc, bx = np.empty((n, n, n)), np.empty((n, n, n))
        lib().qpo_tables(self._h, _ptr(f), _ptr(jj), _ptr(kk), _ptr(bc), _ptr(bx))
        # col-major -> index [i-1, j-1] with transpose
        return dict(fock=f.T.copy(), jj=jj.T.copy(), kk=kk.T.copy(),
                    big_coul=bc.transpose(2, 1, 0).copy(), big_exch=bx.transpose(2, 1, 0).copy())

    def bilinear(self):
        N = self.n_det
        ua, ub = self.n_unique()
        arrs = [np.empty(N, np.int32) for _ in range(6)]
        cl = np.empty(ub + 1, np.int32)
        rl = np.empty(ua + 1, np.int32)
        lib().qpo_bilinear(self._h, *arrs, cl, rl)
        keys = ["rows", "cols", "order", "t_rows", "t_cols", "t_order"]
        d = dict(zip(keys, arrs))
        d["col_loc"], d["row_loc"] = cl, rl
        a = np.empty((ua, self.n_int), np.uint64)
        b = np.empty((ub, self.n_int), np.uint64)
        lib().qpo_unique_strings(self._h, a.ravel(), b.ravel())
        d["alpha_unique"], d["beta_unique"] = a, b
        return d

    def h_s2_u0(self, u0):
        """u0: (N_st, N) -> (v0, s0) each (N_st, N)  [H_S2_u_0_nstates_openmp]."""
        u0 = np.ascontiguousarray(np.atleast_2d(u0), dtype=np.float64)
        nst, n = u0.shape
        v = np.zeros_like(u0)
        s = np.zeros_like(u0)
        rc = lib().qpo_h_s2_u0(self._h, v.ravel(), s.ravel(), u0.ravel(), nst, n)
        if rc != 0:
            raise ValueError(f"qpo_h_s2_u0 failed ({rc})")
        return v, s

    def h_s2_u0_work(self, u_t, istart, iend, ishift=0, istep=1):
        """Range variant in bilinear order; u_t: (N, N_st) states fastest."""
        u_t = np.ascontiguousarray(u_t, dtype=np.float64)
        nst = u_t.shape[1]
        v = np.zeros_like(u_t)
        s = np.zeros_like(u_t)
        rc = lib().qpo_h_s2_u0_work(self._h, v.ravel(), s.ravel(), u_t.ravel(), nst, istart, iend, ishift, istep)
        if rc != 0:
            raise ValueError(f"qpo_h_s2_u0_work failed ({rc})")
        return v, s

    def h_s2_u0_rows(self, u0, rows):
        """Sigma of the determinants `rows` (0-based psi_det) only: u0 (N_st, N) ->
        (v, s) each (N_st, len(rows)), the worker loops restricted to those rows."""
        u0 = np.ascontiguousarray(np.atleast_2d(u0), dtype=np.float64)
        nst, n = u0.shape
        r = np.ascontiguousarray(rows, dtype=np.int32)
        v = np.zeros((len(r), nst))
        s = np.zeros((len(r), nst))
        rc = lib().qpo_h_s2_u0_rows(self._h, v.ravel(), s.ravel(), u0.ravel(), nst, n, r, len(r))
        if rc != 0:
            raise ValueError(f"qpo_h_s2_u0_rows failed ({rc})")
        return v.T.copy(), s.T.copy()

    def connected_pairs_rows(self, rows):
        """(I, J, cls) of the pairs of the determinants `rows` (0-based psi_det), sorted by (I, J)."""
        L = lib()
        r = np.ascontiguousarray(np.unique(np.asarray(rows)), dtype=np.int32)
        e32 = np.empty(1, np.int32)
        n = L.qpo_connected_pairs_rows(self._h, r, len(r), e32, e32, np.empty(1, np.int8), 0)
        if n < 0:
            raise ValueError("qpo_connected_pairs_rows: bad rows")
        I = np.empty(n, np.int32)
        J = np.empty(n, np.int32)
        cls = np.empty(n, np.int8)
        L.qpo_connected_pairs_rows(self._h, r, len(r), I, J, cls, n)
        o = np.lexsort((J, I))
        return I[o], J[o], cls[o]

    def connected_pairs(self):
        """(I, J, cls) arrays (0-based original order), sorted by (I, J)."""
        L = lib()
        empty32 = np.empty(1, np.int32)
        n = L.qpo_connected_pairs(self._h, empty32, empty32, np.empty(1, np.int8), 0)
        I = np.empty(n, np.int32)
        J = np.empty(n, np.int32)
        cls = np.empty(n, np.int8)
        L.qpo_connected_pairs(self._h, I, J, cls, n)
        o = np.lexsort((J, I))
        return I[o], J[o], cls[o]

    def pair_excitation(self, i, j, cls):
        exc = np.zeros(4, np.int32)
        hij, sij = C.c_double(), C.c_double()
        ph = lib().qpo_pair_excitation(self._h, int(i), int(j), int(cls), exc, C.byref(hij), C.byref(sij))
        return ph, exc, hij.value, sij.value

    def pair_excitations(self, I, J, cls):
        """Batched pair_excitation: (phase int8, exc (n,4) int32, hij, sij)."""
        n = len(I)
        ph = np.empty(n, np.int8)
        exc = np.empty((n, 4), np.int32)
        hij = np.empty(n)
        sij = np.empty(n)
        rc = lib().qpo_pair_excitations(self._h, n, np.ascontiguousarray(I, np.int32), np.ascontiguousarray(J, np.int32),
                                        np.ascontiguousarray(cls, np.int8), ph, exc.ravel(), hij, sij)
        if rc != 0:
            raise RuntimeError("qpo_pair_excitations failed")
        return ph, exc, hij, sij

    def diag(self):
        h = np.empty(self.n_det)
        s = np.empty(self.n_det)
        lib().qpo_diag(self._h, _ptr(h), _ptr(s))
        return h, s

    def i_h_j(self, di, dj):
        return lib().qpo_i_h_j(self._h, np.ascontiguousarray(di, np.uint64).ravel(),
                               np.ascontiguousarray(dj, np.uint64).ravel())

    def get_s2(self, di, dj):
        return lib().qpo_get_s2(self._h, np.ascontiguousarray(di, np.uint64).ravel(),
                                np.ascontiguousarray(dj, np.uint64).ravel())

    def dense(self, with_s2=True):
        N = self.n_det
        H = np.empty((N, N))
        S = np.empty((N, N)) if with_s2 else None
        lib().qpo_dense(self._h, _ptr(H), _ptr(S))
        return H, S

    def davidson(self, guess, n_states, davidson_sze_max=8, threshold=1e-12, s2_eig=True, max_sigma=500,
                 state_following=False):
        """guess: (N_st_diag, N).  Returns (energies, s2, vectors, n_sigma, residuals)."""
        u = np.ascontiguousarray(guess, dtype=np.float64).copy()
        nsd, n = u.shape
        e = np.zeros(nsd)
        s2 = np.zeros(nsd)
        res = np.zeros(max(n_states, 1))
        rc = lib().qpo_davidson(self._h, u.ravel(), n, e, s2, n_states, nsd, davidson_sze_max,
                                threshold, int(bool(s2_eig)), max_sigma, res, int(bool(state_following)))
        if rc < 0:
            raise RuntimeError(f"qpo_davidson failed ({rc})")
        return e, s2, u, rc, res

    def select_pt2(self, coef, e0, n_gen, n_sel, buf_size):
        """CIPSI selection with the second-order energy (selection.irp.f restated).

        The context's determinants must be in psi_det_sorted order (sort_by_weight);
        coef: (n_st, N) in that order, e0: (n_st,) denominators, generators and
        selectors the first n_gen / n_sel determinants.  Returns (pt2 (n_st,),
        buffer determinants (n, 2, N_int), buffer values (n,) ascending, number of
        external determinants with a non-zero numerator)."""
        coef = np.atleast_2d(np.asarray(coef, dtype=np.float64))
        n_st = coef.shape[0]
        cm = np.ascontiguousarray(coef)  # (n_st, N) row-major == (N, n_st) column-major
        e0 = np.ascontiguousarray(np.atleast_1d(e0), dtype=np.float64)
        pt2 = np.zeros(n_st)
        nint = (self.n_mo + 63) // 64
        dets = np.zeros((max(buf_size, 1), 2, nint), np.uint64)
        vals = np.zeros(max(buf_size, 1))
        n_ext = C.c_int64(0)
        n = lib().qpo_select_pt2(self._h, cm.ravel(), n_st, e0, int(n_gen), int(n_sel), int(buf_size), pt2,
                                 dets.ravel(), vals, C.byref(n_ext))
        if n < 0:
            raise ValueError("qpo_select_pt2: bad arguments")
        return pt2, dets[:n].copy(), vals[:n].copy(), n_ext.value


def sort_by_weight(coef, weights=None):
    """psi_det_sorted (determinants.irp.f:228-293): the order of determinants
    by decreasing state-averaged norm contribution sum_k w_k c_ik^2
    (normalised to 1), coef (n_states, N).  Returns (order, sorted
    contributions)."""
    coef = np.atleast_2d(coef)
    w = np.ones(coef.shape[0]) if weights is None else np.asarray(weights, dtype=np.float64)
    contrib = (coef * coef * (w + 1e-31)[:, None]).sum(axis=0)
    contrib = contrib / contrib.sum()
    order = np.argsort(-contrib, kind="stable")
    return order, contrib[order]


def n_generators(contrib_sorted, threshold=0.99):
    """N_det_generators of Generators_full (generators.irp.f:3-22): the first
    determinants whose cumulative contribution reaches threshold."""
    c = np.cumsum(contrib_sorted)
    hit = np.nonzero(c >= threshold)[0]
    return max(int(hit[0]) + 1 if len(hit) else len(c), 1)


def n_selectors(contrib_sorted, n_gen, threshold=0.999, threshold_generators=0.99):
    """N_det_selectors of Selectors_full (selectors.irp.f:3-25)."""
    n = len(contrib_sorted)
    if threshold_generators < 1.0:
        c = np.cumsum(contrib_sorted)
        hit = np.nonzero(c > threshold)[0]
        n = int(hit[0]) + 1 if len(hit) else n
        n = max(n, n_gen)
    return n


def num_threads() -> int:
    return lib().qpo_num_threads()


def build_flags() -> str:
    """CXXFLAGS of the oracle build (oracle/Makefile)."""
    try:
        with open(os.path.join(_HERE, "Makefile")) as f:
            for ln in f:
                if ln.startswith("CXXFLAGS"):
                    return ln.split("=", 1)[1].strip()
    except OSError:
        pass
    return "unknown"
