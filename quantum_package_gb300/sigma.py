"""Host-side mirror of Quantum Package's sigma interface over libqpgpu.

The reference keeps the determinant set and integrals in IRPF90 providers and
exposes ``H_S2_u_0_nstates_openmp(v_0, s_0, u_0, N_st, sze)``
(src/Davidson/u0Hu0.irp.f:15-66) and its range variant
``H_S2_u_0_nstates_openmp_work(v_t, s_t, u_t, N_st, sze, istart, iend, ishift,
istep)`` (:69-96).  ``Wavefunction`` plays the role of those providers: it
holds a device context (integral tables, bilinear index, connected pairs) and
offers the same entry points with the same argument meaning.

Array conventions: a Fortran array ``u_0(sze, N_st)`` is a C-contiguous numpy
array of shape ``(N_st, sze)``; ``u_t(N_st, N_det)`` is shape ``(N_det, N_st)``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FP32, FP64, check


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def stream_handle(stream):
    """C-ABI stream argument: NULL selects the context's stream, so torch's
    legacy default stream (handle 0) is passed as cudaStreamLegacy (0x1)."""
    if stream is None:
        return None
    h = stream.cuda_stream
    return C.c_void_p(h if h else 1)


class Wavefunction:
    """Providers of one orbital space and determinant set, on the GPU."""

    def __init__(self, n_mo: int, n_alpha: int, n_beta: int, h=None, eri=None, psi_det=None, sigma_mode=0,
                 line_keys=None):
        L = _lib.load()
        self.n_mo, self.n_alpha, self.n_beta = n_mo, n_alpha, n_beta
        self.n_int = (n_mo - 1) // 64 + 1
        h_ = C.c_void_p()
        rc = L.qpgpu_create(n_mo, n_alpha, n_beta, self.n_int, C.byref(h_))
        if rc != 0:
            raise _lib.QPGPUError(rc, "qpgpu_create failed (device or arguments)")
        self._ctx = h_
        self.n_det = 0
        if sigma_mode:
            self.set_sigma_mode(sigma_mode)
        if line_keys is not None:
            self.set_line_keys(*line_keys)
        if h is not None:
            self.set_integrals(h, eri)
        if psi_det is not None:
            self.set_dets(psi_det)

    @classmethod
    def from_problem(cls, prob, sigma_mode=0, line_keys=None):
        return cls(prob.n_mo, prob.n_alpha, prob.n_beta, prob.ints.h, prob.ints.eri, prob.dets, sigma_mode,
                   line_keys)

    def set_sigma_mode(self, mode):
        """SIGMA_AUTO (0), SIGMA_STORED (1) or SIGMA_DIRECT (2); takes effect at the next set_dets."""
        check(_lib.load().qpgpu_set_sigma_mode(self._ctx, int(mode)), self._ctx)

    def set_line_keys(self, min_single=-1, min_double=-1, hash_bits=64):
        """Deletion-key tables for the lines holding more than min_single /
        min_double determinants (-1: defaults, KEYS_OFF: none); hash_bits < 64
        only to test colliding keys.  Takes effect at the next set_dets."""
        check(_lib.load().qpgpu_set_line_keys(self._ctx, int(min_single), int(min_double), int(hash_bits)),
              self._ctx)

    def close(self):
        if getattr(self, "_ctx", None):
            _lib.load().qpgpu_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def set_integrals(self, h, eri):
        hf = np.ascontiguousarray(np.asarray(h, dtype=np.float64).T)  # column-major h(i,j)
        e = np.ascontiguousarray(eri, dtype=np.float64)
        check(_lib.load().qpgpu_set_integrals(self._ctx, _p(hf), _p(e)), self._ctx)

    def set_dets(self, psi_det):
        d = np.ascontiguousarray(psi_det, dtype=np.uint64)
        if d.ndim != 3 or d.shape[1] != 2 or d.shape[2] != self.n_int:
            raise ValueError("psi_det must have shape (N_det, 2, N_int)")
        check(_lib.load().qpgpu_set_dets(self._ctx, _p(d), d.shape[0]), self._ctx)
        self.n_det = d.shape[0]

    def info(self) -> dict:
        i = _lib.Info()
        check(_lib.load().qpgpu_get_info(self._ctx, C.byref(i)), self._ctx)
        return {f: getattr(i, f) for f, _ in i._fields_}

    def u_0_H_u_0(self, u_0):
        """e_0[i] = <u_0[i]|H|u_0[i]> (not divided by the norm, as the reference); u_0: (N_st, sze)."""
        u = np.ascontiguousarray(np.atleast_2d(u_0), dtype=np.float64)
        n_st, ld = u.shape
        e = np.zeros(n_st)
        check(_lib.load().qpgpu_u0_h_u0(self._ctx, _p(e), _p(u), n_st, ld), self._ctx)
        return e

    # --- sigma ---------------------------------------------------------
    def H_S2_u_0_nstates_openmp(self, u_0):
        """v_0 = H u_0, s_0 = S^2 u_0 (no S_z(S_z-1) shift); u_0: (N_st, sze) -> (v_0, s_0)."""
        u = np.ascontiguousarray(np.atleast_2d(u_0), dtype=np.float64)
        n_st, ld = u.shape
        v = np.zeros_like(u)
        s = np.zeros_like(u)
        check(_lib.load().qpgpu_h_s2_u0(self._ctx, _p(v), _p(s), _p(u), n_st, ld), self._ctx)
        return v, s

    def H_S2_u_0_nstates_openmp_work(self, u_t, istart, iend, ishift=0, istep=1, v_t=None, s_t=None):
        """Range variant in bilinear order; u_t: (N_det, N_st).  Rows outside the range are untouched."""
        u = np.ascontiguousarray(u_t, dtype=np.float64)
        v = np.zeros_like(u) if v_t is None else v_t
        s = np.zeros_like(u) if s_t is None else s_t
        check(_lib.load().qpgpu_h_s2_u0_work(self._ctx, _p(v), _p(s), _p(u), u.shape[1], istart, iend, ishift,
                                             istep), self._ctx)
        return v, s

    def h_s2_u0_device(self, v0, s0, u0, precision=FP64, stream=None):
        """torch CUDA tensors (N_st, ld) float64; asynchronous on `stream` (torch stream or None)."""
        n_st, ld = u0.shape
        st = stream_handle(stream)
        check(_lib.load().qpgpu_h_s2_u0_device(self._ctx, C.c_void_p(v0.data_ptr()), C.c_void_p(s0.data_ptr()),
                                               C.c_void_p(u0.data_ptr()), n_st, ld, precision, st), self._ctx)

    def sigma_bilinear(self, v_t, s_t, u_t, u_t32=None, precision=FP64, stream=None):
        """Internal layout: torch CUDA tensors (N_det, N_st), bilinear order."""
        st = stream_handle(stream)
        p32 = C.c_void_p(u_t32.data_ptr()) if u_t32 is not None else None
        check(_lib.load().qpgpu_sigma_bilinear(self._ctx, C.c_void_p(v_t.data_ptr()), C.c_void_p(s_t.data_ptr()),
                                               C.c_void_p(u_t.data_ptr()), p32, u_t.shape[1], precision, st),
              self._ctx)

    def bilinear_order(self):
        o = np.empty(self.n_det, np.int32)
        check(_lib.load().qpgpu_bilinear_order(self._ctx, _p(o)), self._ctx)
        return o

    def diag(self):
        """(H_jj, <I|S+S-|I>) in psi_det order."""
        h = np.empty(self.n_det)
        s = np.empty(self.n_det)
        check(_lib.load().qpgpu_diag(self._ctx, _p(h), _p(s)), self._ctx)
        return h, s

    def connected_pairs(self):
        """Pairs sorted by (I, J): I, J (0-based psi_det), class, phase, exc (P,4), hij."""
        L = _lib.load()
        n = C.c_int64()
        check(L.qpgpu_connected_pairs(self._ctx, C.byref(n), None, None, None, None, None, None, 0), self._ctx)
        P = n.value
        I = np.empty(P, np.int32)
        J = np.empty(P, np.int32)
        cls = np.empty(P, np.int8)
        ph = np.empty(P, np.int8)
        exc = np.empty((P, 4), np.int16)
        hij = np.empty(P)
        check(L.qpgpu_connected_pairs(self._ctx, C.byref(n), _p(I), _p(J), _p(cls), _p(ph), _p(exc), _p(hij), P),
              self._ctx)
        o = np.lexsort((J, I))
        return dict(I=I[o], J=J[o], cls=cls[o], phase=ph[o], exc=exc[o], hij=hij[o])

    # --- CIPSI selection ------------------------------------------------
    def select_pt2(self, coef, e0, n_gen, n_sel, buf_size):
        """Selection with the second-order energy (qpgpu_select_pt2) over this
        set, which must be in psi_det_sorted order.  coef: (n_st, N) (the
        sorted coefficients), e0: (n_st,) electronic denominators.  Returns
        (pt2 (n_st,), buffer determinants (k, 2, N_int), buffer values (k,),
        number of external determinants with a non-zero numerator)."""
        cm = np.ascontiguousarray(np.atleast_2d(coef), dtype=np.float64)
        n_st = cm.shape[0]
        e0 = np.ascontiguousarray(np.atleast_1d(e0), dtype=np.float64)
        if e0.shape != (n_st,) or cm.shape[1] != self.n_det:
            raise ValueError("select_pt2: coef must be (n_st, N_det) and e0 (n_st,)")
        nint = self.n_int
        pt2 = np.zeros(n_st)
        bd = np.zeros((max(buf_size, 1), 2, nint), np.uint64)
        bv = np.zeros(max(buf_size, 1))
        n_ext = C.c_int64()
        rc = _lib.load().qpgpu_select_pt2(self._ctx, _p(cm), n_st, _p(e0), int(n_gen), int(n_sel), int(buf_size),
                                          _p(pt2), _p(bd), _p(bv), C.byref(n_ext))
        if rc < 0:
            check(rc, self._ctx)
        return pt2, bd[:rc].copy(), bv[:rc].copy(), n_ext.value

    def pt2_generators(self, coef, e0, n_sel, gens):
        """pt2_detail (len(gens), n_st) of the listed generators
        (qpgpu_pt2_generators); coef (n_st, N) sorted, gens 0-based."""
        cm = np.ascontiguousarray(np.atleast_2d(coef), dtype=np.float64)
        n_st = cm.shape[0]
        e0 = np.ascontiguousarray(np.atleast_1d(e0), dtype=np.float64)
        g = np.ascontiguousarray(np.asarray(gens), dtype=np.int32)
        out = np.zeros((max(len(g), 1), n_st))
        check(_lib.load().qpgpu_pt2_generators(self._ctx, _p(cm), n_st, _p(e0), int(n_sel), _p(g), len(g), _p(out)),
              self._ctx)
        return out[:len(g)]

    # --- dressing (MRCC / MRCEPA0) ---------------------------------------
    def set_dressing(self, idx_ref, idx_non_ref, delta_ij, delta_ij_s2, delta_ii=None):
        """Dressing of one state (delta_ij(istate,:,:) of the reference's providers):
        idx_ref (n_ref,), idx_non_ref (n_non_ref,) psi_det indices (0-based);
        delta_ij, delta_ij_s2 arrays (n_ref, n_non_ref) [the Fortran (n_non_ref, n_ref)];
        delta_ii (n_ref,) or None."""
        r = np.ascontiguousarray(idx_ref, np.int32)
        nr = np.ascontiguousarray(idx_non_ref, np.int32)
        d = np.ascontiguousarray(delta_ij, np.float64)
        ds = np.ascontiguousarray(delta_ij_s2, np.float64)
        assert d.shape == (len(r), len(nr)) and ds.shape == d.shape
        dii = None if delta_ii is None else np.ascontiguousarray(delta_ii, np.float64)
        check(_lib.load().qpgpu_set_dressing(self._ctx, len(r), _p(r), len(nr), _p(nr), _p(d), _p(ds), _p(dii)),
              self._ctx)

    def clear_dressing(self):
        check(_lib.load().qpgpu_clear_dressing(self._ctx), self._ctx)

    def H_S2_u_0_mrcc_nstates(self, u_0):
        """H_S2_u_0_mrcc_nstates (plugins/MRCC_Utils/davidson.irp.f:955): sigma of H plus the dressing."""
        u = np.ascontiguousarray(np.atleast_2d(u_0), dtype=np.float64)
        v = np.empty_like(u)
        s = np.empty_like(u)
        check(_lib.load().qpgpu_h_s2_u0_dressed(self._ctx, _p(v), _p(s), _p(u), u.shape[0], u.shape[1]), self._ctx)
        return v, s

    def connected_pairs_rows(self, rows):
        """Pairs of the determinants `rows` (0-based psi_det indices) only, sorted by (I, J)."""
        L = _lib.load()
        r = np.ascontiguousarray(np.unique(np.asarray(rows)), dtype=np.int32)
        n = C.c_int64()
        check(L.qpgpu_connected_pairs_rows(self._ctx, _p(r), len(r), C.byref(n), None, None, None, None, None, None,
                                           0), self._ctx)
        P = n.value
        I = np.empty(P, np.int32)
        J = np.empty(P, np.int32)
        cls = np.empty(P, np.int8)
        ph = np.empty(P, np.int8)
        exc = np.empty((P, 4), np.int16)
        hij = np.empty(P)
        check(L.qpgpu_connected_pairs_rows(self._ctx, _p(r), len(r), C.byref(n), _p(I), _p(J), _p(cls), _p(ph),
                                           _p(exc), _p(hij), P), self._ctx)
        o = np.lexsort((J, I))
        return dict(I=I[o], J=J[o], cls=cls[o], phase=ph[o], exc=exc[o], hij=hij[o])

    # --- Davidson ------------------------------------------------------
    def davidson_diag_hs2(self, u_in, n_states, davidson_sze_max=8, threshold=1e-12, s2_eig=True,
                          precision=FP64, defect_every=0, preconditioner=0, max_iter=500, collect_every=0,
                          collect_max=8, trace_cap=1024, algebra=0, state_following=False, dressed=False):
        """davidson_diag_hs2 (diagonalization_hs2.irp.f:1-49) on this determinant set.

        u_in: (N_st_diag, N) guess vectors (all of them, seeded by the caller).
        precision=FP64 is the reference's loop in FP64; FP32 runs the FP32
        sigma with an FP64 sigma at each restart (defect correction), FF the
        same with a float-float restart sigma; both mixed modes run the
        projections and Gram-Schmidt in float-float, accept convergence only
        on restart iterations and report FP64-accurate energies.
        preconditioner=1 uses the learned step (see mlp_*) in place of the
        diagonal one; preconditioner=2 adds it as an extra direction (in the
        correction slot of Ritz vector n_states + k); collect_every > 0
        captures training pairs for it.  algebra=ALGEBRA_FP64 keeps the
        mixed modes' projections, Gram-Schmidt, Ritz vectors and step in FP64
        (only sigma in FP32); state_following keeps the Ritz vectors that
        overlap most with the guesses (the reference's EZFIO flag); dressed
        runs davidson_diag_mrcc_hs2 with the context's dressing.  Returns dict(energies, s2, vectors,
        n_sigma, converged, n_fallback, n_samples, trace) with electronic energies.
        """
        u = np.ascontiguousarray(np.atleast_2d(u_in), dtype=np.float64).copy()
        nsd, n = u.shape
        prm = _lib.DavidsonParams(n_states=n_states, n_states_diag=nsd, davidson_sze_max=davidson_sze_max,
                                  s2_eig=int(bool(s2_eig)), threshold=threshold, precision=precision,
                                  defect_every=defect_every, preconditioner=preconditioner, max_iter=max_iter,
                                  collect_every=collect_every, collect_max=collect_max,
                                  state_following=int(bool(state_following)), algebra=algebra,
                                  dressed=int(bool(dressed)))
        prec = np.zeros(trace_cap, np.int32)
        en = np.zeros((trace_cap, n_states))
        rs = np.zeros((trace_cap, n_states))
        el = np.zeros(trace_cap)
        tr = _lib.DavidsonTrace(cap=trace_cap, n=0, n_sigma=0, converged=0, sigma_precision=prec.ctypes.data,
                                energies=en.ctypes.data, residuals=rs.ctypes.data, elapsed_ms=el.ctypes.data)
        e = np.zeros(nsd)
        s2 = np.zeros(nsd)
        rc = _lib.load().qpgpu_davidson_hs2(self._ctx, _p(u), n, _p(e), _p(s2), C.byref(prm), C.byref(tr))
        if rc < 0:
            check(rc, self._ctx)
        k = tr.n
        return dict(energies=e, s2=s2, vectors=u, n_sigma=rc, converged=bool(tr.converged),
                    n_fallback=tr.n_fallback, n_samples=tr.n_samples,
                    trace=dict(precision=prec[:k].copy(), energies=en[:k].copy(), residuals=rs[:k].copy(),
                               elapsed_ms=el[:k].copy()))

    # --- learned preconditioner -----------------------------------------
    def mlp_init(self, seed=0):
        check(_lib.load().qpgpu_mlp_init(self._ctx, seed), self._ctx)

    def mlp_weights(self):
        w = np.empty(_lib.MLP_NPARAM, np.float32)
        check(_lib.load().qpgpu_mlp_get_weights(self._ctx, _p(w)), self._ctx)
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        check(_lib.load().qpgpu_mlp_set_weights(self._ctx, _p(w)), self._ctx)

    def mlp_add_samples(self, X, g, w):
        X = np.ascontiguousarray(X, np.float32)
        g = np.ascontiguousarray(g, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        check(_lib.load().qpgpu_mlp_add_samples(self._ctx, _p(X), _p(g), _p(w), len(g)), self._ctx)

    def mlp_clear_samples(self):
        check(_lib.load().qpgpu_mlp_clear_samples(self._ctx), self._ctx)

    def mlp_n_samples(self):
        return _lib.load().qpgpu_mlp_n_samples(self._ctx)

    def mlp_gradient(self, X, g, w):
        X = np.ascontiguousarray(X, np.float32)
        g = np.ascontiguousarray(g, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        grad = np.empty(_lib.MLP_NPARAM, np.float32)
        loss = C.c_float()
        check(_lib.load().qpgpu_mlp_gradient(self._ctx, _p(X), _p(g), _p(w), len(g), _p(grad), C.byref(loss)),
              self._ctx)
        return grad, loss.value

    def mlp_predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        y = np.empty(len(X), np.float32)
        check(_lib.load().qpgpu_mlp_predict(self._ctx, _p(X), len(X), _p(y)), self._ctx)
        return y

    def mlp_train(self, epochs=20, batch=4096, lr=1e-3, seed=0):
        loss = C.c_float()
        check(_lib.load().qpgpu_mlp_train(self._ctx, epochs, batch, lr, seed, C.byref(loss)), self._ctx)
        return loss.value
