"""Batches of independent CI problems solved together on one GPU.

Wraps qpgpu_batch_* (include/qpgpu.h): one persistent sigma launch per
Davidson iteration for all problems, batched Davidson algebra, CUDA-graph
replay of the device part of each iteration, autotuned launch shape.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FP64


class BatchError(RuntimeError):
    pass


class Batch:
    def __init__(self, wavefunctions):
        self.wfs = list(wavefunctions)
        L = _lib.load()
        arr = (C.c_void_p * len(self.wfs))(*[w.ctx for w in self.wfs])
        h = C.c_void_p()
        rc = L.qpgpu_batch_create(arr, len(self.wfs), C.byref(h))
        if rc != 0:
            raise BatchError(f"qpgpu_batch_create failed ({rc})")
        self._b = h

    def close(self):
        if getattr(self, "_b", None):
            _lib.load().qpgpu_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def davidson(self, guesses, n_states, threshold=1e-10, s2_eig=False, precision=FP64, davidson_sze_max=8,
                 max_iter=500):
        """guesses[p]: (N_st_diag, N_p) arrays; n_states[p] <= N_st_diag.
        Returns dict(energies (n, N_st_diag), s2, vectors, stats)."""
        L = _lib.load()
        np_ = len(self.wfs)
        us = [np.ascontiguousarray(g, dtype=np.float64).copy() for g in guesses]
        nsd = us[0].shape[0]
        ptrs = (C.c_void_p * np_)(*[u.ctypes.data for u in us])
        dims = np.array([u.shape[1] for u in us], np.int64)
        nst = np.array(n_states, np.int32)
        e = np.zeros((np_, nsd))
        s2 = np.zeros((np_, nsd))
        iters = np.zeros(np_, np.int32)
        prm = _lib.DavidsonParams(n_states=int(nst.max()), n_states_diag=nsd, davidson_sze_max=davidson_sze_max,
                                  s2_eig=int(bool(s2_eig)), threshold=threshold, precision=precision,
                                  defect_every=0, preconditioner=0, max_iter=max_iter, collect_every=0,
                                  collect_max=0)
        st = _lib.BatchStats(iters=iters.ctypes.data)
        rc = L.qpgpu_batch_davidson(self._b, ptrs, dims.ctypes.data, nst.ctypes.data, e.ctypes.data, s2.ctypes.data,
                                    C.byref(prm), C.byref(st))
        if rc != 0:
            raise BatchError(f"{_lib.ERRORS.get(rc, rc)}: {L.qpgpu_batch_last_error(self._b).decode()}")
        stats = {f: getattr(st, f) for f, _ in st._fields_ if f not in ("iters", "pad")}
        stats["iters"] = iters
        return dict(energies=e, s2=s2, vectors=us, stats=stats)
