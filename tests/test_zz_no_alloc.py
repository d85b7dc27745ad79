"""qpgpu_sigma_bilinear_noalloc: sigma for callers that cannot let the library allocate.

Some hosts own all device memory through their own pool allocator, or overlap
sigma with work on other streams and cannot accept the device-wide
synchronisation of cudaMalloc/cudaFree.  This entry point keeps its scratch in
a fixed array of the library instead.  The test calls it through the C-ABI,
twice in a row, and checks it against qpgpu_sigma_bilinear (the regular entry
point) at the tolerance of the other sigma tests; it also checks that a
problem too large for the fixed scratch is refused with QPGPU_ERR_ARG, as are
float-float requests, and that a direct-sigma set is refused with
QPGPU_ERR_STATE.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from quantum_package_gb300 import FP32, FP64
from quantum_package_gb300 import _lib
from quantum_package_gb300 import generate as G

pytestmark = pytest.mark.gpu

REL = {FP64: 1e-12, FP32: 2e-6}


def _sigma(L, wf, fn, u, u32, prec):
    import torch
    v = torch.full_like(u, float("nan"))
    s = torch.full_like(u, float("nan"))
    rc = fn(wf.ctx, C.c_void_p(v.data_ptr()), C.c_void_p(s.data_ptr()), C.c_void_p(u.data_ptr()),
            C.c_void_p(u32.data_ptr()), u.shape[1], prec, None)
    _lib.check(rc, wf.ctx)
    torch.cuda.synchronize()
    return v.cpu().numpy(), s.cpu().numpy()


@pytest.mark.parametrize("cfg,n_det,n_st", [(1, 5_000, 1), (2, 20_000, 4)])
def test_noalloc_matches_regular_entry_point_twice(cfg, n_det, n_st):
    import torch
    from quantum_package_gb300.sigma import Wavefunction
    L = _lib.load()
    p = G.make_problem(cfg, n_det=n_det, n_states=n_st)
    wf = Wavefunction.from_problem(p)
    if cfg == 2:
        # rows split over several work chunks: the fixed scratch is really used
        assert wf.info()["n_split_rows"] > 0
    u = torch.from_numpy(np.ascontiguousarray(G.random_coefficients(p.n_det, n_st, 7).T)).cuda()
    u32 = u.float()
    for prec in (FP64, FP32):
        ref_v, ref_s = _sigma(L, wf, L.qpgpu_sigma_bilinear, u, u32, prec)
        for _ in range(2):
            v, s = _sigma(L, wf, L.qpgpu_sigma_bilinear_noalloc, u, u32, prec)
            scale = np.abs(ref_v).max()
            assert np.isfinite(v).all() and np.isfinite(s).all()
            assert np.abs(v - ref_v).max() <= REL[prec] * scale
            assert np.abs(s - ref_s).max() <= REL[prec] * max(1.0, np.abs(ref_s).max())


def test_noalloc_refuses_problems_beyond_its_scratch():
    import torch
    from quantum_package_gb300.sigma import Wavefunction
    L = _lib.load()
    p = G.make_problem(1, n_det=70_000)
    wf = Wavefunction.from_problem(p)
    u = torch.zeros((p.n_det, 8), dtype=torch.float64, device="cuda")
    v, s = torch.empty_like(u), torch.empty_like(u)
    rc = L.qpgpu_sigma_bilinear_noalloc(wf.ctx, C.c_void_p(v.data_ptr()), C.c_void_p(s.data_ptr()),
                                        C.c_void_p(u.data_ptr()), None, 8, FP64, None)
    assert rc == -1
    assert b"scratch" in L.qpgpu_last_error(wf.ctx)


def test_noalloc_first_fp32_call_and_refusals():
    # an FP32 call on a fresh context (no FP32 launch shape tuned yet) runs the
    # default shape; float-float precision and direct-sigma sets are refused
    import torch
    from quantum_package_gb300 import FF, SIGMA_DIRECT
    from quantum_package_gb300.sigma import Wavefunction
    L = _lib.load()
    p = G.make_problem(2, n_det=20_000, n_states=2)
    wf = Wavefunction.from_problem(p)
    u = torch.from_numpy(np.ascontiguousarray(G.random_coefficients(p.n_det, 2, 9).T)).cuda()
    u32 = u.float()
    v, s = _sigma(L, wf, L.qpgpu_sigma_bilinear_noalloc, u, u32, FP32)
    ref_v, ref_s = _sigma(L, wf, L.qpgpu_sigma_bilinear, u, u32, FP32)
    assert np.abs(v - ref_v).max() <= REL[FP32] * np.abs(ref_v).max()
    assert np.abs(s - ref_s).max() <= REL[FP32] * max(1.0, np.abs(ref_s).max())
    out = torch.empty_like(u)
    rc = L.qpgpu_sigma_bilinear_noalloc(wf.ctx, C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()),
                                        C.c_void_p(u.data_ptr()), C.c_void_p(u32.data_ptr()), 2, FF, None)
    assert rc == -1  # QPGPU_ERR_ARG
    q = G.make_problem(1, n_det=3_000)
    wd = Wavefunction.from_problem(q, sigma_mode=SIGMA_DIRECT)
    ud = torch.zeros((q.n_det, 1), dtype=torch.float64, device="cuda")
    vd = torch.empty_like(ud)
    rc = L.qpgpu_sigma_bilinear_noalloc(wd.ctx, C.c_void_p(vd.data_ptr()), C.c_void_p(vd.data_ptr()),
                                        C.c_void_p(ud.data_ptr()), None, 1, FP64, None)
    assert rc == -2  # QPGPU_ERR_STATE
    assert b"stored pairs" in L.qpgpu_last_error(wd.ctx)
