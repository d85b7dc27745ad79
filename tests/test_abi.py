"""The C-ABI library builds for sm_103a, loads and exports every declared symbol (no GPU needed)."""
import ctypes

from quantum_package_gb300 import _lib


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = _lib.declared_symbols()
    assert "qpgpu_h_s2_u0" in names and "qpgpu_set_dets" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_create_rejects_bad_shapes_without_gpu_work():
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.qpgpu_create(300, 2, 2, 5, ctypes.byref(h)) == -1      # n_mo too large
    assert L.qpgpu_create(129, 4, 4, 3, ctypes.byref(h)) == -1      # N_int = 3 (n_mo <= 128 supported)
    assert L.qpgpu_create(80, 14, 14, 1, ctypes.byref(h)) == -1     # wrong n_int
    assert L.qpgpu_create(80, 10, 12, 2, ctypes.byref(h)) == -1     # n_alpha < n_beta
    assert L.qpgpu_destroy(None) == -1


def test_every_entry_point_has_a_signature_and_rejects_null_arguments():
    """Each function of include/qpgpu.h is bound with its C signature, and called with null
    handles / pointers and zero sizes it returns an error (or its null-handle value) before
    touching the device, as the Fortran shim relies on to turn failures into `stop`."""
    L = _lib.load()
    for name in _lib.declared_symbols():
        f = getattr(L, name)
        assert f.argtypes is not None, f"{name} has no ctypes signature"
        args = []
        for t in f.argtypes:
            if t in (ctypes.c_int, ctypes.c_int64, ctypes.c_uint64):
                args.append(0)
            elif t is ctypes.c_float:
                args.append(0.0)
            else:
                args.append(None)
        r = f(*args)
        if f.restype is ctypes.c_char_p:
            assert r in (b"null context", b"null batch"), (name, r)
        else:
            assert r < 0, (name, r)
