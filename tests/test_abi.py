"""C ABI of libjcg.so: loads without a GPU, exports every declared symbol, and
validates descriptors on the host (error codes, no device work)."""
import ctypes
import os
import re

import pytest

from jax_cosmo_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "jcg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jcg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the whole header
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def _geom(n_tr=2, n_ell=10, n_limber=512):
    g = _lib.Geometry()
    g.abi_version = _lib.ABI_VERSION
    g.n_tracers = n_tr
    g.n_ell = n_ell
    g.n_limber = n_limber
    g.zmax = 4.0
    for t in range(min(n_tr, _lib.MAX_TRACERS)):
        g.kind[t] = _lib.TRACER_WL
        g.nz_a[t], g.nz_b[t], g.nz_z0[t], g.nz_zmax[t] = 1.0, 2.0, 0.5 + t, 4.0
        g.probe_zmax[t] = 4.0
        g.noise[t] = 1e-9
    return g


def test_host_validation_codes():
    lib = _lib.load()
    sz = ctypes.c_size_t()
    g = _geom()
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == 0
    assert sz.value > 0
    g.n_limber = 511
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_ODD_N
    assert b"even" in lib.jcg_last_error_string()
    g = _geom()
    g.abi_version = 99
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_ABI
    g = _geom(n_tr=17)
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_SHAPE
    g = _geom()
    g.nz_z0[0] = float("nan")
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_VALUE
    g = _geom()
    g.kind[1] = 7
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_ARG
    assert lib.jcg_workspace_size(ctypes.byref(_geom()), 0, 0, ctypes.byref(sz)) == _lib.ERR_SHAPE
    assert lib.jcg_workspace_size(ctypes.byref(_geom()), 4, 5, ctypes.byref(sz)) == _lib.ERR_ARG
    # workspace grows linearly with the number of cosmologies
    s1, s2 = ctypes.c_size_t(), ctypes.c_size_t()
    lib.jcg_workspace_size(ctypes.byref(_geom()), 1, 1, ctypes.byref(s1))
    lib.jcg_workspace_size(ctypes.byref(_geom()), 9, 1, ctypes.byref(s2))
    assert s2.value > 8 * s1.value // 2


def test_null_pointer_and_workspace_checks_do_not_touch_the_device():
    lib = _lib.load()
    g = _geom()
    rc = lib.jcg_angular_cl(ctypes.byref(g), None, None, 1, 0, None, None, 0, None)
    assert rc == _lib.ERR_ARG
    buf = ctypes.create_string_buffer(512)
    addr = (ctypes.addressof(buf) + 255) // 256 * 256
    rc = lib.jcg_angular_cl(ctypes.byref(g), ctypes.c_void_p(addr), ctypes.c_void_p(addr), 1, 0,
                            ctypes.c_void_p(addr), ctypes.c_void_p(addr), 16, None)
    assert rc == _lib.ERR_WORKSPACE
    assert lib.jcg_gaussian_covariance(None, 3, 2, None, None, None, 1, 0.25, 1, None, None) == _lib.ERR_ARG


def test_error_mapping():
    with pytest.raises(ValueError):
        _lib.check(_lib.ERR_ODD_N)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.ERR_UNSUPPORTED)
    with pytest.raises(_lib.JcgError):
        _lib.check(_lib.ERR_CUDA)
