"""C ABI of libjcg.so: loads without a GPU, exports every declared symbol, and
validates descriptors on the host (error codes, no device work)."""
import ctypes
import os
import re

import pytest

from jax_cosmo_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = "".join(open(os.path.join(ROOT, "include", h)).read() for h in ("jcg.h", "jcg_calib.h"))
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
    # host-buffer entry: NULL geometry, then a workspace below jcg_host_workspace_size
    assert lib.jcg_angular_cl_host(ctypes.byref(g), None, ctypes.c_void_p(addr), 1, 0, ctypes.c_void_p(addr),
                                   ctypes.c_void_p(addr), 16, None) == _lib.ERR_ARG
    rc = lib.jcg_angular_cl_host(ctypes.byref(g), ctypes.c_void_p(addr), ctypes.c_void_p(addr), 1, 0,
                                 ctypes.c_void_p(addr), ctypes.c_void_p(addr), 16, None)
    assert rc == _lib.ERR_WORKSPACE
    s1, s2 = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.jcg_workspace_size(ctypes.byref(g), 7, 1, ctypes.byref(s1)) == 0
    assert lib.jcg_host_workspace_size(ctypes.byref(g), 7, 1, ctypes.byref(s2)) == 0
    assert s2.value >= s1.value + 7 * 8 * 8


def test_error_mapping():
    with pytest.raises(ValueError):
        _lib.check(_lib.ERR_ODD_N)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.ERR_UNSUPPORTED)
    with pytest.raises(_lib.JcgError):
        _lib.check(_lib.ERR_CUDA)


def test_jacobian_and_request_validation_on_the_host():
    """Argument checks of the Jacobian and ragged-request entry points return
    error codes before any device work."""
    import numpy as np

    lib = _lib.load()
    g = _geom()
    sz = ctypes.c_size_t()
    assert lib.jcg_jacobian_workspace_size(ctypes.byref(g), 0, _lib.FP64, ctypes.byref(sz)) == _lib.ERR_SHAPE
    assert lib.jcg_jacobian_workspace_size(ctypes.byref(g), 2, 7, ctypes.byref(sz)) == _lib.ERR_ARG
    assert lib.jcg_jacobian_workspace_size(ctypes.byref(g), 2, _lib.FP32C, ctypes.byref(sz)) == 0
    s64, s32 = ctypes.c_size_t(), ctypes.c_size_t()
    lib.jcg_jacobian_workspace_size(ctypes.byref(g), 64, _lib.FP64, ctypes.byref(s64))
    lib.jcg_jacobian_workspace_size(ctypes.byref(g), 64, _lib.FP32C, ctypes.byref(s32))
    assert s64.value > 0 and s32.value > 0
    assert lib.jcg_angular_cl_jacobian(ctypes.byref(g), None, None, 1, _lib.FP64, None, None, None, 0,
                                       None) == _lib.ERR_ARG
    # the gamma direction needs the gamma growth and a direction in 0..7
    assert lib.jcg_angular_cl_jacobian_dir(ctypes.byref(g), None, None, 1, _lib.FP64, 0, None, None, None, 0,
                                           None) == _lib.ERR_ARG
    assert b"GROWTH_GAMMA" in lib.jcg_last_error_string()
    g.physics = _lib.GROWTH_GAMMA
    assert lib.jcg_angular_cl_jacobian_dir(ctypes.byref(g), None, None, 1, _lib.FP64, 8, None, None, None, 0,
                                           None) == _lib.ERR_ARG
    g.physics = 0
    lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
    table = np.zeros(2, _lib.REQUEST_DTYPE)
    tp = ctypes.c_void_p(table.ctypes.data)
    # no requests, too many, unknown mode or precision
    assert lib.jcg_requests_workspace_size(tp, 0, _lib.REQ_CL, _lib.FP64, ctypes.byref(lo),
                                           ctypes.byref(hi)) == _lib.ERR_SHAPE
    assert lib.jcg_requests_workspace_size(tp, _lib.MAX_REQUESTS + 1, _lib.REQ_CL, _lib.FP64, ctypes.byref(lo),
                                           ctypes.byref(hi)) == _lib.ERR_SHAPE
    assert lib.jcg_requests_workspace_size(tp, 2, 9, _lib.FP64, ctypes.byref(lo), ctypes.byref(hi)) == _lib.ERR_ARG
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_CL, 5, ctypes.byref(lo), ctypes.byref(hi)) == _lib.ERR_ARG
    # a request without a geometry, then one whose pointers are missing
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_CL, _lib.FP64, ctypes.byref(lo),
                                           ctypes.byref(hi)) == _lib.ERR_ARG
    g2 = _geom(n_tr=3, n_ell=7)
    fake = 4096  # host-side checks only look at NULL-ness; nothing is dereferenced
    for i, gg in enumerate((g, g2)):
        table[i] = (ctypes.addressof(gg), fake, fake, fake, 0, 0, 0, 0)
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_CL, _lib.FP64, ctypes.byref(lo), ctypes.byref(hi)) == 0
    assert lo.value == hi.value > 0
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_JACOBIAN, _lib.FP32C, ctypes.byref(lo),
                                           ctypes.byref(hi)) == _lib.ERR_ARG  # jac NULL
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, ctypes.byref(lo),
                                           ctypes.byref(hi)) == _lib.ERR_ARG  # data / prec / out NULL
    for i, gg in enumerate((g, g2)):
        table[i] = (ctypes.addressof(gg), fake, fake, 0, 0, fake, fake, fake)
    assert lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, ctypes.byref(lo),
                                           ctypes.byref(hi)) == 0
    assert hi.value >= lo.value > 0
    # the workspace is additive in the requests: two requests need more than one
    one_lo = ctypes.c_size_t()
    lib.jcg_requests_workspace_size(tp, 1, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, ctypes.byref(one_lo),
                                    ctypes.byref(hi))
    assert lo.value > one_lo.value
    # run refuses a NULL or misaligned workspace before any launch
    assert lib.jcg_requests_run(tp, 2, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, None, 0, None) == _lib.ERR_ARG
    # a geometry with an odd Limber N inside a request is reported with its index
    g2.n_limber = 511
    rc = lib.jcg_requests_workspace_size(tp, 2, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, ctypes.byref(lo),
                                         ctypes.byref(hi))
    assert rc == _lib.ERR_ODD_N
    assert b"request 1" in lib.jcg_last_error_string()


def test_ragged_requests_refuse_the_gamma_growth_on_the_host():
    """A request carries 8 parameters and 8 derivative columns, so a geometry
    with the gamma growth (a 9th parameter) is refused before any launch."""
    import numpy as np

    lib = _lib.load()
    g = _geom()
    g.physics = _lib.GROWTH_GAMMA
    lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
    table = np.zeros(1, _lib.REQUEST_DTYPE)
    fake = 4096  # never dereferenced: the check comes first
    table[0] = (ctypes.addressof(g), fake, fake, fake, fake, fake, fake, fake)
    tp = ctypes.c_void_p(table.ctypes.data)
    for mode in (_lib.REQ_CL, _lib.REQ_JACOBIAN, _lib.REQ_LOGLIKE_GRAD):
        rc = lib.jcg_requests_workspace_size(tp, 1, mode, _lib.FP32C, ctypes.byref(lo), ctypes.byref(hi))
        assert rc == _lib.ERR_UNSUPPORTED
        assert b"GROWTH_GAMMA" in lib.jcg_last_error_string()
        assert lib.jcg_requests_run(tp, 1, mode, _lib.FP64, None, 0, None) == _lib.ERR_UNSUPPORTED


def test_limber_entry_points_refuse_caller_redshift_nodes():
    """A geometry on caller redshift nodes (jcg_geometry_build_nodes) has no
    Limber grid: angular_cl and the Limber stage refuse it on the host, as the
    no-allocation and Jacobian entry points do."""
    lib = _lib.load()
    g = _geom()
    g.n_nodes = 40
    buf = ctypes.create_string_buffer(1 << 16)
    addr = ctypes.c_void_p((ctypes.addressof(buf) + 255) // 256 * 256)
    assert lib.jcg_angular_cl(ctypes.byref(g), addr, addr, 1, _lib.FP64, addr, addr, 1 << 12, None) == _lib.ERR_ARG
    assert b"Limber grid" in lib.jcg_last_error_string()
    assert lib.jcg_stage_limber(ctypes.byref(g), addr, addr, 1, _lib.FP32C, addr, addr, 1 << 12,
                                None) == _lib.ERR_ARG
    assert b"Limber grid" in lib.jcg_last_error_string()
    assert lib.jcg_angular_cl_noalloc(ctypes.byref(g), addr, addr, 1, _lib.FP64, addr, None) == _lib.ERR_ARG
    assert lib.jcg_angular_cl_host(ctypes.byref(g), addr, addr, 1, _lib.FP64, addr, addr, 1 << 12,
                                   None) == _lib.ERR_ARG
