"""jcg_angular_cl_noalloc: the entry point for callers that cannot allocate.

Callers such as code inside an XLA custom call or a JAX host callback, where
the framework has already reserved the GPU memory, cannot cudaMalloc a
workspace.  For them jcg_angular_cl_noalloc keeps its scratch in a fixed array
of the library's static device memory.  This test calls it through the C ABI,
twice in a row on different cosmologies (the second call runs on scratch left
by the first), and checks each result against jcg_angular_cl with a caller
workspace, at the tolerances of the other GPU tests.  It also checks that a
request larger than the fixed scratch is refused before anything runs.

The file name sorts last so that a run stopping at the first failure has run
every other test already; it builds everything it needs itself, so it also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from jax_cosmo_gb300 import _geometry, _lib  # noqa: E402

RT64 = 1e-9


def _probes():
    nz = [jc.redshift.smail_nz(1.0, 2.0, z0, gals_per_arcmin2=10.0) for z0 in (0.5, 0.9, 1.3)]
    return [jc.probes.WeakLensing(nz, sigma_e=0.26),
            jc.probes.NumberCounts(nz[:2], jc.bias.constant_linear_bias(1.2))]


def _params(seed, n):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 8))
    p[:, 0] = rng.uniform(0.20, 0.35, n)
    p[:, 1] = rng.uniform(0.04, 0.06, n)
    p[:, 2] = rng.uniform(0.60, 0.80, n)
    p[:, 3] = rng.uniform(0.90, 1.00, n)
    p[:, 4] = rng.uniform(0.60, 1.00, n)
    p[:, 6] = rng.uniform(-1.3, -0.7, n)
    return torch.as_tensor(p, device="cuda")


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)
    lib = _lib.load()
    ell = np.logspace(1, np.log10(3000.0), 40)
    g = _geometry.describe(_probes(), ell.size, 512)
    size = ctypes.c_size_t()
    assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(size)) == 0
    geo = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    ell_t = torch.as_tensor(ell, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.jcg_geometry_build(ctypes.byref(g), ctypes.c_void_p(ell_t.data_ptr()),
                                  ctypes.c_void_p(geo.data_ptr()), size, stream) == 0
    return lib, g, geo, ell_t, stream


def _with_workspace(lib, g, geo, params, prec, stream):
    n = params.shape[0]
    wsz = ctypes.c_size_t()
    assert lib.jcg_workspace_size(ctypes.byref(g), n, prec, ctypes.byref(wsz)) == 0
    ws = torch.empty(wsz.value, dtype=torch.uint8, device="cuda")
    out = torch.empty(n, _geometry.n_cls_of(g), g.n_ell, dtype=torch.float64, device="cuda")
    rc = lib.jcg_angular_cl(ctypes.byref(g), ctypes.c_void_p(geo.data_ptr()),
                            ctypes.c_void_p(params.data_ptr()), n, prec,
                            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()), wsz,
                            stream)
    assert rc == 0, lib.jcg_last_error_string()
    return out


def _no_alloc(lib, g, geo, params, prec, stream):
    n = params.shape[0]
    out = torch.full((n, _geometry.n_cls_of(g), g.n_ell), float("nan"), dtype=torch.float64,
                     device="cuda")
    rc = lib.jcg_angular_cl_noalloc(ctypes.byref(g), ctypes.c_void_p(geo.data_ptr()),
                                    ctypes.c_void_p(params.data_ptr()), n, prec,
                                    ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0, lib.jcg_last_error_string()
    return out


@pytest.mark.parametrize("prec,tol", [(_lib.FP64, RT64), (_lib.FP32C, RT64)])
def test_no_alloc_matches_workspace_entry_point_twice(setup, prec, tol):
    lib, g, geo, ell_t, stream = setup
    for call, (seed, n) in enumerate([(1, 24), (2, 7)]):
        params = _params(seed, n)
        got = _no_alloc(lib, g, geo, params, prec, stream)
        ref = _with_workspace(lib, g, geo, params, prec, stream)
        torch.cuda.synchronize()
        assert torch.isfinite(got).all(), f"call {call}: non-finite output"
        err = ((got - ref).abs() / ref.abs()).max().item()
        assert err <= tol, f"call {call}: max rel err {err:.3e}"


def test_no_alloc_rejects_requests_above_the_scratch_limit(setup):
    lib, g, geo, ell_t, stream = setup
    # smallest batch whose scratch (jcg_workspace_size) exceeds the fixed array
    per = ctypes.c_size_t()
    lib.jcg_workspace_size(ctypes.byref(g), 1, _lib.FP64, ctypes.byref(per))
    n_too_many = max(1, _lib.NOALLOC_SCRATCH_BYTES // per.value)
    need = ctypes.c_size_t()
    while True:
        assert lib.jcg_workspace_size(ctypes.byref(g), n_too_many, _lib.FP64, ctypes.byref(need)) == 0
        if need.value > _lib.NOALLOC_SCRATCH_BYTES:
            break
        n_too_many += 1
    assert need.value > _lib.NOALLOC_SCRATCH_BYTES
    params = _params(3, n_too_many)
    out = torch.empty(n_too_many, _geometry.n_cls_of(g), g.n_ell, dtype=torch.float64, device="cuda")
    rc = lib.jcg_angular_cl_noalloc(ctypes.byref(g), ctypes.c_void_p(geo.data_ptr()),
                                    ctypes.c_void_p(params.data_ptr()), n_too_many, _lib.FP64,
                                    ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == _lib.ERR_WORKSPACE
    assert b"fixed limit" in lib.jcg_last_error_string()
