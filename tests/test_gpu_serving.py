"""GPU tests of the ragged-request path and the serving loop.

* jcg_requests_run forward modes: each request of a ragged list (own probes,
  tracer count and ell grid) equals angular_cl of that request alone (FP64:
  1e-14 relative; FP32C: 1e-4 of FP64);
* served log-likelihood + gradient (covariance fixed) against the public API
  differentiated by torch.autograd (fp64: 1e-10 / 1e-8 of the largest
  component) and against the float64 oracle differentiated by torch autograd
  (fp64: 1e-8; fp32c: 1e-4);
* each result is the same alone and in a mix of chains (fp64: 1e-12, fp32c:
  1e-6 of the largest component: only the grouping of the a-split partial sums
  may differ);
* admission under a small HBM budget completes every request within budget.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from jax_cosmo_gb300 import serving  # noqa: E402
from oracle import jc_oracle as O  # noqa: E402

NAMES = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
FID = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]
BOX_LO = np.array([0.20, 0.04, 0.60, 0.90, 0.60, 0.0, -1.3, 0.0])
BOX_HI = np.array([0.35, 0.06, 0.80, 1.00, 1.00, 0.0, -0.7, 0.0])


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)


def cosmo_of(row, grad=False):
    return jc.Cosmology(**{n: (torch.tensor(float(v), dtype=torch.float64, requires_grad=True) if grad else float(v))
                           for n, v in zip(NAMES, row)})


def chain_spec(seed, max_tr=10, max_ell=500):
    """Seeded chain: 1..max_tr tracers (WeakLensing / NumberCounts mix), smail_nz
    a=1, b=2, z0 in U[0.3, 1.5], 20..max_ell log-spaced ell in [10, 5000]."""
    rng = np.random.default_rng(seed)
    n_tr = int(rng.integers(1, max_tr + 1))
    n_wl = int(rng.integers(0, n_tr + 1))
    z0 = rng.uniform(0.3, 1.5, n_tr)
    n_ell = int(rng.integers(20, max_ell + 1))
    ell = np.logspace(1, np.log10(5000), n_ell)
    probes, spec = [], []
    if n_wl:
        bins = [(1.0, 2.0, float(z), 10.0, 10.0) for z in z0[:n_wl]]
        probes.append(jc.probes.WeakLensing([jc.redshift.smail_nz(1.0, 2.0, z, gals_per_arcmin2=10.0) for z in z0[:n_wl]],
                                            sigma_e=0.26))
        spec.append(O.Probe("wl", [O.Smail(*b) for b in bins], sigma_e=0.26))
    if n_tr > n_wl:
        bins = [(1.0, 2.0, float(z), 10.0, 10.0) for z in z0[n_wl:]]
        probes.append(jc.probes.NumberCounts([jc.redshift.smail_nz(1.0, 2.0, z, gals_per_arcmin2=10.0) for z in z0[n_wl:]],
                                             jc.bias.constant_linear_bias(1.2)))
        spec.append(O.Probe("nc", [O.Smail(*b) for b in bins], bias=1.2))
    return probes, ell, spec


def make_model(seed, **kw):
    probes, ell, spec = chain_spec(seed, **kw)
    mu = jc.cl.angular_cl(cosmo_of(FID), ell, probes).flatten()
    rng = np.random.default_rng(seed + 1000)
    data = mu * (1.0 + 0.01 * torch.as_tensor(rng.standard_normal(mu.numel()), device=mu.device))
    return serving.ChainModel(probes, ell, data), probes, ell, spec


def box_point(rng):
    return list(BOX_LO + (BOX_HI - BOX_LO) * rng.uniform(size=8))


def scale_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_ragged_forward_matches_single():
    rng = np.random.default_rng(5)
    items = []
    for seed in (11, 12, 13, 14):
        probes, ell, _ = chain_spec(seed, max_ell=120)
        items.append((cosmo_of(box_point(rng)), ell, probes))
    out64 = serving.angular_cl_ragged(items, precision="fp64")
    out32 = serving.angular_cl_ragged(items, precision="fp32c")
    for (c, ell, probes), a, b in zip(items, out64, out32):
        ref = jc.cl.angular_cl(c, ell, probes)
        assert a.shape == ref.shape
        assert float(((a - ref) / ref).abs().max()) < 1e-14
        assert float(((b - ref) / ref).abs().max()) < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_served_matches_api_and_oracle(precision):
    model, probes, ell, spec = make_model(21, max_ell=60)
    row = [0.27, 0.05, 0.70, 0.95, 0.78, 0.0, -0.9, 0.0]
    with serving.Server(hbm_budget=256 << 20, precision=precision) as srv:
        r = srv.submit(model, row).result(timeout=120)
    tv, tg = (1e-10, 1e-8) if precision == "fp64" else (1e-4, 1e-4)
    # public API: angular_cl differentiated by autograd, covariance fixed
    c = cosmo_of(row, grad=True)
    mu = jc.cl.angular_cl(c, ell, probes).flatten()
    res = mu - model.data
    alpha = torch.einsum("lpq,ql->pl", model.prec, res.reshape(model.n_cls, model.n_ell)).flatten()
    ll = -0.5 * torch.dot(res, alpha)
    ll.backward()
    g = np.array([float(getattr(c, n).grad) for n in NAMES])
    assert abs(r.loglike - float(ll.detach())) <= tv * abs(float(ll.detach()))
    assert scale_err(r.grad, g) < tg
    # oracle differentiated by torch autograd
    v = torch.tensor(row, dtype=torch.float64, requires_grad=True)
    mu_o = O.angular_cl(O.Cosmo.from_vector(v), ell, spec).flatten()
    res_o = mu_o - model.data.cpu()
    P = model.prec.cpu()
    ll_o = -0.5 * torch.dot(res_o, torch.einsum("lpq,ql->pl", P, res_o.reshape(model.n_cls, model.n_ell)).flatten())
    ll_o.backward()
    assert abs(r.loglike - float(ll_o.detach())) <= max(tv, 1e-8) * abs(float(ll_o.detach()))
    assert scale_err(r.grad, v.grad.numpy()) < tg


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32c", 1e-6)])
def test_alone_equals_mix(precision, tol):
    models = [make_model(s, max_ell=150)[0] for s in (31, 32, 33, 34, 35, 36)]
    rng = np.random.default_rng(9)
    rows = [[box_point(rng) for _ in range(3)] for _ in models]
    alone = {}
    with serving.Server(hbm_budget=512 << 20, n_streams=1, precision=precision) as srv:
        for i, m in enumerate(models):
            for j, row in enumerate(rows[i]):
                alone[(i, j)] = srv.submit(m, row).result(timeout=120)
    with serving.Server(hbm_budget=512 << 20, n_streams=2, precision=precision) as srv:
        futs = {(i, j): srv.submit(m, row) for i, m in enumerate(models) for j, row in enumerate(rows[i])}
        mix = {k: f.result(timeout=120) for k, f in futs.items()}
        st = srv.stats()
    assert st["max_batch"] > 1  # the mix did share launches
    for k in alone:
        assert abs(mix[k].loglike - alone[k].loglike) <= tol * abs(alone[k].loglike)
        assert scale_err(mix[k].grad, alone[k].grad) < tol


def test_small_hbm_budget_admission():
    models = [make_model(s, max_ell=100)[0] for s in (41, 42, 43)]
    budget = int(2.5 * max(m.footprint for m in models))
    rng = np.random.default_rng(3)
    with serving.Server(hbm_budget=budget, n_streams=2) as srv:
        futs = [srv.submit(models[k % 3], box_point(rng)) for k in range(12)]
        res = [f.result(timeout=300) for f in futs]
        st = srv.stats()
    assert st["completed"] == 12 and st["failed"] == 0
    assert st["arena_peak_bytes"] <= budget
    assert all(np.isfinite(r.loglike) and np.all(np.isfinite(r.grad)) for r in res)


def test_batches_overlap_on_two_streams():
    """Continuous batching: requests that arrive while a batch runs launch on
    the second stream at once, and the two batches' device intervals (CUDA
    events around each batch on its stream) intersect."""
    models = [make_model(s, max_ell=500)[0] for s in (51, 52, 53, 54)]
    rng = np.random.default_rng(4)
    with serving.Server(hbm_budget=4 << 30, n_streams=2, max_batch=24, trace=True) as srv:
        futs = [srv.submit(models[k % 4], box_point(rng)) for k in range(96)]
        res = [f.result(timeout=300) for f in futs]
    iv = srv.device_intervals()
    assert len(res) == 96 and all(np.isfinite(r.loglike) for r in res)
    assert {s for s, _, _ in iv} == {0, 1}
    overlaps = [(a, b) for a in iv for b in iv
                if a[0] == 0 and b[0] == 1 and b[1] < a[2] and a[1] < b[2]]
    print("batches", len(iv), "overlapping pairs", len(overlaps), "first intervals", iv[:4])
    assert overlaps, iv


def test_requests_run_does_not_wait_for_the_stream():
    """jcg_requests_run returns while earlier work still runs on its stream:
    the request tables go through the pinned staging ring, not a pageable
    copy.  A 50 ms spin kernel (torch.cuda._sleep, a bounded wait) is queued
    first; the call returns in a small fraction of it, and the results equal
    those of an unobstructed call."""
    import ctypes
    import time

    from jax_cosmo_gb300 import _lib

    model = make_model(61, max_ell=80)[0]
    n = 8
    rng = np.random.default_rng(6)
    params = torch.as_tensor(np.array([box_point(rng) for _ in range(n)]), device="cuda").contiguous()
    out = torch.zeros(n, 9, dtype=torch.float64, device="cuda")
    table = np.zeros(n, _lib.REQUEST_DTYPE)
    for i in range(n):
        model._fill(table, i, params.data_ptr() + 64 * i, out.data_ptr() + 72 * i)
    tp = ctypes.c_void_p(table.ctypes.data)
    lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
    _lib.call("jcg_requests_workspace_size", tp, n, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, ctypes.byref(lo),
              ctypes.byref(hi))
    ws = _lib.workspace(hi.value, params.device)
    stream = torch.cuda.current_stream()
    st = ctypes.c_void_p(stream.cuda_stream)

    def run():
        _lib.call("jcg_requests_run", tp, n, _lib.REQ_LOGLIKE_GRAD, _lib.FP32C, _lib.ptr(ws),
                  ctypes.c_size_t(ws.numel()), st)

    run()  # first call: constant tables and the staging ring are set up
    torch.cuda.synchronize()
    ref = out.clone()
    out.zero_()
    torch.cuda.synchronize()
    torch.cuda._sleep(100_000_000)  # about 50 ms at the 2.07 GHz SM clock
    t0 = time.perf_counter()
    run()
    dt = time.perf_counter() - t0
    torch.cuda.synchronize()
    print("jcg_requests_run host time %.3f ms behind a 50 ms kernel" % (dt * 1e3))
    assert dt < 0.01, dt
    assert torch.equal(out, ref)
