"""Request descriptors: probes + ell grid -> ``jcg_geometry`` and its device buffer.

The cosmology-independent tables of a request (Limber nodes, n(z) on every
grid, interpolation segments, ell factors) are built on the device once per
distinct (probes, ell, N) and cached, so repeated likelihood calls with the same
survey set-up only run the per-cosmology kernels.
"""
from __future__ import annotations

import collections
import ctypes
import threading

import numpy as np
import torch

from jax_cosmo_gb300 import _lib
from jax_cosmo_gb300.probes import NumberCounts, WeakLensing
from jax_cosmo_gb300.redshift import delta_nz, redshift_distribution, smail_nz

_CACHE_SIZE = 64
_cache = collections.OrderedDict()
_cache_lock = threading.Lock()


def describe(probes, n_ell, n_limber=512, n_nodes=0, zmax=None, physics=0):
    """Fill a ``jcg_geometry`` from a list of probes (angular_cl.py:63, probes.py)."""
    g = _lib.Geometry()
    g.abi_version = _lib.ABI_VERSION
    g.physics = int(physics)
    n = 0
    for p in probes:
        if isinstance(p, WeakLensing):
            ms = p.multiplicative_biases()
            noise = p.noise().numpy()
            kind = _lib.TRACER_WL
            biases = p.ia_specs()
        elif isinstance(p, NumberCounts):
            ms = [0.0] * p.n_tracers
            noise = p.noise().numpy()
            kind = _lib.TRACER_NC
            biases = p.bias_specs()
        else:
            raise NotImplementedError(f"probe type {type(p).__name__} is not supported")
        pzmax = p.zmax
        for b, pz in enumerate(p.params[0]):
            if not isinstance(pz, redshift_distribution):
                raise NotImplementedError(
                    f"redshift distribution {type(pz).__name__} is not on the accelerated path"
                )
            if isinstance(pz, delta_nz) and kind != _lib.TRACER_WL:
                raise NotImplementedError("single-plane delta_nz bins are supported on WeakLensing probes only")
            if n >= _lib.MAX_TRACERS:
                raise ValueError(f"at most {_lib.MAX_TRACERS} redshift bins per request")
            g.kind[n] = kind
            if isinstance(pz, smail_nz):
                a, bb, z0, zm = pz.device_params()
                g.nz_kind[n] = _lib.NZ_SMAIL
                g.nz_a[n], g.nz_b[n], g.nz_z0[n], g.nz_zmax[n] = a, bb, z0, zm
            elif isinstance(pz, delta_nz):
                # probes.py:53-64: the plane's redshift, no z' integral
                g.nz_kind[n] = _lib.NZ_DELTA
                g.nz_a[n], g.nz_b[n], g.nz_z0[n], g.nz_zmax[n] = 0.0, 0.0, float(pz.params[0]), float(pz.zmax)
            else:
                g.nz_kind[n] = _lib.NZ_TABLE
                g.nz_a[n], g.nz_b[n], g.nz_z0[n], g.nz_zmax[n] = 0.0, 0.0, 1.0, float(pz.zmax)
            g.probe_zmax[n] = float(pzmax)
            bk, bamp, beta, bz0 = biases[b]
            g.bias_kind[n] = int(bk)
            g.bias[n] = bamp
            g.bias_eta[n] = beta
            g.bias_z0[n] = bz0
            g.mult[n] = float(ms[b])
            g.noise[n] = float(noise[b])
            n += 1
    if n == 0:
        raise ValueError("no tracers")
    g.n_tracers = n
    g.n_ell = int(n_ell)
    g.n_limber = int(n_limber)
    g.n_nodes = int(n_nodes)
    g.zmax = float(max(p.zmax for p in probes) if zmax is None else zmax)
    return g


def n_cls_of(g):
    return g.n_tracers * (g.n_tracers + 1) // 2


def ell_host(ell):
    """The ell grid as a 1-D float64 NumPy array (a device tensor is copied once)."""
    if isinstance(ell, torch.Tensor):
        ell = ell.detach().cpu().numpy()
    return np.atleast_1d(np.asarray(ell, dtype=np.float64)).reshape(-1)


def _bins(probes):
    return [pz for p in probes for pz in p.params[0]]


def _nz_key(probes):
    """Cache identity of the tabulated n(z) bins (Smail bins live in the descriptor)."""
    return tuple(pz.cache_key() if not isinstance(pz, (smail_nz, delta_nz)) else "" for pz in _bins(probes))


def _build(g, probes, ell_t, z_nodes, geo, device):
    """Build the geometry; tabulated n(z) bins are evaluated at libjcg's points on the device."""
    st = _lib.stream_of(device)
    bins = _bins(probes)
    if all(isinstance(pz, (smail_nz, delta_nz)) for pz in bins):
        if z_nodes is None:
            _lib.call("jcg_geometry_build", ctypes.byref(g), _lib.ptr(ell_t), _lib.ptr(geo),
                      ctypes.c_size_t(geo.numel()), st)
        else:
            _lib.call("jcg_geometry_build_nodes", ctypes.byref(g), _lib.ptr(ell_t), _lib.ptr(z_nodes),
                      _lib.ptr(geo), ctypes.c_size_t(geo.numel()), st)
        return
    count = ctypes.c_size_t()
    _lib.call("jcg_geometry_nz_points", ctypes.byref(g), _lib.ptr(z_nodes), None, ctypes.byref(count), st)
    zp = torch.empty(count.value, dtype=torch.float64, device=device)
    _lib.call("jcg_geometry_nz_points", ctypes.byref(g), _lib.ptr(z_nodes), _lib.ptr(zp), ctypes.byref(count), st)
    pzv = torch.zeros_like(zp)
    na = g.n_nodes if g.n_nodes > 0 else g.n_limber + 1
    off = 0
    for t, pz in enumerate(bins):
        cnt = 257 + na + (na * 257 if g.kind[t] == _lib.TRACER_WL else 0)
        if not isinstance(pz, (smail_nz, delta_nz)):
            with torch.cuda.device(device):
                pzv[off : off + cnt] = torch.as_tensor(pz.pz_fn(zp[off : off + cnt]), dtype=torch.float64)
        off += cnt
    _lib.call("jcg_geometry_build_nz", ctypes.byref(g), _lib.ptr(ell_t), _lib.ptr(z_nodes), _lib.ptr(pzv),
              ctypes.c_size_t(pzv.numel()), _lib.ptr(geo), ctypes.c_size_t(geo.numel()), st)


def get_geometry(probes, ell, n_limber, device, physics=0):
    """(descriptor, device buffer, device ell) for probes on the ell grid, cached.

    The cache key is the descriptor bytes and the ell values, so repeated calls
    with the same survey set-up build nothing and copy nothing.
    """
    ell_np = ell_host(ell)
    g = describe(probes, ell_np.size, n_limber, physics=physics)
    key = (bytes(g), ell_np.tobytes(), str(device), _nz_key(probes))
    with _cache_lock:
        hit = _cache.get(key)
        if hit is not None:
            _cache.move_to_end(key)
            return hit
    ell_t = torch.as_tensor(ell_np).to(device)
    size = ctypes.c_size_t()
    _lib.call("jcg_geometry_size", ctypes.byref(g), ctypes.byref(size))
    buf = _lib.workspace(size.value, device)
    _build(g, probes, ell_t, None, buf, device)
    val = (g, buf, ell_t)
    with _cache_lock:
        _cache[key] = val
        while len(_cache) > _CACHE_SIZE:
            _cache.popitem(last=False)
    return val


def clear_cache():
    with _cache_lock:
        _cache.clear()


def probe_kernel(probe, cosmo, z, ell):
    """Radial kernel of one probe at arbitrary redshifts on the device.

    Returns (nbins, nz), or (B, nbins, nz) for a batched cosmology, with the
    ell factor and (1 + m) of probes.py:71-74, 205-207 applied.
    """
    device = _lib.require_cuda()
    z_t = torch.as_tensor(np.atleast_1d(np.asarray(z, dtype=np.float64))).reshape(-1).to(device)
    ell_f = float(np.asarray(ell, dtype=np.float64).reshape(-1)[0])
    ell_t = torch.tensor([ell_f], dtype=torch.float64, device=device)
    g = describe([probe], 1, 512, n_nodes=z_t.numel(), physics=cosmo.physics_bits())
    size = ctypes.c_size_t()
    _lib.call("jcg_geometry_size", ctypes.byref(g), ctypes.byref(size))
    geo = _lib.workspace(size.value, device)
    st = _lib.stream_of(device)
    _build(g, [probe], ell_t, z_t, geo, device)
    params = cosmo.param_tensor(device)
    B = params.shape[0]
    wsz = ctypes.c_size_t()
    _lib.call("jcg_workspace_size", ctypes.byref(g), B, _lib.FP64, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    _lib.call("jcg_stage_cosmo_tables", ctypes.byref(g), _lib.ptr(params), B, _lib.FP64,
              _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
    _lib.call("jcg_stage_tracer_kernels", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params), B,
              _lib.FP64, _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
    nb, nz = g.n_tracers, z_t.numel()
    out = torch.empty(B, nb, nz, dtype=torch.float64, device=device)
    for i in range(B):
        _lib.call("jcg_workspace_read", ctypes.byref(g), B, _lib.FP64, _lib.ptr(ws), i, 4,
                  _lib.ptr(out[i]), ctypes.c_size_t(nb * nz), st)
    if isinstance(probe, WeakLensing):
        ef = np.sqrt((ell_f - 1) * (ell_f) * (ell_f + 1) * (ell_f + 2)) / (ell_f + 0.5) ** 2
        out = out * ef
    return out if cosmo.batch_size is not None else out[0]
