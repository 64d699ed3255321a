"""Angular power spectra and their Gaussian covariance (jax_cosmo/angular_cl.py).

Drop-in for ``angular_cl``, ``noise_cl``, ``gaussian_cl_covariance`` and
``gaussian_cl_covariance_and_mean``.  All computation runs in libjcg on the GPU:

* ``angular_cl`` -> ``jcg_angular_cl``: background tables, halofit rows, tracer
  kernels and the fused Limber integral, for one cosmology or a batch of B
  cosmologies (Cosmology parameters given as length-B tensors) in one launch
  sequence;
* ``gaussian_cl_covariance`` -> ``jcg_gaussian_covariance``.

Extra keyword arguments (not in the reference): ``precision`` ("fp64" — the
plain float64 method — or "fp32c" — float32 Limber integrand with compensated
sums and float64 tables) and ``n_limber`` (the reference's hard-coded 512
Simpson intervals, angular_cl.py:96).  Results are torch float64 tensors on the
current CUDA device.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from jax_cosmo_gb300 import _geometry, _lib
from jax_cosmo_gb300 import power as power
from jax_cosmo_gb300 import transfer as tklib

__all__ = [
    "angular_cl",
    "noise_cl",
    "gaussian_cl_covariance",
    "gaussian_cl_covariance_and_mean",
]

_PRECISION = {"fp64": _lib.FP64, "fp32c": _lib.FP32C}


def _get_cl_ordering(probes):
    """angular_cl.py:15-25"""
    n_tracers = sum([p.n_tracers for p in probes])
    cl_index = []
    for i in range(n_tracers):
        for j in range(i, n_tracers):
            cl_index.append((i, j))
    return cl_index


def _get_cov_blocks_ordering(probes):
    """angular_cl.py:28-46"""
    cl_index = _get_cl_ordering(probes)
    pos = {p: n for n, p in enumerate(cl_index)}

    def find_index(a, b):
        return pos[(a, b)] if (a, b) in pos else pos[(b, a)]

    cov_blocks = []
    for i, j in cl_index:
        for m, n in cl_index:
            cov_blocks.append(
                (find_index(i, m), find_index(j, n), find_index(i, n), find_index(j, m))
            )
    return cov_blocks


def physics_code(transfer_fn, nonlinear_fn):
    """libjcg physics switches for the operator points of angular_cl.

    transfer_fn: ``transfer.Eisenstein_Hu`` with type "eisenhu_osc" (default) or
    "eisenhu" (transfer.py:99-153), bound with ``functools.partial``;
    nonlinear_fn: ``power.halofit`` with prescription "takahashi2012" (default)
    or "smith2003" (power.py:182-244), or ``power.linear_matter_power``.
    Anything else raises NotImplementedError, as the reference does for an
    unknown type or prescription (transfer.py:155, power.py:226).
    """
    return tklib.transfer_bits(transfer_fn) | power.model_bits(nonlinear_fn)


def _precision_code(precision):
    try:
        return _PRECISION[precision]
    except KeyError:
        raise ValueError(f"precision must be one of {sorted(_PRECISION)}") from None


def angular_cl_device(params, ell, probes, precision="fp64", n_limber=512, out=None, physics=0):
    """C_ell for a [B, 8] float64 parameter tensor on the device -> [B, n_cls, n_ell]
    ([B, 9] with gamma last when ``physics`` has GROWTH_GAMMA).

    Lower-level entry used by the public function, the autograd wrapper and the
    serving loop; ``params`` (and ``out``) live on the device, ``ell`` is a host
    array (the device copy is cached with the geometry); ``physics`` is the
    code of ``physics_code``.
    """
    device = params.device
    g, geo, _ = _geometry.get_geometry(probes, ell, n_limber, device, physics)
    B = params.shape[0]
    prec = _precision_code(precision)
    n_cls = _geometry.n_cls_of(g)
    wsz = ctypes.c_size_t()
    _lib.call("jcg_workspace_size", ctypes.byref(g), B, prec, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    if out is None:
        out = torch.empty(B, n_cls, g.n_ell, dtype=torch.float64, device=device)
    _lib.call(
        "jcg_angular_cl", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params), B, prec,
        _lib.ptr(out), _lib.ptr(ws), ctypes.c_size_t(ws.numel()), _lib.stream_of(device),
    )
    return out


def angular_cl_host(params, ell, probes, precision="fp64", n_limber=512, out=None, physics=0, device=None):
    """C_ell for a [B, 8] float64 parameter tensor in HOST memory -> a host
    [B, n_cls, n_ell] tensor (``jcg_angular_cl_host``).

    The caller without device arrays (a JAX host callback, a CPU sampler):
    the parameters go to the GPU and the C_ell come back inside the call, the
    copies out overlapping the Limber integral of the next range of
    cosmologies.  Pinned tensors (``pin_memory()``) keep the call
    asynchronous: ``out`` is complete after ``torch.cuda.synchronize()`` (or
    the current stream's synchronisation); with pageable tensors the call
    returns after the copies.  ``[B, 9]`` with gamma last when ``physics``
    has GROWTH_GAMMA.
    """
    device = _lib.require_cuda(device)
    if params.device.type != "cpu" or params.dtype != torch.float64 or params.dim() != 2:
        raise ValueError("params must be a [B, 8] float64 host tensor")
    params = params.contiguous()
    g, geo, _ = _geometry.get_geometry(probes, ell, n_limber, device, physics)
    B = params.shape[0]
    prec = _precision_code(precision)
    n_cls = _geometry.n_cls_of(g)
    if out is None:
        out = torch.empty(B, n_cls, g.n_ell, dtype=torch.float64, pin_memory=params.is_pinned())
    elif out.device.type != "cpu" or out.shape != (B, n_cls, g.n_ell) or not out.is_contiguous():
        raise ValueError("out must be a contiguous [B, n_cls, n_ell] float64 host tensor")
    wsz = ctypes.c_size_t()
    _lib.call("jcg_host_workspace_size", ctypes.byref(g), B, prec, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    _lib.call(
        "jcg_angular_cl_host", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params), B, prec,
        _lib.ptr(out), _lib.ptr(ws), ctypes.c_size_t(ws.numel()), _lib.stream_of(device),
    )
    # ws returns to the allocator of the current stream, which has waited for
    # the copies: later work that reuses it runs after them
    return out


def angular_cl(
    cosmo,
    ell,
    probes,
    transfer_fn=tklib.Eisenstein_Hu,
    nonlinear_fn=power.halofit,
    precision="fp64",
    n_limber=512,
):
    """Limber angular power spectra, shape [n_cls, n_ell] (angular_cl.py:49-98).

    A batched cosmology gives [B, n_cls, n_ell].  Differentiable with respect to
    Cosmology parameters that are tensors with ``requires_grad``.
    """
    physics = physics_code(transfer_fn, nonlinear_fn) | cosmo.physics_bits()
    device = _lib.require_cuda()
    ell_np = _geometry.ell_host(ell)
    if cosmo.requires_grad():
        from jax_cosmo_gb300 import autodiff

        cl = autodiff.angular_cl_autograd(cosmo, ell_np, probes, precision, n_limber, physics)
    else:
        params = cosmo.param_tensor(device)
        cl = angular_cl_device(params, ell_np, probes, precision, n_limber, physics=physics)
    return cl if cosmo.batch_size is not None else cl[0]


def noise_cl(ell, probes):
    """Noise on the auto-spectra, [n_cls, n_ell] (angular_cl.py:101-117)."""
    device = _lib.require_cuda()
    n_ell = len(np.atleast_1d(np.asarray(ell)))
    noise = torch.cat([p.noise() for p in probes]).to(device)
    cl_index = _get_cl_ordering(probes)
    out = torch.zeros(len(cl_index), n_ell, dtype=torch.float64, device=device)
    for k, (i, j) in enumerate(cl_index):
        if i == j:
            out[k] = noise[i] * 1.0
    return out


def _covariance(ell_t, n_tracers, cl_signal, cl_noise, tracer_noise, f_sky, sparse):
    device = ell_t.device
    sig = cl_signal.to(device=device, dtype=torch.float64).contiguous()
    batched = sig.dim() == 3
    if not batched:
        sig = sig[None]
    B, n_cls, n_ell = sig.shape
    if n_cls != n_tracers * (n_tracers + 1) // 2 or n_ell != ell_t.numel():
        raise ValueError(f"cl_signal shape {tuple(cl_signal.shape)} does not match the probes and ell")
    cn = None
    if cl_noise is not None:
        cn = torch.as_tensor(cl_noise, dtype=torch.float64).to(device)
        cn = cn.expand(n_cls, n_ell).contiguous()
    tn = None if tracer_noise is None else tracer_noise.to(device=device, dtype=torch.float64).contiguous()
    N = n_cls * n_ell
    shape = (B, n_cls, n_cls, n_ell) if sparse else (B, N, N)
    out = torch.empty(shape, dtype=torch.float64, device=device)
    _lib.call(
        "jcg_gaussian_covariance", _lib.ptr(ell_t), n_ell, n_tracers, _lib.ptr(sig), _lib.ptr(cn),
        _lib.ptr(tn), B, ctypes.c_double(float(f_sky)), 1 if sparse else 0, _lib.ptr(out),
        _lib.stream_of(device),
    )
    return out if batched else out[0]


def gaussian_cl_covariance(ell, probes, cl_signal, cl_noise, f_sky=0.25, sparse=True):
    """Gaussian covariance (angular_cl.py:120-163).

    sparse=True: (n_cls, n_cls, n_ell) block diagonals; else the dense
    (n_cls n_ell, n_cls n_ell) matrix.  A leading batch axis on cl_signal is kept.
    """
    device = _lib.require_cuda()
    ell_t = torch.as_tensor(_geometry.ell_host(ell)).to(device)
    n_tr = sum(p.n_tracers for p in probes)
    if not isinstance(cl_signal, torch.Tensor):
        cl_signal = torch.as_tensor(np.asarray(cl_signal, dtype=np.float64))
    if cl_signal.requires_grad:
        from jax_cosmo_gb300 import autodiff

        return autodiff.covariance_autograd(cl_signal, ell_t, n_tr, cl_noise, None, f_sky, sparse)
    return _covariance(ell_t, n_tr, cl_signal, cl_noise, None, f_sky, sparse)


def gaussian_cl_covariance_and_mean(
    cosmo,
    ell,
    probes,
    transfer_fn=tklib.Eisenstein_Hu,
    nonlinear_fn=power.halofit,
    f_sky=0.25,
    sparse=False,
    precision="fp64",
    n_limber=512,
):
    """(signal mean flattened [n_cls*n_ell], covariance) (angular_cl.py:166-196).

    The mean is the signal only; the covariance uses signal + noise.  Both are
    differentiable in the Cosmology parameters that require grad.
    """
    device = _lib.require_cuda()
    ell_np = _geometry.ell_host(ell)
    cl_signal = angular_cl(cosmo, ell_np, probes, transfer_fn, nonlinear_fn, precision, n_limber)
    _, _, ell_t = _geometry.get_geometry(probes, ell_np, n_limber, device)
    tracer_noise = torch.cat([p.noise() for p in probes])
    n_tr = tracer_noise.numel()
    if cl_signal.requires_grad:
        from jax_cosmo_gb300 import autodiff

        cov = autodiff.covariance_autograd(cl_signal, ell_t, n_tr, None, tracer_noise, f_sky, sparse)
    else:
        cov = _covariance(ell_t, n_tr, cl_signal, None, tracer_noise, f_sky, sparse)
    if cl_signal.dim() == 3:
        return cl_signal.reshape(cl_signal.shape[0], -1), cov
    return cl_signal.flatten(), cov
