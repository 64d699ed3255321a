"""Derivatives of the angular_cl path for torch.autograd.

jax_cosmo differentiates its whole stack with ``jax.grad`` / ``jax.hessian``
(README.md:14-27).  Here the three functions of the path are
``torch.autograd.Function``s whose backward passes run in libjcg:

* ``angular_cl``: backward = v^T J by ``jcg_angular_cl_vjp`` (tables
  differentiated forward, the Limber integrand by a hand-written reverse
  sweep weighted by the cotangent, so that fp32c never forms J; theta = the
  8 Cosmology leaves of core.py:98-108);
* ``gaussian_cl_covariance``: the Knox formula (angular_cl.py:144-147) is a
  product of two C_ell, its vector-Jacobian product is applied with index
  additions on the device;
* ``gaussian_log_likelihood``: d logL / d mu = -C^-1 r (C^-1 r from the same
  per-ell Cholesky as the value), d logL / d C = (C^-1 r r^T C^-1 + C^-1) / 2
  with the reference's +0.5 logdet sign (likelihood.py:61).

``angular_cl_jacobian`` returns J itself, and ``fisher_matrix`` the Gaussian
Fisher matrix J^T C^-1 J of a C_ell data vector (the construction of the
reference's intro notebook).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from jax_cosmo_gb300 import _geometry, _lib

PARAM_ORDER = ("Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa")
FISHER_PARAMS = ("Omega_c", "Omega_b", "h", "n_s", "sigma8", "w0", "wa")


def jacobian_device(params, ell, probes, n_limber=512, precision="fp64", physics=0, gamma_dir=-1):
    """(C_ell [B, n_cls, n_ell], dC/dtheta [B, n_cls, n_ell, 8]) for [B, 8] params on the device
    ([B, 9] with gamma last when ``physics`` has GROWTH_GAMMA).

    precision "fp64" (plain) or "fp32c" (float32 lensing kernels and Limber
    integrand with its reverse sweep, compensated a-sums; float64 tables);
    physics: the code of ``angular_cl.physics_code``; gamma_dir in 0..7: that
    column of the Jacobian holds dC/dgamma instead of its parameter's.
    """
    from jax_cosmo_gb300.angular_cl import _precision_code

    prec = _precision_code(precision)
    device = params.device
    g, geo, _ = _geometry.get_geometry(probes, ell, n_limber, device, physics)
    B = params.shape[0]
    n_cls = _geometry.n_cls_of(g)
    wsz = ctypes.c_size_t()
    _lib.call("jcg_jacobian_workspace_size", ctypes.byref(g), B, prec, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    cl = torch.empty(B, n_cls, g.n_ell, dtype=torch.float64, device=device)
    jac = torch.empty(B, n_cls, g.n_ell, len(PARAM_ORDER), dtype=torch.float64, device=device)
    _lib.call(
        "jcg_angular_cl_jacobian_dir", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params.contiguous()), B, prec,
        int(gamma_dir), _lib.ptr(cl), _lib.ptr(jac), _lib.ptr(ws), ctypes.c_size_t(ws.numel()),
        _lib.stream_of(device),
    )
    return cl, jac


def vjp_device(params, ell, probes, cl_bar, n_limber=512, precision="fp64", physics=0, gamma_dir=-1,
               want_cl=False):
    """Vector-Jacobian product of angular_cl for [B, 8] params (``jcg_angular_cl_vjp``):
    grad [B, 8] = sum_{p,l} cl_bar[b, p, l] dC_p(l)/dtheta, and C_ell [B, n_cls, n_ell]
    when ``want_cl``.  fp32c forms no Jacobian (the Limber integrand's reverse
    sweep weighted by the cotangent); fp64 contracts the FP64 Jacobian."""
    from jax_cosmo_gb300.angular_cl import _precision_code

    prec = _precision_code(precision)
    device = params.device
    g, geo, _ = _geometry.get_geometry(probes, ell, n_limber, device, physics)
    B = params.shape[0]
    n_cls = _geometry.n_cls_of(g)
    wsz = ctypes.c_size_t()
    _lib.call("jcg_vjp_workspace_size", ctypes.byref(g), B, prec, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    vb = cl_bar.to(device=device, dtype=torch.float64).expand(B, n_cls, g.n_ell).contiguous()
    grad = torch.empty(B, len(PARAM_ORDER), dtype=torch.float64, device=device)
    cl = torch.empty(B, n_cls, g.n_ell, dtype=torch.float64, device=device) if want_cl else None
    _lib.call("jcg_angular_cl_vjp", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params.contiguous()), B, prec,
              int(gamma_dir), _lib.ptr(vb), _lib.ptr(cl), _lib.ptr(grad), _lib.ptr(ws), ctypes.c_size_t(ws.numel()),
              _lib.stream_of(device))
    return (grad, cl) if want_cl else grad


class _AngularCl(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, ell, probes, precision, n_limber, physics):
        from jax_cosmo_gb300.angular_cl import angular_cl_device

        ctx.meta = (ell, probes, n_limber, precision, physics)
        ctx.save_for_backward(params)
        return angular_cl_device(params.detach().contiguous(), ell, probes, precision, n_limber, physics=physics)

    @staticmethod
    def backward(ctx, gcl):
        (params,) = ctx.saved_tensors
        ell, probes, n_limber, precision, physics = ctx.meta
        p = params.detach().contiguous()
        g64 = gcl.to(torch.float64)
        gp = vjp_device(p, ell, probes, g64, n_limber, precision, physics)
        if params.shape[1] > gp.shape[1]:
            # gamma (the 9th leaf): a second product with the gamma tangent in direction 0
            gg = vjp_device(p, ell, probes, g64, n_limber, precision, physics, gamma_dir=0)
            gp = torch.cat([gp, gg[:, :1]], dim=1)
        return gp, None, None, None, None, None


def angular_cl_autograd(cosmo, ell, probes, precision="fp64", n_limber=512, physics=0):
    device = _lib.require_cuda()
    params = cosmo.param_tensor(device, differentiable=True)
    return _AngularCl.apply(params, ell, probes, precision, n_limber, physics)


def angular_cl_jacobian(cosmo, ell, probes, n_limber=512, precision="fp64", transfer_fn=None, nonlinear_fn=None):
    """(C_ell, dC_ell/dtheta) with theta = (Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa),
    and gamma last when the Cosmology has one (the pytree leaves of core.py:52-60).

    Shapes [n_cls, n_ell] and [n_cls, n_ell, 8] (9 with gamma; a leading
    batch axis for a batched Cosmology).  precision "fp64" or "fp32c";
    transfer_fn and nonlinear_fn as in ``angular_cl`` (None: the defaults).
    """
    from jax_cosmo_gb300 import power, transfer
    from jax_cosmo_gb300.angular_cl import physics_code

    physics = physics_code(transfer_fn or transfer.Eisenstein_Hu, nonlinear_fn or power.halofit)
    physics |= cosmo.physics_bits()
    device = _lib.require_cuda()
    params = cosmo.param_tensor(device)
    ell_np = _geometry.ell_host(ell)
    cl, jac = jacobian_device(params, ell_np, probes, n_limber, precision, physics)
    if params.shape[1] > len(PARAM_ORDER):
        _, jg = jacobian_device(params, ell_np, probes, n_limber, precision, physics, gamma_dir=0)
        jac = torch.cat([jac, jg[..., :1]], dim=-1)
    if cosmo.batch_size is None:
        return cl[0], jac[0]
    return cl, jac


# ------------------------------------------------------------- covariance ----
def _cov_index(n_tr, device):
    from jax_cosmo_gb300.angular_cl import _get_cov_blocks_ordering

    class _P:  # minimal probe stand-in with n_tracers
        n_tracers = n_tr

    blocks = torch.as_tensor(np.array(_get_cov_blocks_ordering([_P()])), device=device)
    return blocks[:, 0], blocks[:, 1], blocks[:, 2], blocks[:, 3]


class _Covariance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, cl_signal, ell_t, n_tr, cl_noise, tracer_noise, f_sky, sparse):
        from jax_cosmo_gb300.angular_cl import _covariance

        ctx.meta = (ell_t, n_tr, cl_noise, tracer_noise, f_sky, sparse)
        ctx.save_for_backward(cl_signal)
        return _covariance(ell_t, n_tr, cl_signal.detach(), cl_noise, tracer_noise, f_sky, sparse)

    @staticmethod
    def backward(ctx, gcov):
        (sig,) = ctx.saved_tensors
        ell_t, n_tr, cl_noise, tracer_noise, f_sky, sparse = ctx.meta
        batched = sig.dim() == 3
        s3 = sig if batched else sig[None]
        g = gcov if batched else gcov[None]
        B, n_cls, n_ell = s3.shape
        if not sparse:  # the entries that depend on C_ell: the per-ell diagonals of each block
            g4 = g.reshape(B, n_cls, n_ell, n_cls, n_ell)
            idx = torch.arange(n_ell, device=g.device)
            g = g4[:, :, idx, :, idx].permute(1, 2, 3, 0)  # [B, n_cls, n_cls, n_ell]
        ell = ell_t.detach().cpu().numpy()
        norm = torch.as_tensor((2 * ell + 1) * np.gradient(ell) * f_sky, device=g.device)
        obs = s3.detach().clone()
        if cl_noise is not None:
            obs = obs + torch.as_tensor(cl_noise, dtype=torch.float64, device=g.device)
        elif tracer_noise is not None:
            tn = tracer_noise.to(g.device, torch.float64)
            from jax_cosmo_gb300.angular_cl import _get_cl_ordering

            class _P:
                n_tracers = n_tr

            for k, (i, j) in enumerate(_get_cl_ordering([_P()])):
                if i == j:
                    obs[:, k] = obs[:, k] + tn[i]
        a, b, c, d = _cov_index(n_tr, g.device)
        gn = g.reshape(B, n_cls * n_cls, n_ell) / norm
        go = torch.zeros_like(obs)
        go.index_add_(1, a, gn * obs[:, b])
        go.index_add_(1, b, gn * obs[:, a])
        go.index_add_(1, c, gn * obs[:, d])
        go.index_add_(1, d, gn * obs[:, c])
        return (go if batched else go[0]), None, None, None, None, None, None


def covariance_autograd(cl_signal, ell_t, n_tr, cl_noise, tracer_noise, f_sky, sparse):
    return _Covariance.apply(cl_signal, ell_t, n_tr, cl_noise, tracer_noise, f_sky, sparse)


# ------------------------------------------------------------- likelihood ----
class _LogLike(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, mu, C, include_logdet, sparse, n_cls, n_ell):
        from jax_cosmo_gb300.likelihood import _loglike_core

        C = C.detach().contiguous()
        alpha = torch.empty(mu.shape, dtype=torch.float64, device=mu.device)
        out, status = _loglike_core(data.detach().contiguous(), mu.detach().contiguous(), C, sparse,
                                    n_cls, n_ell, include_logdet, alpha=alpha)
        ctx.meta = (include_logdet, sparse, n_cls, n_ell)
        ctx.save_for_backward(alpha, C, status)
        return out

    @staticmethod
    def backward(ctx, gout):
        alpha, C, status = ctx.saved_tensors
        include_logdet, sparse, n_cls, n_ell = ctx.meta
        go = gout.to(torch.float64)
        g_data = alpha * go[:, None]
        g_mu = -g_data
        g_C = None
        if ctx.needs_input_grad[2]:
            B = alpha.shape[0]
            if sparse:
                a3 = alpha.reshape(B, n_cls, n_ell)
                g = torch.einsum("bpl,bql->bpql", a3, a3)
                if include_logdet:
                    g = g + _sparse_inv_batched(C)
                g_C = 0.5 * g * go[:, None, None, None]
            else:
                g = torch.einsum("bi,bj->bij", alpha, alpha)
                if include_logdet:
                    g = g + _dense_inverse(C, status, n_cls, n_ell)
                g_C = 0.5 * g * go[:, None, None]
        return g_data, g_mu, g_C, None, None, None, None


def _dense_blocks(C, n_cls, n_ell):
    """[B, N, N] (cls, ell)-ordered, block diagonal in ell -> [B, n_cls, n_cls, n_ell]."""
    B = C.shape[0]
    g4 = C.reshape(B, n_cls, n_ell, n_cls, n_ell)
    idx = torch.arange(n_ell, device=C.device)
    return g4[:, :, idx, :, idx].permute(1, 2, 3, 0).contiguous()  # [B, n_cls, n_cls, n_ell]


def _sparse_inv_batched(S):
    from jax_cosmo_gb300 import sparse as sp

    return sp.inv_batched(S)


def _dense_inverse(C, status, n_cls, n_ell):
    """C^-1 of [B, N, N] (cls, ell)-ordered matrices: one batched per-ell block
    inverse (libjcg) scattered into the dense layout; a matrix flagged as not
    block diagonal in ell (status 1) is inverted whole (torch Cholesky)."""
    from jax_cosmo_gb300 import sparse as sp

    B = C.shape[0]
    blocks = _dense_blocks(C, n_cls, n_ell)                       # [B, n_cls, n_cls, n_ell]
    ib = sp.inv_batched(blocks)
    out = torch.zeros_like(C)
    idx = torch.arange(n_ell, device=C.device)
    out.view(B, n_cls, n_ell, n_cls, n_ell)[:, :, idx, :, idx] = ib.permute(3, 0, 1, 2)
    whole = status == 1
    if bool(whole.any()):  # a user covariance with ell-ell correlations
        for i in whole.nonzero().flatten().tolist():
            out[i] = torch.cholesky_inverse(torch.linalg.cholesky(C[i]))
    return out


def loglike_autograd(data2, mu2, Cb, include_logdet, sparse, n_cls, n_ell):
    return _LogLike.apply(data2, mu2, Cb, include_logdet, sparse, n_cls, n_ell)


# ----------------------------------------------------------------- Fisher ----
def fisher_matrix(cosmo, ell, probes, f_sky=0.25, n_limber=512, params=FISHER_PARAMS, precision="fp64"):
    """Gaussian Fisher matrix F = J^T C^-1 J of the C_ell data vector.

    J = dC_ell/dtheta for the named parameters (a subset of PARAM_ORDER), C the
    Gaussian covariance with noise (angular_cl.py:120-163) at ``cosmo``, inverted
    per ell block.
    """
    from jax_cosmo_gb300.angular_cl import gaussian_cl_covariance, noise_cl

    cl, jac = angular_cl_jacobian(cosmo, ell, probes, n_limber, precision)
    if cl.dim() != 2:
        raise ValueError("fisher_matrix takes a single (unbatched) cosmology")
    names = PARAM_ORDER + (("gamma",) if jac.shape[-1] > len(PARAM_ORDER) else ())
    unknown = [p for p in params if p not in names]
    if unknown:
        raise ValueError(f"unknown parameters {unknown}; this cosmology has {names}")
    sel = [names.index(p) for p in params]
    J = jac[..., sel]  # [n_cls, n_ell, P]
    cov = gaussian_cl_covariance(ell, probes, cl, noise_cl(ell, probes), f_sky, sparse=True)
    Cl = cov.permute(2, 0, 1)  # [n_ell, n_cls, n_cls]
    Jl = J.permute(1, 0, 2)  # [n_ell, n_cls, P]
    X = torch.linalg.solve(Cl, Jl)
    return torch.einsum("lcp,lcq->pq", Jl, X)


# ----------------------------------------------------------------- Hessian ---
def jacobian_branch(params, ell, probes, n_limber=512, seg_in=None, want_seg=False):
    """FP64 (C_ell, dC/dtheta) of [B, 8] params with the halofit root find's
    segments exposed (``jcg_angular_cl_jacobian_branch``): ``seg_in`` [B, na]
    imposes them, ``want_seg`` returns them as a third value."""
    device = params.device
    g, geo, _ = _geometry.get_geometry(probes, ell, n_limber, device, 0)
    B = params.shape[0]
    n_cls = _geometry.n_cls_of(g)
    na = int(g.n_limber) + 1
    wsz = ctypes.c_size_t()
    _lib.call("jcg_jacobian_workspace_size", ctypes.byref(g), B, _lib.FP64, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    cl = torch.empty(B, n_cls, g.n_ell, dtype=torch.float64, device=device)
    jac = torch.empty(B, n_cls, g.n_ell, len(PARAM_ORDER), dtype=torch.float64, device=device)
    seg = torch.empty(B, na, dtype=torch.int32, device=device) if want_seg else None
    if seg_in is not None:
        seg_in = seg_in.to(device=device, dtype=torch.int32).expand(B, na).contiguous()
    _lib.call("jcg_angular_cl_jacobian_branch", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params.contiguous()), B,
              _lib.ptr(seg_in), _lib.ptr(seg), _lib.ptr(cl), _lib.ptr(jac), _lib.ptr(ws),
              ctypes.c_size_t(ws.numel()), _lib.stream_of(device))
    return (cl, jac, seg) if want_seg else (cl, jac)


def loglike_hessian(cosmo, ell, probes, data, f_sky=0.25, n_limber=512, include_logdet=True, rel_step=1e-3):
    """Hessian of the README likelihood over the 8 Cosmology leaves
    (README.md:14-27: ``F = -jax.hessian(likelihood)(cosmo)``), with

        mu, C = gaussian_cl_covariance_and_mean(cosmo, ell, probes, f_sky)
        likelihood = gaussian_log_likelihood(data, mu, C, include_logdet)

    mean and covariance both at the cosmology (angular_cl.py:166-196,
    likelihood.py:9-61).  Returns (H [8, 8], gradient [8], logL).

    The gradient is exact (the hand-written FP64 Jacobian of C_ell, then the
    covariance and likelihood adjoints).  Each Hessian column is the
    derivative of that gradient along one leaf, taken by central differences
    of the exact gradient at steps h and h/2 combined by Richardson
    extrapolation (error O(h^4)), all 32 parameter points in one batched
    Jacobian launch.  The points are evaluated on the piece of the base
    point: the halofit root find's interpolation segments found at the base
    point are imposed on every perturbed point, which is the derivative
    jax.hessian takes (the argmin is locally constant).  Steps: rel_step
    times |theta_b|, or rel_step absolute for a zero-valued leaf.
    """
    device = _lib.require_cuda()
    if cosmo.batch_size is not None:
        raise ValueError("loglike_hessian takes a single (unbatched) cosmology")
    if cosmo.physics_bits():
        raise NotImplementedError("loglike_hessian: the gamma growth is not supported")

    ell_np = _geometry.ell_host(ell)
    p0 = cosmo.param_tensor(device)[:1]
    D = len(PARAM_ORDER)
    _, _, seg = jacobian_branch(p0, ell_np, probes, n_limber, want_seg=True)
    x0 = p0[0].detach().cpu().numpy()
    steps = np.where(x0 != 0.0, rel_step * np.abs(x0), rel_step)
    pts = []
    for scale in (1.0, 0.5):
        for b in range(D):
            for sgn in (1.0, -1.0):
                x = x0.copy()
                x[b] += sgn * scale * steps[b]
                pts.append(x)
    pts.append(x0)
    P = torch.as_tensor(np.array(pts), dtype=torch.float64, device=device)
    cl, jac = jacobian_branch(P, ell_np, probes, n_limber, seg_in=seg)
    B, n_cls, n_ell = cl.shape
    _, _, ell_t = _geometry.get_geometry(probes, ell_np, n_limber, device)
    tracer_noise = torch.cat([p.noise() for p in probes])
    mu = cl.detach().reshape(B, -1).clone().requires_grad_(True)
    cov = covariance_autograd(mu.reshape(B, n_cls, n_ell), ell_t, tracer_noise.numel(), None, tracer_noise,
                              f_sky, True)
    data_t = torch.as_tensor(data, dtype=torch.float64).to(device).reshape(1, -1).expand(B, -1).contiguous()
    ll = loglike_autograd(data_t, mu, cov, include_logdet, True, n_cls, n_ell)
    (dmu,) = torch.autograd.grad(ll.sum(), mu)
    g = torch.einsum("bn,bnd->bd", dmu, jac.reshape(B, n_cls * n_ell, D))  # exact gradients [B, 8]
    g = g.cpu().numpy()
    h = steps
    d1 = (g[0:2 * D:2] - g[1:2 * D:2]) / (2.0 * h[:, None])               # step h:   rows = leaf b
    d2 = (g[2 * D:4 * D:2] - g[2 * D + 1:4 * D:2]) / (1.0 * h[:, None])    # step h/2
    H = (4.0 * d2 - d1) / 3.0
    H = 0.5 * (H + H.T)
    return torch.as_tensor(H), torch.as_tensor(g[-1]), float(ll[-1].detach())
