"""GPU parity of the derivatives: libjcg's Jacobian dC_ell/dtheta (FP64) and the
autograd backward passes of angular_cl, the covariance and the log-likelihood,
against the float64 oracle differentiated by torch autograd (it stands in for
jax.grad / jax.hessian of the reference) and against central finite differences
(step 1e-4 relative) of libjcg's own FP64 forward.

Tolerances: Jacobian vs oracle autograd 1e-8 of each column's largest entry
(fp64) and 1e-4 (fp32c: float32 lensing kernels and Limber integrand with its
reverse sweep); vs central FD 1e-5 of the column scale (FD truncation error at
h = 1e-4); gradients of the log-likelihood 1e-7 relative (fp64), 1e-4 (fp32c).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from oracle import jc_oracle as O  # noqa: E402

NAMES = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
FID = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]
OTHER = [0.31, 0.045, 0.66, 0.98, 0.72, 0.0, -0.85, 0.15]
TOL_J = 1e-8
TOL_FD = 1e-5
TOL_G = 1e-7
TOL_J32 = 1e-4
TOL_G32 = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)


def cosmo_of(row, grad=False):
    return jc.Cosmology(**{n: (torch.tensor(float(v), dtype=torch.float64, requires_grad=True) if grad else float(v))
                           for n, v in zip(NAMES, row)})


def cosmo_batch(rows):
    rows = np.asarray(rows)
    return jc.Cosmology(**{n: torch.tensor(rows[:, i]) for i, n in enumerate(NAMES)})


# (kind, [(a, b, z0, zmax, gals_per_arcmin2)], extra)
MIXED = [("wl", [(1.0, 2.0, 0.5, 4.0, 10), (1.0, 2.0, 1.0, 4.0, 10)], {"sigma_e": 0.26, "m": 0.01}),
         ("nc", [(1.0, 2.0, 0.8, 4.0, 5)], {"bias": 1.2})]
WL5 = [("wl", [(1.0, 2.0, z0, 10.0, 10) for z0 in np.linspace(0.3, 1.5, 5)], {"sigma_e": 0.26})]
TWO_GROUPS = [("wl", [(1.0, 2.0, 0.6, 3.0, 8)], {"sigma_e": 0.28}),
              ("wl", [(1.0, 2.0, 1.1, 6.0, 8)], {"sigma_e": 0.25})]


def jc_probes(spec):
    out = []
    for kind, bins, extra in spec:
        nz = [jc.redshift.smail_nz(a, b, z0, gals_per_arcmin2=ng, zmax=zm) for a, b, z0, zm, ng in bins]
        if kind == "wl":
            out.append(jc.probes.WeakLensing(nz, sigma_e=extra.get("sigma_e", 0.26),
                                             multiplicative_bias=extra.get("m", 0.0)))
        else:
            out.append(jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(extra["bias"])))
    return out


def oracle_probes(spec):
    out = []
    for kind, bins, extra in spec:
        e = {"sigma_e": extra.get("sigma_e", 0.26), "m": extra.get("m", 0.0)} if kind == "wl" else {"bias": extra["bias"]}
        out.append(O.Probe(kind, [O.Smail(a, b, z0, zm, ng) for a, b, z0, zm, ng in bins], **e))
    return out


def oracle_jacobian(row, ell, spec, n_limber):
    probes = oracle_probes(spec)

    def f(v):
        return O.angular_cl(O.Cosmo.from_vector(v), ell, probes, n_limber=n_limber)

    v0 = torch.tensor(row, dtype=torch.float64)
    return f(v0), torch.autograd.functional.jacobian(f, v0)


def col_err(J, Jref):
    """max over parameters of max|J - Jref| / max|Jref| for that parameter."""
    J = J.detach().cpu().double()
    Jref = Jref.detach().cpu().double()
    errs = []
    for d in range(Jref.shape[-1]):
        scale = float(Jref[..., d].abs().max())
        errs.append(float((J[..., d] - Jref[..., d]).abs().max()) / max(scale, 1e-300))
    return max(errs)


@pytest.mark.parametrize("spec,ell,n_limber", [
    (MIXED, np.geomspace(10, 3000, 6), 128),
    (TWO_GROUPS, np.array([3.0, 40.0, 700.0, 2500.0]), 96),
])
def test_jacobian_vs_oracle_autograd(spec, ell, n_limber):
    for row in (FID, OTHER):
        cl_o, J_o = oracle_jacobian(row, ell, spec, n_limber)
        cl, J = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, jc_probes(spec), n_limber)
        assert J.shape == J_o.shape
        # the Jacobian entry point's C_ell is the FP64 forward up to summation order
        fwd = jc.cl.angular_cl(cosmo_of(row), ell, jc_probes(spec), n_limber=n_limber)
        assert float(((cl - fwd) / fwd).abs().max()) < 1e-12
        assert float(((cl.cpu() - cl_o) / cl_o).abs().max()) < 1e-9
        assert col_err(J, J_o) < TOL_J, col_err(J, J_o)
        cl32, J32 = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, jc_probes(spec), n_limber, "fp32c")
        assert float(((cl32.cpu() - cl_o) / cl_o).abs().max()) < 1e-4
        assert col_err(J32, J_o) < TOL_J32, col_err(J32, J_o)


def test_jacobian_with_intrinsic_alignment_vs_oracle():
    """NLA intrinsic alignment (des_y1, constant, inverse-growth biases) and
    inverse-growth NumberCounts bias: Jacobian vs the oracle's autograd."""
    ell = np.geomspace(10, 3000, 5)
    pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
    pc = jc.redshift.smail_nz(1.0, 2.0, 0.8, gals_per_arcmin2=5, zmax=4.0)
    probes = [jc.probes.WeakLensing([pa, pc], ia_bias=[jc.bias.des_y1_ia_bias(1.2, 0.6, 0.62),
                                                       jc.bias.inverse_growth_linear_bias(0.7)],
                                    multiplicative_bias=[0.01, -0.02]),
              jc.probes.NumberCounts([pa], jc.bias.inverse_growth_linear_bias(1.3))]
    oa, oc = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 0.8, 4.0, 5)
    oprobes = [O.Probe("wl", [oa, oc], m=[0.01, -0.02], ia=[("desy1", 1.2, 0.6, 0.62), ("invg", 0.7)]),
               O.Probe("nc", [oa], bias=("invg", 1.3))]

    def f(v):
        return O.angular_cl(O.Cosmo.from_vector(v), ell, oprobes, n_limber=128)

    v0 = torch.tensor(OTHER, dtype=torch.float64)
    cl_o = f(v0)
    J_o = torch.autograd.functional.jacobian(f, v0, strategy="forward-mode", vectorize=True)
    for prec, tc, tj in (("fp64", 1e-9, TOL_J), ("fp32c", 1e-4, TOL_J32)):
        cl, J = jc.autodiff.angular_cl_jacobian(cosmo_of(OTHER), ell, probes, 128, prec)
        fwd = jc.cl.angular_cl(cosmo_of(OTHER), ell, probes, n_limber=128, precision=prec)
        assert float(((fwd.cpu() - cl_o) / cl_o).abs().max()) < tc
        assert float(((cl.cpu() - cl_o) / cl_o).abs().max()) < tc
        assert col_err(J, J_o) < tj, (prec, col_err(J, J_o))


def test_jacobian_vs_central_fd():
    ell = np.geomspace(10, 3000, 8)
    probes = jc_probes(MIXED)
    _, J = jc.autodiff.angular_cl_jacobian(cosmo_of(OTHER), ell, probes, 128)
    rows = []
    steps = []
    for d in range(8):
        h = 1e-4 * max(abs(OTHER[d]), 1.0) if d != 5 else 1e-4
        for s in (+1, -1):
            r = list(OTHER)
            r[d] += s * h
            rows.append(r)
        steps.append(h)
    cl = jc.cl.angular_cl(cosmo_batch(rows), ell, probes, n_limber=128)
    fd = torch.stack([(cl[2 * d] - cl[2 * d + 1]) / (2 * steps[d]) for d in range(8)], dim=-1)
    assert col_err(J, fd) < TOL_FD, col_err(J, fd)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32c", 1e-6)])
def test_batched_jacobian_matches_single(precision, tol):
    """Only the grouping of the a-split partial sums depends on the batch size."""
    ell = np.geomspace(20, 3000, 10)
    probes = jc_probes(WL5)
    rows = [FID, OTHER, [0.22, 0.055, 0.72, 0.93, 0.9, 0.0, -1.2, 0.0]]
    cl_b, J_b = jc.autodiff.angular_cl_jacobian(cosmo_batch(rows), ell, probes, 256, precision)
    for i, row in enumerate(rows):
        cl, J = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, probes, 256, precision)
        assert float(((cl_b[i] - cl) / cl).abs().max()) < tol
        assert col_err(J_b[i], J) < tol


def test_angular_cl_backward():
    ell = np.geomspace(10, 3000, 6)
    c = cosmo_of(FID, grad=True)
    cl = jc.cl.angular_cl(c, ell, jc_probes(MIXED), n_limber=128)
    w = torch.linspace(0.5, 1.5, cl.numel(), dtype=torch.float64, device=cl.device).reshape(cl.shape)
    (cl * w / cl.detach()).sum().backward()
    _, J_o = oracle_jacobian(FID, ell, MIXED, 128)
    cl_o = O.angular_cl(O.Cosmo.from_vector(FID), ell, oracle_probes(MIXED), n_limber=128)
    g_o = torch.einsum("pl,pld->d", w.cpu() / cl_o, J_o)
    g = torch.stack([getattr(c, n).grad for n in NAMES])
    err = float((g.cpu() - g_o).abs().max() / g_o.abs().max())
    assert err < TOL_G, err


def _loglike_setup(ell, spec):
    """data = fiducial C_ell + seeded noise drawn from its own covariance (f_sky = 0.25)."""
    probes = jc_probes(spec)
    mu, cov = jc.cl.gaussian_cl_covariance_and_mean(cosmo_of(FID), ell, probes, sparse=False)
    L = torch.linalg.cholesky(cov)
    gen = torch.Generator(device="cpu").manual_seed(7)
    z = torch.randn(mu.numel(), generator=gen, dtype=torch.float64).to(mu.device)
    return (mu + L @ z).detach()


@pytest.mark.parametrize("sparse,include_logdet,precision", [(True, True, "fp64"), (False, True, "fp64"),
                                                              (True, False, "fp64"), (True, True, "fp32c")])
def test_loglike_gradient_vs_oracle(sparse, include_logdet, precision):
    """d logL / d(7 parameters) through mean AND covariance, vs oracle autograd."""
    ell = np.geomspace(10, 3000, 12)
    data = _loglike_setup(ell, WL5)
    c = cosmo_of(OTHER, grad=True)
    mu, cov = jc.cl.gaussian_cl_covariance_and_mean(c, ell, jc_probes(WL5), sparse=sparse, n_limber=256,
                                                    precision=precision)
    ll = jc.likelihood.gaussian_log_likelihood(data, mu, cov, include_logdet=include_logdet)
    ll.backward()
    g = torch.stack([getattr(c, n).grad for n in NAMES])

    v = torch.tensor(OTHER, dtype=torch.float64, requires_grad=True)
    mu_o, cov_o = O.gaussian_cl_covariance_and_mean(O.Cosmo.from_vector(v), ell, oracle_probes(WL5),
                                                    sparse=sparse, n_limber=256)
    ll_o = O.gaussian_log_likelihood(data.cpu(), mu_o, cov_o, include_logdet=include_logdet)
    ll_o.backward()
    tol_v, tol_g = (1e-9, TOL_G) if precision == "fp64" else (1e-4, TOL_G32)
    assert abs(float(ll.detach()) - float(ll_o.detach())) <= tol_v * abs(float(ll_o.detach()))
    sel = [0, 1, 2, 3, 4, 6, 7]  # Omega_k is not a sampled parameter of the likelihood
    err = float((g[sel].cpu() - v.grad[sel]).abs().max() / v.grad[sel].abs().max())
    assert err < tol_g, err


def test_loglike_gradient_in_mu_and_cov():
    """Backward of the log-likelihood alone, against torch autograd of the dense formula."""
    torch.manual_seed(3)
    n_cls, n_ell = 6, 9
    N = n_cls * n_ell
    A = torch.randn(n_ell, n_cls, n_cls, dtype=torch.float64)
    blocks = (A @ A.transpose(1, 2) + n_cls * torch.eye(n_cls, dtype=torch.float64)).permute(1, 2, 0).contiguous()
    data = torch.randn(N, dtype=torch.float64)
    mu = torch.randn(N, dtype=torch.float64)
    for sparse in (True, False):
        C = blocks if sparse else O.to_dense(blocks)
        mu_d = mu.cuda().requires_grad_(True)
        C_d = C.cuda().requires_grad_(True)
        jc.likelihood.gaussian_log_likelihood(data.cuda(), mu_d, C_d).backward()
        mu_r = mu.clone().requires_grad_(True)
        C_r = C.clone().requires_grad_(True)
        Cd = O.to_dense(C_r) if sparse else C_r
        r = mu_r - data
        (-0.5 * (r @ torch.linalg.solve(Cd, r) - torch.linalg.slogdet(Cd)[1])).backward()
        assert float((mu_d.grad.cpu() - mu_r.grad).abs().max()) < 1e-10 * float(mu_r.grad.abs().max())
        assert float((C_d.grad.cpu() - C_r.grad).abs().max()) < 1e-10 * float(C_r.grad.abs().max())


def test_fisher_matrix_vs_oracle():
    ell = np.geomspace(10, 3000, 12)
    F = jc.autodiff.fisher_matrix(cosmo_of(FID), ell, jc_probes(WL5), n_limber=256)
    _, J_o = oracle_jacobian(FID, ell, WL5, 256)
    cl_o = O.angular_cl(O.Cosmo.from_vector(FID), ell, oracle_probes(WL5), n_limber=256)
    cov_o = O.gaussian_cl_covariance(ell, 5, cl_o, O.noise_cl(ell, oracle_probes(WL5)), 0.25, sparse=True)
    sel = [0, 1, 2, 3, 4, 6, 7]
    Jl = J_o[..., sel].permute(1, 0, 2)
    F_o = torch.einsum("lcp,lcq->pq", Jl, torch.linalg.solve(cov_o.permute(2, 0, 1), Jl))
    assert F.shape == (7, 7)
    err = float((F.cpu() - F_o).abs().max() / F_o.abs().max())
    assert err < TOL_G, err


def _vjp_case(spec, ell, physics=0, gamma=None, B=5, seed=3):
    """A batch around the fiducial, a seeded cotangent and the FP64 Jacobian."""
    from jax_cosmo_gb300 import _geometry
    from jax_cosmo_gb300.autodiff import jacobian_device

    rng = np.random.default_rng(seed)
    rows = np.array([FID] * B) * (1.0 + 0.04 * rng.uniform(-1, 1, (B, 8)))
    rows[:, 5] = 0.0
    rows[:, 7] = 0.02 * rng.uniform(-1, 1, B)
    if gamma is not None:
        rows = np.concatenate([rows, np.full((B, 1), gamma)], axis=1)
    params = torch.as_tensor(rows, device="cuda").contiguous()
    probes = jc_probes(spec)
    ell = _geometry.ell_host(ell)
    n_cls = sum(len(b) for _, b, _ in spec)
    n_cls = n_cls * (n_cls + 1) // 2
    vbar = torch.as_tensor(rng.standard_normal((B, n_cls, len(ell))), device="cuda")
    cl64, J64 = jacobian_device(params, ell, probes, 512, "fp64", physics)
    return params, probes, ell, vbar, cl64, J64


@pytest.mark.parametrize("physics", [0, "smith2003", "linear", "nowiggle"])
def test_vjp_matches_jacobian_contraction(physics):
    """jcg_angular_cl_vjp against the FP64 Jacobian contracted with the same
    cotangent: FP64 to 1e-12 and fp32c to 1e-4 of the scale sum |v| |J| per
    (cosmology, direction) (a cotangent of random signs cancels, so the scale
    is that of the summed terms); the forward form's C_ell (fp32c) against
    the FP64 C_ell at 1e-5."""
    from jax_cosmo_gb300 import _lib
    from jax_cosmo_gb300.autodiff import vjp_device

    code = {0: 0, "smith2003": _lib.PK_SMITH2003, "linear": _lib.PK_LINEAR, "nowiggle": _lib.TF_NOWIGGLE}[physics]
    params, probes, ell, vbar, cl64, J64 = _vjp_case(MIXED, np.logspace(1, np.log10(3000), 37), code)
    ref = torch.einsum("bpl,bpld->bd", vbar, J64)
    scale = torch.einsum("bpl,bpld->bd", vbar.abs(), J64.abs())
    for prec, tol in (("fp64", 1e-12), ("fp32c", 1e-4)):
        g, cl = vjp_device(params, ell, probes, vbar, 512, prec, code, want_cl=True)
        err = float(((g - ref).abs() / scale).max())
        print(physics, prec, "vjp err / sum|v||J|: %.2e" % err)
        assert err < tol, (prec, err)
        assert float(((cl - cl64).abs() / cl64.abs()).max()) < (1e-12 if prec == "fp64" else 1e-5)


def test_vjp_gamma_direction_and_many_ell():
    """The gamma growth's derivative through gamma_dir, and an ell grid longer
    than one cotangent tile of the product kernel (16 tracers, 300 ell)."""
    from jax_cosmo_gb300 import _lib
    from jax_cosmo_gb300.autodiff import jacobian_device, vjp_device

    params, probes, ell, vbar, _, _ = _vjp_case(WL5, np.logspace(1, np.log10(3000), 29), _lib.GROWTH_GAMMA, 0.55, B=3)
    _, Jg = jacobian_device(params, ell, probes, 512, "fp64", _lib.GROWTH_GAMMA, gamma_dir=2)
    ref = torch.einsum("bpl,bpld->bd", vbar, Jg)
    scale = torch.einsum("bpl,bpld->bd", vbar.abs(), Jg.abs())
    g = vjp_device(params, ell, probes, vbar, 512, "fp32c", _lib.GROWTH_GAMMA, gamma_dir=2)
    assert float(((g - ref).abs() / scale).max()) < 1e-4
    spec16 = [("wl", [(1.0, 2.0, z0, 6.0, 10) for z0 in np.linspace(0.3, 1.6, 10)], {"sigma_e": 0.26}),
              ("nc", [(1.0, 2.0, z0, 6.0, 5) for z0 in np.linspace(0.4, 1.2, 6)], {"bias": 1.3})]
    params, probes, ell, vbar, _, J64 = _vjp_case(spec16, np.logspace(1, np.log10(5000), 300), B=2)
    ref = torch.einsum("bpl,bpld->bd", vbar, J64)
    scale = torch.einsum("bpl,bpld->bd", vbar.abs(), J64.abs())
    g = vjp_device(params, ell, probes, vbar, 512, "fp32c")
    assert float(((g - ref).abs() / scale).max()) < 1e-4


def test_vjp_reverse_lensing_with_ia_groups_and_single_plane():
    """The fp32c product applies the WeakLensing shear integral in reverse
    (its cotangents gathered on the chi table's nodes); the NLA intrinsic
    alignment, NumberCounts and single-plane terms keep forward tangents.
    Against the FP64 Jacobian contracted with a seeded cotangent: two lensing
    groups (different probe zmax), NLA with des_y1 and inverse-growth bias,
    multiplicative bias, an inverse-growth NumberCounts bin and a delta_nz
    bin; 1e-4 of the summed terms."""
    from jax_cosmo_gb300 import _geometry
    from jax_cosmo_gb300.autodiff import jacobian_device, vjp_device

    ell = _geometry.ell_host(np.geomspace(10, 3000, 23))
    pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
    pc = jc.redshift.smail_nz(1.0, 2.0, 0.8, gals_per_arcmin2=5, zmax=4.0)
    pd = jc.redshift.delta_nz(0.9)
    probes = [jc.probes.WeakLensing([pa, pc], ia_bias=[jc.bias.des_y1_ia_bias(1.2, 0.6, 0.62),
                                                       jc.bias.inverse_growth_linear_bias(0.7)],
                                    multiplicative_bias=[0.01, -0.02]),
              jc.probes.WeakLensing([pd]),
              jc.probes.NumberCounts([pa], jc.bias.inverse_growth_linear_bias(1.3))]
    rng = np.random.default_rng(17)
    rows = np.array([OTHER, FID, OTHER])
    rows[2] = rows[2] * (1.0 + 0.03 * rng.uniform(-1, 1, 8))
    params = torch.as_tensor(rows, device="cuda").contiguous()
    _, J64 = jacobian_device(params, ell, probes, 256, "fp64")
    n_cls = J64.shape[1]
    vbar = torch.as_tensor(rng.standard_normal((3, n_cls, len(ell))), device="cuda")
    ref = torch.einsum("bpl,bpld->bd", vbar, J64)
    scale = torch.einsum("bpl,bpld->bd", vbar.abs(), J64.abs())
    g = vjp_device(params, ell, probes, vbar, 256, "fp32c")
    err = float(((g - ref).abs() / scale).max())
    print("reverse lensing vjp err / sum|v||J|: %.2e" % err)
    assert err < 1e-4, err


def test_vjp_uniform_reverse_lensing_lanes_over_cosmologies():
    """A uniform fp32c batch with one lensing group and no single-plane bin
    takes the shear integral's values and cotangents with lanes over
    cosmologies (the chi table's segments split among the warps).  37
    cosmologies (a partial group of 32 lanes), 3 WeakLensing bins with NLA
    and multiplicative bias next to an inverse-growth NumberCounts bin:
    against the FP64 Jacobian contracted with the cotangent at 1e-4 of the
    summed terms, and one cosmology alone equal bit for bit to its row of the
    batch."""
    from jax_cosmo_gb300 import _geometry
    from jax_cosmo_gb300.autodiff import jacobian_device, vjp_device

    ell = _geometry.ell_host(np.geomspace(10, 3000, 19))
    nzs = [jc.redshift.smail_nz(1.0, 2.0, z0, gals_per_arcmin2=8, zmax=5.0) for z0 in (0.4, 0.8, 1.2)]
    probes = [jc.probes.WeakLensing(nzs, ia_bias=jc.bias.des_y1_ia_bias(1.1, 0.5, 0.62),
                                    multiplicative_bias=[0.01, -0.01, 0.02]),
              jc.probes.NumberCounts([nzs[1]], jc.bias.inverse_growth_linear_bias(1.4))]
    rng = np.random.default_rng(29)
    B = 37
    rows = np.array([FID] * B) * (1.0 + 0.05 * rng.uniform(-1, 1, (B, 8)))
    rows[:, 5] = 0.0
    rows[:, 7] = 0.03 * rng.uniform(-1, 1, B)
    params = torch.as_tensor(rows, device="cuda").contiguous()
    _, J64 = jacobian_device(params, ell, probes, 256, "fp64")
    vbar = torch.as_tensor(rng.standard_normal((B,) + tuple(J64.shape[1:3])), device="cuda")
    ref = torch.einsum("bpl,bpld->bd", vbar, J64)
    scale = torch.einsum("bpl,bpld->bd", vbar.abs(), J64.abs())
    g, cl = vjp_device(params, ell, probes, vbar, 256, "fp32c", want_cl=True)
    err = float(((g - ref).abs() / scale).max())
    print("uniform reverse lensing vjp err / sum|v||J|: %.2e" % err)
    assert err < 1e-4, err
    k = 33
    g1, cl1 = vjp_device(params[k:k + 1].contiguous(), ell, probes, vbar[k:k + 1].contiguous(), 256, "fp32c",
                         want_cl=True)
    assert torch.equal(g1[0], g[k])
    assert torch.equal(cl1[0], cl[k])


def test_vjp_large_batch_matches_small_batches_bit_for_bit():
    """At 640 cosmologies the product kernel runs all chunks of a cosmology
    in one CTA (C_ell summed in shared memory, chunk order); at 160 per call
    the chunks spread over CTAs (C_ell summed by the last chunk's CTA).  The
    same sums in the same order: C_ell and the gradient equal bit for bit
    (both sizes above the small-batch scalar kernel's 128)."""
    from jax_cosmo_gb300.autodiff import vjp_device

    rng = np.random.default_rng(41)
    B = 640
    rows = np.array([FID] * B) * (1.0 + 0.05 * rng.uniform(-1, 1, (B, 8)))
    rows[:, 5] = 0.0
    rows[:, 7] = 0.03 * rng.uniform(-1, 1, B)
    params = torch.as_tensor(rows, device="cuda").contiguous()
    probes = jc_probes(WL5)
    ell = np.geomspace(20, 3000, 40)
    n_cls = 15
    vbar = torch.as_tensor(rng.standard_normal((B, n_cls, len(ell))), device="cuda")
    g, cl = vjp_device(params, ell, probes, vbar, 256, "fp32c", want_cl=True)
    for i in range(0, B, 160):
        gi, cli = vjp_device(params[i:i + 160].contiguous(), ell, probes, vbar[i:i + 160].contiguous(), 256,
                             "fp32c", want_cl=True)
        assert torch.equal(gi, g[i:i + 160])
        assert torch.equal(cli, cl[i:i + 160])
