"""GPU parity at the exact sizes of the benchmark set's single-cosmology
configurations (the batched and serving configurations are the bench's).

* 10 tracers (5 WeakLensing + 5 NumberCounts, constant bias 1.2, smail_nz a=1,
  b=2, z0 = linspace(0.3, 1.5, 5) for both), 55 spectra x 200 log-spaced ell in
  [10, 5000], N = 512: FP64 against the float64 oracle (1e-9 relative), and the
  compensated form's per-spectrum maximum relative error against FP64
  (bound 1e-4); the Gaussian covariance (f_sky = 0.25) against the oracle.
* 5 WeakLensing bins x 50 ell in [10, 3000]: the log-likelihood gradient with
  respect to (Omega_c, Omega_b, h, n_s, sigma8, w0, wa) at the fiducial, data =
  fiducial C_ell + seeded noise from its own covariance, against the oracle
  differentiated by torch autograd (1e-7 of the largest component) and central
  finite differences; the 7 x 7 Fisher matrix J^T C^-1 J against the oracle's
  (1e-7).  The reference's halofit root find interpolates log R linearly
  between sigma^2(R) table nodes (power.py:112-115), so the likelihood has
  kinks where a Limber node's root crosses a table node; central differences
  with step 1e-4 relative straddle some of them and differ from the local
  derivative by up to ~2% (the oracle shows the same: sigma8 1451.2 at 1e-4
  vs 1420.09 at 1e-5 and by autograd).  The test checks FD at 1e-5 relative
  (1e-5 absolute for the zero-valued w_a) to 1e-4 of the largest component,
  and at 1e-4 relative to 5e-2.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from oracle import jc_oracle as O  # noqa: E402

NAMES = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
FID = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]
SEL = [0, 1, 2, 3, 4, 6, 7]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)


def cosmo_of(row, grad=False):
    return jc.Cosmology(**{n: (torch.tensor(float(v), dtype=torch.float64, requires_grad=True) if grad else float(v))
                           for n, v in zip(NAMES, row)})


BOX = {"Omega_c": (0.20, 0.35), "Omega_b": (0.04, 0.06), "h": (0.60, 0.80), "n_s": (0.90, 1.00),
       "sigma8": (0.60, 1.00), "w0": (-1.3, -0.7)}


def box_rows(n, seed):
    """n cosmologies from the batched workload's seeded box (wa = Omega_k = 0),
    then the four corners in (w0, sigma8) with the other parameters at the box
    centre."""
    rng = np.random.default_rng(seed)
    rows = np.zeros((n + 4, 8))
    for i, name in enumerate(NAMES):
        if name in BOX:
            lo, hi = BOX[name]
            rows[:n, i] = rng.uniform(lo, hi, n)
            rows[n:, i] = 0.5 * (lo + hi)
    for k, (w0, s8) in enumerate(((-1.3, 0.6), (-1.3, 1.0), (-0.7, 0.6), (-0.7, 1.0))):
        rows[n + k, NAMES.index("w0")] = w0
        rows[n + k, NAMES.index("sigma8")] = s8
    return rows


def test_batched_workload_shape_vs_oracle():
    """The batched configuration's exact shape (5 WeakLensing smail bins, z0 =
    linspace(0.3, 1.5, 5), 100 log-spaced ell in [20, 3000], N = 512) on 16
    seeded box cosmologies and the 4 (w0, sigma8) box corners, in one batched
    call per precision: FP64 <= 1e-9 and fp32c <= 1e-4 relative against the
    float64 oracle, every C_ell."""
    rows = box_rows(16, 20261204)
    ell = np.logspace(np.log10(20.0), np.log10(3000.0), 100)
    probes, oprobes = _wl5()
    batch = jc.Cosmology(*[torch.tensor(rows[:, i], dtype=torch.float64) for i in range(8)])
    cl64 = jc.cl.angular_cl(batch, ell, probes).cpu()
    cl32 = jc.cl.angular_cl(batch, ell, probes, precision="fp32c").cpu()
    assert cl64.shape == (20, 15, 100)
    err64, err32 = [], []
    for b, row in enumerate(rows):
        ref = O.angular_cl(O.Cosmo.from_vector(row), ell, oprobes, n_limber=512)
        err64.append(float(((cl64[b] - ref) / ref).abs().max()))
        err32.append(float(((cl32[b] - ref) / ref).abs().max()))
    print("batched shape: max rel err per cosmology, fp64", ["%.1e" % e for e in err64])
    print("batched shape: max rel err per cosmology, fp32c", ["%.1e" % e for e in err32])
    assert max(err64) < 1e-9, err64
    assert max(err32) < 1e-4, err32


def test_ten_tracers_against_the_stored_oracle_spectra():
    """Config-2 spectra (10 tracers x 200 ell) against the oracle's stored
    output (tests/golden/c2_oracle.npz, the file the benchmark's accuracy
    fields use): FP64 1e-9 and fp32c 1e-4 per spectrum."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "c2_oracle.npz"))
    ell = d["ell"]
    z0 = np.linspace(0.3, 1.5, 5)
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z), gals_per_arcmin2=10.0) for z in z0]
    probes = [jc.probes.WeakLensing(nz, sigma_e=0.26), jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(1.2))]
    ref = torch.as_tensor(d["cl"])
    for prec, tol in (("fp64", 1e-9), ("fp32c", 1e-4)):
        cl = jc.cl.angular_cl(cosmo_of(FID), ell, probes, precision=prec).cpu()
        per = ((cl - ref) / ref).abs().amax(dim=1)
        print(prec, "per-spectrum max rel err vs oracle: max %.2e median %.2e" % (float(per.max()),
                                                                                 float(per.median())))
        assert float(per.max()) < tol, per


def test_ten_tracers_200_ell():
    z0 = np.linspace(0.3, 1.5, 5)
    ell = np.logspace(1, np.log10(5000), 200)
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z), gals_per_arcmin2=10.0) for z in z0]
    probes = [jc.probes.WeakLensing(nz, sigma_e=0.26), jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(1.2))]
    onz = [O.Smail(1.0, 2.0, float(z), 10.0, 10.0) for z in z0]
    oprobes = [O.Probe("wl", onz, sigma_e=0.26), O.Probe("nc", onz, bias=1.2)]
    c = cosmo_of(FID)
    cl64 = jc.cl.angular_cl(c, ell, probes)
    cl32 = jc.cl.angular_cl(c, ell, probes, precision="fp32c")
    assert cl64.shape == (55, 200)
    ref = O.angular_cl(O.Cosmo.from_vector(FID), ell, oprobes, n_limber=512)
    assert float(((cl64.cpu() - ref) / ref).abs().max()) < 1e-9
    per_spectrum = ((cl32 - cl64) / cl64).abs().amax(dim=1)
    assert float(per_spectrum.max()) < 1e-4, per_spectrum
    mu, cov = jc.cl.gaussian_cl_covariance_and_mean(c, ell, probes, sparse=True)
    mu_o, cov_o = O.gaussian_cl_covariance_and_mean(O.Cosmo.from_vector(FID), ell, oprobes, sparse=True)
    assert float(((mu.cpu() - mu_o) / mu_o).abs().max()) < 1e-9
    nz_mask = cov_o != 0
    assert float(((cov.cpu()[nz_mask] - cov_o[nz_mask]) / cov_o[nz_mask]).abs().max()) < 1e-9


def _wl5():
    z0 = np.linspace(0.3, 1.5, 5)
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z), gals_per_arcmin2=10.0) for z in z0]
    onz = [O.Smail(1.0, 2.0, float(z), 10.0, 10.0) for z in z0]
    return [jc.probes.WeakLensing(nz, sigma_e=0.26)], [O.Probe("wl", onz, sigma_e=0.26)]


def test_wl5_50ell_gradient_and_fisher():
    ell = np.logspace(1, np.log10(3000), 50)
    probes, oprobes = _wl5()
    mu0, cov0 = jc.cl.gaussian_cl_covariance_and_mean(cosmo_of(FID), ell, probes, sparse=False)
    gen = torch.Generator().manual_seed(11)
    z = torch.randn(mu0.numel(), generator=gen, dtype=torch.float64).to(mu0.device)
    data = (mu0 + torch.linalg.cholesky(cov0) @ z).detach()

    def loglike(row, grad):
        c = cosmo_of(row, grad)
        mu, cov = jc.cl.gaussian_cl_covariance_and_mean(c, ell, probes, sparse=True)
        return c, jc.likelihood.gaussian_log_likelihood(data, mu, cov)

    c, ll = loglike(FID, True)
    ll.backward()
    g = np.array([float(getattr(c, n).grad) for n in NAMES])
    # oracle autograd
    v = torch.tensor(FID, dtype=torch.float64, requires_grad=True)
    mu_o, cov_o = O.gaussian_cl_covariance_and_mean(O.Cosmo.from_vector(v), ell, oprobes, sparse=True)
    ll_o = O.gaussian_log_likelihood(data.cpu(), mu_o, cov_o)
    ll_o.backward()
    go = v.grad.numpy()
    assert abs(float(ll.detach()) - float(ll_o.detach())) <= 1e-9 * abs(float(ll_o.detach()))
    assert np.max(np.abs(g[SEL] - go[SEL])) / np.max(np.abs(go[SEL])) < 1e-7
    # central finite differences of the FP64 log-likelihood
    for rel, tol in ((1e-5, 1e-4), (1e-4, 5e-2)):
        fd = np.zeros(8)
        for i in SEL:
            h = rel * abs(FID[i]) if FID[i] != 0 else rel
            up, dn = list(FID), list(FID)
            up[i] += h
            dn[i] -= h
            fd[i] = (float(loglike(up, False)[1]) - float(loglike(dn, False)[1])) / (2 * h)
        assert np.max(np.abs(g[SEL] - fd[SEL])) / np.max(np.abs(fd[SEL])) < tol, (rel, g, fd)
    # Fisher J^T C^-1 J at the fiducial vs the oracle's (forward-mode Jacobian)
    F = jc.autodiff.fisher_matrix(cosmo_of(FID), ell, probes).cpu().numpy()

    def f(vec):
        return O.angular_cl(O.Cosmo.from_vector(vec), ell, oprobes, n_limber=512)

    J = torch.autograd.functional.jacobian(f, torch.tensor(FID, dtype=torch.float64), strategy="forward-mode",
                                           vectorize=True)[..., SEL]
    cl_o = f(torch.tensor(FID, dtype=torch.float64))
    cov_s = O.gaussian_cl_covariance(ell, 5, cl_o, O.noise_cl(ell, oprobes), 0.25, sparse=True)
    Jl = J.permute(1, 0, 2)
    F_o = torch.einsum("lcp,lcq->pq", Jl, torch.linalg.solve(cov_s.permute(2, 0, 1), Jl)).numpy()
    assert F.shape == (7, 7)
    assert np.max(np.abs(F - F_o)) / np.max(np.abs(F_o)) < 1e-7


def test_wl5_50ell_hessian_vs_oracle():
    """-jax.hessian(likelihood) of the README (README.md:14-27) at the
    gradient configuration (5 WL x 50 ell in [10, 3000], fiducial, stored
    noisy data; mean and covariance both at the cosmology): the 8 x 8 Hessian
    of loglike_hessian against torch.autograd.functional.hessian of the
    float64 oracle (tests/golden/c4_oracle.npz), 1e-6 of the largest entry
    and 1e-5 of each diagonal entry; its gradient against the oracle's
    autograd (1e-8); and central differences of the GPU FP64 gradient at
    step 1e-5 relative, taken on the same root-find branch, against the
    Hessian (1e-5)."""
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "c4_oracle.npz"))
    ell = d["ell"]
    probes, _ = _wl5()
    data = torch.as_tensor(d["data"])
    H, g, ll = jc.autodiff.loglike_hessian(cosmo_of(FID), ell, probes, data)
    H, g = H.numpy(), g.numpy()
    Ho, go = d["hess"], d["grad"]
    scale = np.max(np.abs(Ho))
    err = np.max(np.abs(H - Ho)) / scale
    derr = np.max(np.abs(np.diag(H) - np.diag(Ho)) / np.abs(np.diag(Ho)))
    print("hessian vs oracle: max err / max |H| %.2e, diagonal rel err %.2e" % (err, derr))
    assert abs(ll - float(d["loglike"])) <= 1e-9 * abs(float(d["loglike"]))
    assert np.max(np.abs(g - go)) / np.max(np.abs(go)) < 1e-8
    assert err < 1e-6, (H, Ho)
    assert derr < 1e-5
    # the same Hessian from central differences of exact gradients at 1e-5
    # relative on the base point's branch (no Richardson step)
    H5, _, _ = jc.autodiff.loglike_hessian(cosmo_of(FID), ell, probes, data, rel_step=1e-5)
    assert np.max(np.abs(H5.numpy() - H)) / scale < 1e-5
