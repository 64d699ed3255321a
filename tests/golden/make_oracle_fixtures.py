"""Oracle outputs at the benchmark configurations, for the accuracy fields of
``bench.py`` (which may not run the oracle itself on the GPU host).

Usage (CPU only, about a minute)::

    python tests/golden/make_oracle_fixtures.py

Writes, from the float64 oracle (``oracle/jc_oracle.py``, itself pinned to the
unmodified reference by ``tests/test_oracle_golden.py``):

c2_oracle.npz  10 tracers (5 WeakLensing + 5 NumberCounts with constant bias
               1.2, smail_nz a=1, b=2, z0 = linspace(0.3, 1.5, 5)), 55 spectra
               x 200 log-spaced ell in [10, 5000], N = 512, fiducial cosmology:
               ``cl`` [55, 200].
c4_oracle.npz  5 WeakLensing bins x 50 log-spaced ell in [10, 3000], N = 512,
               fiducial cosmology: ``data`` = mean + L z (L the Cholesky factor
               of the dense covariance with noise, f_sky = 0.25; z standard
               normal from numpy seed 11), the log-likelihood ``loglike`` of
               gaussian_cl_covariance_and_mean + gaussian_log_likelihood (mean
               and covariance both at the cosmology), its gradient ``grad`` [8]
               and Hessian ``hess`` [8, 8] over the 8 Cosmology leaves by
               torch autograd, and the Gauss-Newton Fisher ``fisher_gn`` [8, 8]
               = J^T C^-1 J.

The tests compare the GPU path with these files and with the live oracle.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import jc_oracle as O  # noqa: E402

FID = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]
Z0 = np.linspace(0.3, 1.5, 5)


def c2_probes():
    nz = [O.Smail(1.0, 2.0, float(z), 10.0, 10.0) for z in Z0]
    return [O.Probe("wl", nz, sigma_e=0.26), O.Probe("nc", nz, bias=1.2)]


def c4_probes():
    nz = [O.Smail(1.0, 2.0, float(z), 10.0, 10.0) for z in Z0]
    return [O.Probe("wl", nz, sigma_e=0.26)]


def c4_ell():
    return np.logspace(1, np.log10(3000.0), 50)


def c4_loglike(v, data, ell, probes):
    mu, cov = O.gaussian_cl_covariance_and_mean(O.Cosmo.from_vector(v), ell, probes, sparse=True)
    return O.gaussian_log_likelihood(data, mu, cov)


def main():
    torch.set_num_threads(os.cpu_count() or 1)
    ell2 = np.logspace(1, np.log10(5000.0), 200)
    cl2 = O.angular_cl(O.Cosmo.from_vector(FID), ell2, c2_probes(), n_limber=512)
    np.savez_compressed(os.path.join(HERE, "c2_oracle.npz"), cl=cl2.numpy(), ell=ell2, fid=np.array(FID))

    ell4, p4 = c4_ell(), c4_probes()
    mu, cov = O.gaussian_cl_covariance_and_mean(O.Cosmo.from_vector(FID), ell4, p4, sparse=False)
    z = np.random.default_rng(11).standard_normal(mu.numel())
    data = (mu + torch.linalg.cholesky(cov) @ torch.as_tensor(z)).detach()
    v = torch.tensor(FID, dtype=torch.float64, requires_grad=True)
    ll = c4_loglike(v, data, ell4, p4)
    (g,) = torch.autograd.grad(ll, v)
    H = torch.autograd.functional.hessian(lambda x: c4_loglike(x, data, ell4, p4), torch.tensor(FID, dtype=torch.float64))

    def f(x):
        return O.angular_cl(O.Cosmo.from_vector(x), ell4, p4, n_limber=512)

    J = torch.autograd.functional.jacobian(f, torch.tensor(FID, dtype=torch.float64), strategy="forward-mode",
                                           vectorize=True)
    cl4 = f(torch.tensor(FID, dtype=torch.float64))
    cov_s = O.gaussian_cl_covariance(ell4, 5, cl4, O.noise_cl(ell4, p4), 0.25, sparse=True)
    Jl = J.permute(1, 0, 2)
    F = torch.einsum("lcp,lcq->pq", Jl, torch.linalg.solve(cov_s.permute(2, 0, 1), Jl))
    np.savez_compressed(os.path.join(HERE, "c4_oracle.npz"), data=data.numpy(), loglike=float(ll),
                        grad=g.numpy(), hess=H.numpy(), fisher_gn=F.numpy(), ell=ell4, fid=np.array(FID))
    print("c2: cl", tuple(cl2.shape), " c4: loglike", float(ll), "grad", g.numpy())


if __name__ == "__main__":
    main()
