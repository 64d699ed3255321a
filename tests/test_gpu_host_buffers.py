"""jcg_angular_cl_host: angular_cl with the parameters and C_ell in host memory.

The entry point of a caller that holds no device arrays (a JAX host callback,
a CPU sampler) copies the parameters in and the C_ell out inside the call,
the copies of each range of cosmologies running on a second stream under the
Limber integral of the next range.  Its C_ell must equal those of
jcg_angular_cl on device buffers bit for bit (the same kernels on the same
inputs; the ranges only split the Limber launch), with pinned and with
pageable host memory, for one range and for several uneven ones.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from jax_cosmo_gb300.angular_cl import angular_cl_device, angular_cl_host  # noqa: E402


def _probes():
    nz = [jc.redshift.smail_nz(1.0, 2.0, z0, gals_per_arcmin2=10.0) for z0 in (0.5, 1.1)]
    return [jc.probes.WeakLensing(nz, sigma_e=0.26),
            jc.probes.NumberCounts(nz[:1], jc.bias.constant_linear_bias(1.2))]


def _params(seed, n):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 8))
    p[:, 0] = rng.uniform(0.20, 0.35, n)
    p[:, 1] = rng.uniform(0.04, 0.06, n)
    p[:, 2] = rng.uniform(0.60, 0.80, n)
    p[:, 3] = rng.uniform(0.90, 1.00, n)
    p[:, 4] = rng.uniform(0.60, 1.00, n)
    p[:, 6] = rng.uniform(-1.3, -0.7, n)
    return torch.as_tensor(p)


@pytest.mark.parametrize("n,precision,pinned", [(5, "fp64", False), (5, "fp32c", True),
                                                (4099, "fp32c", True), (2100, "fp32c", False)])
def test_host_buffers_equal_device_buffers(n, precision, pinned):
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)
    ell = np.logspace(1, np.log10(3000.0), 24)
    probes = _probes()
    p = _params(11 + n, n)
    ref = angular_cl_device(p.cuda(), ell, probes, precision).cpu()
    hp = p.pin_memory() if pinned else p.clone()
    out = torch.full(ref.shape, float("nan"), dtype=torch.float64)
    if pinned:
        out = out.pin_memory()
    got = angular_cl_host(hp, ell, probes, precision, out=out)
    torch.cuda.synchronize()
    assert got.data_ptr() == out.data_ptr()
    assert torch.isfinite(got).all()
    assert torch.equal(got, ref)
    # a second call into the same buffers (the copy stream and events reused)
    p2 = _params(12 + n, n)
    hp.copy_(p2)
    angular_cl_host(hp, ell, probes, precision, out=out)
    torch.cuda.synchronize()
    assert torch.equal(out, angular_cl_device(p2.cuda(), ell, probes, precision).cpu())
