"""The gradient oracle: torch autograd of oracle/jc_oracle.py (which stands in
for jax.grad of the reference, not installed here) against central finite
differences of the same oracle, for the 8 Cosmology parameters and, with the
gamma growth, gamma (background.py:515-582).  Small grids so that it runs in
seconds on the CPU."""
import numpy as np
import pytest
import torch

from oracle import jc_oracle as O

ROW = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]
ELL = np.array([60.0, 700.0])


def _probes():
    pa, pb = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10)
    return [O.Probe("wl", [pa], sigma_e=0.26), O.Probe("nc", [pb], bias=1.2)]


def _cl(v, gamma):
    c = O.Cosmo.from_vector(v[:8])
    if gamma:
        c.gamma = v[8]
    return O.angular_cl(c, ELL, _probes(), n_limber=64)


@pytest.mark.parametrize("gamma", [False, True], ids=["ode_growth", "gamma_growth"])
def test_autograd_matches_central_differences(gamma):
    v0 = torch.tensor(ROW + ([0.55] if gamma else []), dtype=torch.float64)
    J = torch.autograd.functional.jacobian(lambda v: _cl(v, gamma), v0, strategy="forward-mode", vectorize=True)
    for d in range(v0.numel()):
        h = 1e-5 * max(abs(float(v0[d])), 0.1)
        vp, vm = v0.clone(), v0.clone()
        vp[d] += h
        vm[d] -= h
        fd = (_cl(vp, gamma) - _cl(vm, gamma)) / (2 * h)
        scale = float(J[..., d].abs().max())
        err = float((J[..., d] - fd).abs().max()) / scale
        assert err < 1e-6, (d, err)
