"""jax_cosmo_gb300: jax_cosmo's angular power spectrum path on GB300.

Same module layout and names as jax_cosmo for the accelerated path
(``angular_cl``, ``gaussian_cl_covariance_and_mean``, ``gaussian_log_likelihood``,
``Cosmology``, ``Planck15``, ``probes.WeakLensing`` / ``NumberCounts``,
``redshift.smail_nz``, ``bias.constant_linear_bias``), differentiable through
torch.autograd (``autodiff``: hand-written Jacobian/adjoint), computed by the CUDA
library ``libjcg.so`` (sm_103a) through its C ABI (include/jcg.h).
"""
__version__ = "0.1.0"

import jax_cosmo_gb300.angular_cl as cl
import jax_cosmo_gb300.autodiff as autodiff
import jax_cosmo_gb300.background as background
import jax_cosmo_gb300.bias as bias
import jax_cosmo_gb300.likelihood as likelihood
import jax_cosmo_gb300.power as power
import jax_cosmo_gb300.probes as probes
import jax_cosmo_gb300.redshift as redshift
import jax_cosmo_gb300.sparse as sparse
import jax_cosmo_gb300.transfer as transfer
from jax_cosmo_gb300.core import *  # noqa: F401,F403
from jax_cosmo_gb300.parameters import *  # noqa: F401,F403
