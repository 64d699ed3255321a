"""CPU timing of the UNMODIFIED reference source on the batched workload: a
correctness baseline on one core, not a performance baseline.

The reference (jax_cosmo) runs here on ``tests/golden/jax_standin.py``, a
NumPy stand-in for the subset of ``jax`` it uses (JAX itself is not
installed), with one Python loop per ``vmap``.  This times ``angular_cl`` for a
slice of the batched workload: the first cosmology of the benchmark's seeded
box draw, 5 WeakLensing smail_nz bins (z0 = linspace(0.3, 1.5, 5), zmax 10,
sigma_e 0.26), the reference's own Limber grid (N = 512), and the first
``--n-ell`` of the benchmark's 100 ell in [20, 3000].  It needs a jax_cosmo
checkout (``--reference``), so it runs where one exists, not on the GPU host.

    python oracle/time_standin_reference.py --reference <path to a jax_cosmo checkout> [--n-ell 2]
"""
import argparse
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--n-ell", type=int, default=2)
    args = ap.parse_args()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import jax_standin

    jax_standin.install()
    sys.path.insert(0, args.reference)
    warnings.filterwarnings("ignore")
    import jax_cosmo as jc

    sys.path.insert(0, ROOT)
    import bench

    row = bench.draw_params(1)[0]
    names = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
    cosmo = jc.Cosmology(**{n: float(v) for n, v in zip(names, row)})
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z0), gals_per_arcmin2=10.0) for z0 in bench.Z0]
    probes = [jc.probes.WeakLensing(nz, sigma_e=0.26)]
    ell = bench.ell_grid()[: args.n_ell]
    t0 = time.perf_counter()
    cl = jc.angular_cl.angular_cl(cosmo, ell, probes)
    dt = time.perf_counter() - t0
    n = int(np.asarray(cl).size)
    print(f"unmodified reference on the NumPy stand-in, 1 core: {n} C_ell (15 spectra x {len(ell)} ell, "
          f"1 cosmology, N = 512) in {dt:.1f} s = {n / dt:.3f} C_ell/s")


if __name__ == "__main__":
    main()
