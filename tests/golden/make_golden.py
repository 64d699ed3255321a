"""Generate the golden fixtures in this folder from the unmodified jax_cosmo source.

Usage (in a container where the jax_cosmo source tree is present; no GPU needed)::

    python tests/golden/make_golden.py --reference <path to a jax_cosmo checkout> [--procs 8]

The reference package runs on top of ``jax_standin`` (NumPy, float64).  Every
fixture is written as a compressed ``.npz``; the committed files are what the
oracle tests (``tests/test_oracle_golden.py``) check against.  The reference
source itself is never copied: only its outputs are stored.

Fixtures
--------
background.npz  chi / growth tables and point queries   (background.py:199-242, 443-488)
power.npz       Eisenstein-Hu T(k), sigma^2(8), linear and halofit P(k, a),
                halofit (k_nl, n_eff, C)                  (transfer.py, power.py)
tracers.npz     smail n(z), WL lensing kernel, NC density kernel, noise
                                                          (redshift.py, probes.py)
cl_wl2.npz      angular_cl, 2 WeakLensing bins (z0 = 0.5, 1.0; zmax = 4), 50 ell
cl_mixed.npz    angular_cl, 2 WeakLensing + 2 NumberCounts bins, 2 cosmologies
cl_ia.npz       angular_cl with NLA intrinsic alignment (des_y1, constant and
                inverse-growth IA biases, a list of biases per bin), two lensing
                groups, NumberCounts with inverse-growth and constant biases
cl_nz.npz       angular_cl with fu_nz, kde_nz (a seeded 200-galaxy catalog, stored
                with the fixture) and systematic_shift(smail_nz) bins
cl_delta.npz    angular_cl with single-plane delta_nz WeakLensing bins beside a
                smail bin, and a NumberCounts bin
power2.npz      the non-default operator points: Eisenstein_Hu type "eisenhu"
                (T, sigma^2(8), linear and halofit P), halofit smith2003 P(k, a),
                nonlinear_matter_power with linear_matter_power
                                                          (transfer.py:99-105, power.py:182-244)
cl_physics.npz  angular_cl, 2 WeakLensing + 1 NumberCounts bins, with
                nonlinear_fn = halofit(smith2003), linear_matter_power, and
                transfer_fn = Eisenstein_Hu(type="eisenhu")
gamma.npz       growth_factor / growth_rate and angular_cl (the cl_physics probes)
                of Cosmologies with a growth-rate index gamma (background.py:515-582)
background2.npz transverse / angular diameter distances (Omega_k = 0, > 0, < 0),
                a_of_chi, growth_rate                     (background.py:245-368, 401-512)
cov_like.npz    gaussian_cl_covariance_and_mean + gaussian_log_likelihood
sparse.npz      sparse.inv / slogdet / to_dense / dot on a random SPD block matrix
"""
import argparse
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# Cosmologies used across fixtures: rows of
# (Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa)
COSMOS = np.array(
    [
        [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0],  # Planck15
        [0.30, 0.05, 0.70, 0.96, 0.80, 0.0, -1.0, 0.0],  # reference test cosmology
        [0.25, 0.045, 0.72, 0.95, 0.78, 0.0, -0.9, 0.1],  # w0wa
        [0.35, 0.04, 0.60, 1.00, 1.00, 0.0, -1.3, 0.0],  # corner of the batch box
    ]
)

_REF = None


def _setup(reference):
    global _REF
    if _REF is not None:
        return _REF
    sys.path.insert(0, HERE)
    import jax_standin

    jax_standin.install()
    sys.path.insert(0, reference)
    warnings.filterwarnings("ignore")
    import jax_cosmo

    _REF = jax_cosmo
    return jax_cosmo


def _cosmo(jc, row, gamma=None):
    names = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
    return jc.Cosmology(**{n: float(v) for n, v in zip(names, row)}, gamma=gamma)


# gamma values of the gamma-growth fixture, one per cosmology in COSMOS[[0, 2]]
GAMMAS = (0.55, 0.62)


def make_gamma_background(jc):
    a_q = np.concatenate([np.logspace(-2.5, 0, 41), np.array([0.2, 0.5, 0.999, 1.0])])
    rows = COSMOS[[0, 2]]
    D, f = [], []
    for row, gm in zip(rows, GAMMAS):
        c = _cosmo(jc, row, gm)
        D.append(jc.background.growth_factor(c, a_q))
        f.append(jc.background.growth_rate(c, a_q))
    return {"cosmos": rows, "gammas": np.array(GAMMAS), "a_q": a_q, "D": np.array(D), "f": np.array(f)}


def make_background(jc):
    a_q = np.concatenate(
        [
            np.logspace(-3, 0, 97),
            np.linspace(0.05, 1.0, 64),
            np.array([1e-3, 0.2, 0.25, 0.5, 0.999, 1.0]),
        ]
    )
    out = {"cosmos": COSMOS, "a_q": a_q}
    chitab, gtab, chi, D, H, dchi = [], [], [], [], [], []
    for row in COSMOS:
        c = _cosmo(jc, row)
        chi.append(jc.background.radial_comoving_distance(c, a_q))
        D.append(jc.background.growth_factor(c, a_q))
        H.append(jc.background.H(c, a_q))
        dchi.append(jc.background.dchioverda(c, a_q))
        chitab.append(c._workspace["background.radial_comoving_distance"]["chi"])
        gtab.append(c._workspace["background.growth_factor"]["g"])
    out.update(
        chitab=np.array(chitab),
        gtab=np.array(gtab),
        chi=np.array(chi),
        D=np.array(D),
        H=np.array(H),
        dchioverda=np.array(dchi),
    )
    return out


# Omega_k = 0, open and closed universes for the curvature-dependent distances
COSMOS_K = np.array(
    [
        [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0],
        [0.30, 0.05, 0.70, 0.96, 0.80, 0.05, -1.0, 0.0],
        [0.25, 0.045, 0.72, 0.95, 0.78, -0.04, -0.9, 0.1],
    ]
)


def make_background2(jc):
    a_q = np.concatenate([np.logspace(-2.5, 0, 61), np.array([0.2, 0.5, 0.999, 1.0])])
    chi_q = np.concatenate([np.linspace(1.0, 6000.0, 41), np.array([0.5, 100.0, 2500.0])])
    out = {"cosmos": COSMOS_K, "a_q": a_q, "chi_q": chi_q}
    fk, da, aoc, f = [], [], [], []
    for row in COSMOS_K:
        c = _cosmo(jc, row)
        fk.append(jc.background.transverse_comoving_distance(c, a_q))
        da.append(jc.background.angular_diameter_distance(c, a_q))
        aoc.append(jc.background.a_of_chi(c, chi_q))
        f.append(jc.background.growth_rate(c, a_q))
    out.update(transverse=np.array(fk), d_a=np.array(da), a_of_chi=np.array(aoc), growth_rate=np.array(f))
    return out


def make_power(jc):
    k = np.logspace(-4, 4, 161)
    a_list = np.array([1.0, 0.7, 0.4, 0.2])
    a_hf = np.linspace(0.08, 1.0, 33)
    # elementwise (k, a) pairs, the way the Limber integrand calls halofit
    rng = np.random.default_rng(7)
    a_pairs = np.sort(rng.uniform(0.1, 1.0, 64))
    k_pairs = np.exp(rng.uniform(np.log(1e-3), np.log(50.0), 64))
    out = {"cosmos": COSMOS, "k": k, "a_list": a_list, "a_hf": a_hf}
    out["a_pairs"], out["k_pairs"] = a_pairs, k_pairs
    T, s8, plin, pnl, knl, neff, C, pnl_pairs = [], [], [], [], [], [], [], []
    for row in COSMOS:
        c = _cosmo(jc, row)
        T.append(jc.transfer.Eisenstein_Hu(c, k))
        s8.append(jc.power.sigmasqr(c, 8.0, jc.transfer.Eisenstein_Hu))
        plin.append([jc.power.linear_matter_power(c, k, a) for a in a_list])
        pnl.append([jc.power.nonlinear_matter_power(c, k, a) for a in a_list])
        kk, nn, cc = jc.power._halofit_parameters(c, a_hf, jc.transfer.Eisenstein_Hu)
        knl.append(kk)
        neff.append(nn)
        C.append(cc)
        pnl_pairs.append(jc.power.nonlinear_matter_power(c, k_pairs, a_pairs))
    out.update(
        T=np.array(T),
        sigmasqr8=np.array(s8),
        plin=np.array(plin),
        pnl=np.array(pnl),
        k_nl=np.array(knl),
        n_eff=np.array(neff),
        C=np.array(C),
        pnl_pairs=np.array(pnl_pairs),
    )
    return out


def make_power2(jc):
    import functools

    k = np.logspace(-4, 4, 97)
    a_list = np.array([1.0, 0.6, 0.25])
    rng = np.random.default_rng(9)
    a_pairs = np.sort(rng.uniform(0.1, 1.0, 48))
    k_pairs = np.exp(rng.uniform(np.log(1e-3), np.log(50.0), 48))
    nw = functools.partial(jc.transfer.Eisenstein_Hu, type="eisenhu")
    smith = functools.partial(jc.power.halofit, prescription="smith2003")
    out = {"cosmos": COSMOS, "k": k, "a_list": a_list, "a_pairs": a_pairs, "k_pairs": k_pairs}
    cols = {n: [] for n in ("T_nw", "s8_nw", "plin_nw", "pnl_nw", "pnl_smith", "pnl_smith_pairs", "pnl_lin")}
    for row in COSMOS:
        c = _cosmo(jc, row)
        cols["T_nw"].append(jc.transfer.Eisenstein_Hu(c, k, type="eisenhu"))
        cols["s8_nw"].append(jc.power.sigmasqr(c, 8.0, nw))
        c = _cosmo(jc, row)
        cols["plin_nw"].append([jc.power.linear_matter_power(c, k, a, transfer_fn=nw) for a in a_list])
        c = _cosmo(jc, row)
        cols["pnl_nw"].append([jc.power.nonlinear_matter_power(c, k, a, transfer_fn=nw) for a in a_list])
        c = _cosmo(jc, row)
        cols["pnl_smith"].append([jc.power.nonlinear_matter_power(c, k, a, nonlinear_fn=smith) for a in a_list])
        cols["pnl_smith_pairs"].append(jc.power.nonlinear_matter_power(c, k_pairs, a_pairs, nonlinear_fn=smith))
        cols["pnl_lin"].append(
            [jc.power.nonlinear_matter_power(c, k, a, nonlinear_fn=jc.power.linear_matter_power) for a in a_list]
        )
    out.update({n: np.array(v) for n, v in cols.items()})
    return out


# operator-point variants of the cl_physics fixture: (transfer type, nonlinear_fn)
PHYSICS_VARIANTS = (("eisenhu_osc", "smith2003"), ("eisenhu_osc", "linear"), ("eisenhu", "takahashi2012"))


def _fns(jc, variant):
    import functools

    tf_type, nl = variant
    tf = functools.partial(jc.transfer.Eisenstein_Hu, type=tf_type)
    if nl == "linear":
        return tf, jc.power.linear_matter_power
    return tf, functools.partial(jc.power.halofit, prescription=nl)


def make_tracers(jc):
    z = np.linspace(0.0, 5.0, 101)
    smail = np.array([[1.0, 2.0, 0.5, 4.0], [1.0, 2.0, 1.0, 4.0], [2.0, 1.5, 0.8, 10.0]])
    nz_vals, norms = [], []
    for a_, b_, z0, zmax in smail:
        nz = jc.redshift.smail_nz(a_, b_, z0, zmax=zmax)
        nz_vals.append(nz(z))
        norms.append(nz._norm)
    out = {"z": z, "smail": smail, "nz": np.array(nz_vals), "nz_norm": np.array(norms)}
    zk = np.linspace(0.01, 3.9, 40)
    out["z_kernel"] = zk
    wl, nc = [], []
    for row in COSMOS[:3]:
        c = _cosmo(jc, row)
        pz = [
            jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10, zmax=4.0),
            jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10, zmax=4.0),
        ]
        wl.append(jc.probes.WeakLensing(pz, sigma_e=0.26).kernel(c, zk, 100.0))
        nc.append(
            jc.probes.NumberCounts(pz, jc.bias.constant_linear_bias(1.2)).kernel(
                c, zk, 100.0
            )
        )
    out["wl_kernel"] = np.array(wl)
    out["nc_kernel"] = np.array(nc)
    pz = [
        jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10, zmax=4.0),
        jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=3, zmax=4.0),
    ]
    out["wl_noise"] = jc.probes.WeakLensing(pz, sigma_e=0.3).noise()
    out["nc_noise"] = jc.probes.NumberCounts(pz, jc.bias.constant_linear_bias(1.0)).noise()
    return out


# ---- angular_cl fixtures: one ell per worker process ----------------------------
def _probes(jc, kind):
    if kind == "wl2":
        pz = [
            jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10, zmax=4.0),
            jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10, zmax=4.0),
        ]
        return [jc.probes.WeakLensing(pz, sigma_e=0.26)]
    if kind == "mixed":
        pz = [
            jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10),
            jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10),
        ]
        return [
            jc.probes.WeakLensing(pz, sigma_e=0.26),
            jc.probes.NumberCounts(pz, jc.bias.constant_linear_bias(1.2)),
        ]
    if kind == "ia":
        pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
        pb = jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10)
        pc = jc.redshift.smail_nz(1.0, 2.0, 0.8, gals_per_arcmin2=5, zmax=4.0)
        return [
            jc.probes.WeakLensing(
                [pa, pb],
                ia_bias=[jc.bias.des_y1_ia_bias(1.2, 0.6, 0.62), jc.bias.constant_linear_bias(0.8)],
                multiplicative_bias=[0.01, -0.02],
                sigma_e=0.26,
            ),
            jc.probes.WeakLensing([pc], ia_bias=jc.bias.inverse_growth_linear_bias(0.7), sigma_e=0.3),
            jc.probes.NumberCounts(
                [pa, pc], [jc.bias.inverse_growth_linear_bias(1.3), jc.bias.constant_linear_bias(1.1)]
            ),
        ]
    if kind == "nz":
        zcat, w = nz_catalog()
        fu = jc.redshift.fu_nz(0.471, 5.1843, 0.7259, gals_per_arcmin2=30)
        kde = jc.redshift.kde_nz(zcat, w, bw=0.1, gals_per_arcmin2=10, zmax=4.0)
        shift = jc.redshift.systematic_shift(jc.redshift.smail_nz(1.0, 2.0, 0.7, gals_per_arcmin2=10), 0.05)
        return [
            jc.probes.WeakLensing([fu, kde, shift], sigma_e=0.26),
            jc.probes.NumberCounts([kde], jc.bias.constant_linear_bias(1.2)),
        ]
    if kind == "physics":
        pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
        pb = jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10)
        return [
            jc.probes.WeakLensing([pa, pb], sigma_e=0.26),
            jc.probes.NumberCounts([pb], jc.bias.constant_linear_bias(1.2)),
        ]
    if kind == "delta":
        pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
        return [
            jc.probes.WeakLensing(
                [pa, jc.redshift.delta_nz(1.0, gals_per_arcmin2=5), jc.redshift.delta_nz(0.4)],
                multiplicative_bias=[0.0, 0.01, -0.02], sigma_e=0.26,
            ),
            jc.probes.NumberCounts([pa], jc.bias.constant_linear_bias(1.2)),
        ]
    raise ValueError(kind)


def nz_catalog():
    """The seeded catalog of the kde_nz fixture: 200 redshifts and weights."""
    rng = np.random.default_rng(20261204)
    zcat = np.clip(rng.normal(0.8, 0.3, 200), 0.05, None)
    w = rng.uniform(0.5, 1.0, 200)
    return zcat, w


def _cl_worker(args):
    reference, kind, row, ell, variant = args
    jc = _setup(reference)
    if isinstance(variant, float):  # a gamma of the Cosmology, default operator points
        return jc.angular_cl.angular_cl(_cosmo(jc, row, variant), np.array([ell]), _probes(jc, kind))[:, 0]
    c = _cosmo(jc, row)
    if variant is None:
        return jc.angular_cl.angular_cl(c, np.array([ell]), _probes(jc, kind))[:, 0]
    tf, nl = _fns(jc, variant)
    return jc.angular_cl.angular_cl(c, np.array([ell]), _probes(jc, kind), tf, nl)[:, 0]


def make_cl(reference, pool, kind, cosmo_rows, ell, variant=None):
    jobs = [(reference, kind, row, float(l), variant) for row in cosmo_rows for l in ell]
    res = pool.map(_cl_worker, jobs)
    n_c, n_l = len(cosmo_rows), len(ell)
    cl = np.array(res).reshape(n_c, n_l, -1).transpose(0, 2, 1)
    return {"cosmos": np.array(cosmo_rows), "ell": np.asarray(ell), "cl": cl}


def make_cov_like(jc):
    out = {}
    # The reference's own likelihood test set-up (tests/test_likelihood.py:12-35)
    ell = np.logspace(1, 3, 5)
    nz1 = jc.redshift.smail_nz(1.0, 2.0, 1.0)
    nz2 = jc.redshift.smail_nz(1.0, 2.0, 0.5)
    P = [jc.probes.NumberCounts([nz1, nz2], jc.bias.constant_linear_bias(1.0))]
    c = jc.Planck15()
    mu, cov_sp = jc.angular_cl.gaussian_cl_covariance_and_mean(c, ell, P, sparse=True)
    mu_d, cov_d = jc.angular_cl.gaussian_cl_covariance_and_mean(c, ell, P, sparse=False)
    data = 1.1 * mu
    ll = {}
    for inc in (True, False):
        ll[f"sparse_{inc}"] = jc.likelihood.gaussian_log_likelihood(
            data, mu, cov_sp, include_logdet=inc
        )
        for m in ("inverse", "cholesky"):
            ll[f"{m}_{inc}"] = jc.likelihood.gaussian_log_likelihood(
                data, mu, cov_d, include_logdet=inc, inverse_method=m
            )
    out.update(
        nc_ell=ell,
        nc_mu=mu,
        nc_cov_sparse=cov_sp,
        nc_cov_dense=cov_d,
        nc_data=data,
        nc_cl_noise=jc.angular_cl.noise_cl(ell, P),
    )
    for k_, v in ll.items():
        out["nc_ll_" + k_] = np.asarray(v)
    # Covariance from fixed signal (tests/test_angular_cl.py:201-213 pattern)
    ell2 = np.logspace(1, 3, 25)
    sig = np.random.default_rng(3).uniform(0.5, 2.0, (3, 25))
    noi = np.random.default_rng(4).uniform(0.1, 0.3, (3, 25))
    out["fixed_ell"] = ell2
    out["fixed_signal"] = sig
    out["fixed_noise"] = noi
    out["fixed_cov_dense"] = jc.angular_cl.gaussian_cl_covariance(
        ell2, P, sig, noi, f_sky=0.3, sparse=False
    )
    out["fixed_cov_sparse"] = jc.angular_cl.gaussian_cl_covariance(
        ell2, P, sig, noi, f_sky=0.3, sparse=True
    )
    return out


def make_sparse(jc):
    rng = np.random.default_rng(11)
    n, nd = 4, 6
    # SPD per-diagonal blocks: A_l = B_l B_l^T + n I
    B = rng.normal(size=(nd, n, n))
    A = np.einsum("lij,lkj->lik", B, B) + n * np.eye(n)[None]
    sp = np.transpose(A, (1, 2, 0)).copy()  # (n, n, nd)
    v = rng.normal(size=n * nd)
    out = {"sparse": sp, "v": v}
    out["inv"] = jc.sparse.inv(sp)
    s, ld = jc.sparse.slogdet(sp)
    out["sign"], out["logdet"] = np.asarray(s), np.asarray(ld)
    out["dense"] = jc.sparse.to_dense(sp)
    out["dot_vec"] = jc.sparse.dot(sp, v)
    out["vec_dot"] = jc.sparse.dot(v, sp)
    out["bilinear"] = jc.sparse.dot(v.reshape(1, -1), sp, v.reshape(-1, 1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    jc = _setup(args.reference)
    only = set(args.only.split(",")) if args.only else None

    def want(name):
        return only is None or name in only

    def save(name, d):
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(f"wrote {name}.npz ({time.time() - t0:.1f}s)", flush=True)

    t0 = time.time()
    if want("background"):
        save("background", make_background(jc))
    if want("background2"):
        save("background2", make_background2(jc))
    if want("power"):
        save("power", make_power(jc))
    if want("power2"):
        save("power2", make_power2(jc))
    if want("tracers"):
        save("tracers", make_tracers(jc))
    if want("cov_like"):
        save("cov_like", make_cov_like(jc))
    if want("sparse"):
        save("sparse", make_sparse(jc))
    if any(want(n) for n in ("cl_wl2", "cl_mixed", "cl_ia", "cl_nz", "cl_delta", "cl_physics", "gamma")):
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(args.procs) as pool:
            if want("cl_wl2"):
                ell = np.logspace(1, np.log10(3000.0), 50)
                save("cl_wl2", make_cl(args.reference, pool, "wl2", COSMOS[:2], ell))
            if want("cl_mixed"):
                ell = np.logspace(1, np.log10(5000.0), 12)
                save(
                    "cl_mixed",
                    make_cl(args.reference, pool, "mixed", COSMOS[[0, 2]], ell),
                )
            if want("cl_ia"):
                ell = np.logspace(1, np.log10(5000.0), 12)
                save("cl_ia", make_cl(args.reference, pool, "ia", COSMOS[[0, 2]], ell))
            if want("cl_nz"):
                ell = np.logspace(1, np.log10(5000.0), 10)
                d = make_cl(args.reference, pool, "nz", COSMOS[[0, 2]], ell)
                d["zcat"], d["w"] = nz_catalog()
                save("cl_nz", d)
            if want("cl_delta"):
                ell = np.logspace(1, np.log10(5000.0), 10)
                save("cl_delta", make_cl(args.reference, pool, "delta", COSMOS[[0, 2]], ell))
            if want("gamma"):
                d = make_gamma_background(jc)
                ell = np.logspace(1, np.log10(5000.0), 10)
                cls = []
                for row, gm in zip(COSMOS[[0, 2]], GAMMAS):
                    cls.append(make_cl(args.reference, pool, "physics", [row], ell, gm)["cl"][0])
                d["ell"], d["cl"] = ell, np.array(cls)
                save("gamma", d)
            if want("cl_physics"):
                ell = np.logspace(1, np.log10(5000.0), 10)
                d = {}
                for v in PHYSICS_VARIANTS:
                    r = make_cl(args.reference, pool, "physics", COSMOS[[0, 2]], ell, v)
                    d["cl_" + "_".join(v)] = r.pop("cl")
                    d.update(r)
                save("cl_physics", d)


if __name__ == "__main__":
    main()
