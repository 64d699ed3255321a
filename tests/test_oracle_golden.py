"""The oracle (oracle/jc_oracle.py) against fixtures from the unmodified reference.

The fixtures were produced by tests/golden/make_golden.py, which runs the
jax_cosmo source on a NumPy stand-in for jax in float64.  Tolerance: 1e-12
relative (observed agreement is ~1e-15; the slack covers libm differences).
"""
import numpy as np
import pytest
import torch

from oracle import jc_oracle as O

RTOL = 1e-12


def rel(a, b):
    a = np.asarray(a.detach() if isinstance(a, torch.Tensor) else a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_background_distances_and_growth_rate(golden):
    """transverse / angular diameter distances for Omega_k = 0, > 0, < 0,
    a_of_chi on the decreasing chi table, growth_rate (background.py:245-512)."""
    g = golden("background2")
    a, chi = torch.tensor(g["a_q"]), torch.tensor(g["chi_q"])
    for i, row in enumerate(g["cosmos"]):
        c = O.Cosmo.from_vector(row)
        assert rel(O.transverse_comoving_distance(c, a), g["transverse"][i]) < RTOL
        assert rel(O.angular_diameter_distance(c, a), g["d_a"][i]) < RTOL
        assert rel(O.a_of_chi(c, chi), g["a_of_chi"][i]) < RTOL
        assert rel(O.growth_rate(c, a), g["growth_rate"][i]) < RTOL


def test_background_tables_and_queries(golden):
    g = golden("background")
    a = torch.tensor(g["a_q"])
    for i, row in enumerate(g["cosmos"]):
        c = O.Cosmo.from_vector(row)
        assert rel(O.chi_table(c)[1][:-1], g["chitab"][i][:-1]) < RTOL
        assert g["chitab"][i][-1] == 0.0 and float(O.chi_table(c)[1][-1]) == 0.0
        assert rel(O.growth_table(c)[1], g["gtab"][i]) < RTOL
        chi = O.radial_comoving_distance(c, a).detach().numpy()
        pos = g["chi"][i] > 0
        assert rel(chi[pos], g["chi"][i][pos]) < RTOL
        assert np.all(np.abs(chi[~pos]) < 1e-9)
        assert rel(O.growth_factor(c, a), g["D"][i]) < RTOL
        assert rel(O.H(c, a), g["H"][i]) < RTOL
        assert rel(O.dchioverda(c, a), g["dchioverda"][i]) < RTOL


def test_power_and_halofit(golden):
    p = golden("power")
    k = torch.tensor(p["k"])
    for i, row in enumerate(p["cosmos"]):
        c = O.Cosmo.from_vector(row)
        assert rel(O.eisenstein_hu(c, k), p["T"][i]) < RTOL
        assert rel(O.sigmasqr(c), p["sigmasqr8"][i]) < RTOL
        kn, ne, C = O.halofit_parameters(c, torch.tensor(p["a_hf"]))
        assert rel(kn, p["k_nl"][i]) < RTOL
        assert rel(ne, p["n_eff"][i]) < RTOL
        assert rel(C, p["C"][i]) < 1e-11  # C = I1^2 + I2 has a cancellation
        for j, a in enumerate(p["a_list"]):
            assert rel(O.linear_matter_power(c, k, a), p["plin"][i][j]) < RTOL
            assert rel(O.halofit(c, k, torch.tensor([a])), p["pnl"][i][j]) < 1e-11
        pairs = O.halofit(c, torch.tensor(p["k_pairs"]), torch.tensor(p["a_pairs"]))
        assert rel(pairs, p["pnl_pairs"][i]) < 1e-11


def test_redshift_and_kernels(golden):
    t = golden("tracers")
    b = golden("background")
    z = torch.tensor(t["z"])
    for i, (a, bb, z0, zm) in enumerate(t["smail"]):
        s = O.Smail(a, bb, z0, zm)
        assert rel(s(z), t["nz"][i]) < RTOL
        assert rel(s.norm, t["nz_norm"][i]) < RTOL
    zk = torch.tensor(t["z_kernel"])
    for i, row in enumerate(b["cosmos"][:3]):
        c = O.Cosmo.from_vector(row)
        pz = [O.Smail(1, 2, 0.5, 4.0, 10), O.Smail(1, 2, 1.0, 4.0, 10)]
        assert rel(O.probe_kernel(c, O.Probe("wl", pz), zk, 100.0), t["wl_kernel"][i]) < RTOL
        nc = O.probe_kernel(c, O.Probe("nc", pz, bias=1.2), zk, 100.0)
        assert rel(nc, t["nc_kernel"][i]) < RTOL
    pz = [O.Smail(1, 2, 0.5, 4.0, 10), O.Smail(1, 2, 1.0, 4.0, 3)]
    assert rel(O.Probe("wl", pz, sigma_e=0.3).noise(), t["wl_noise"]) < RTOL
    assert rel(O.Probe("nc", pz).noise(), t["nc_noise"]) < RTOL


def ia_probes():
    """The intrinsic-alignment fixture's probes (make_golden.py, kind "ia")."""
    pa, pb, pc = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10), O.Smail(1, 2, 0.8, 4.0, 5)
    return [
        O.Probe("wl", [pa, pb], sigma_e=0.26, m=[0.01, -0.02], ia=[("desy1", 1.2, 0.6, 0.62), ("const", 0.8)]),
        O.Probe("wl", [pc], sigma_e=0.3, ia=("invg", 0.7)),
        O.Probe("nc", [pa, pc], bias=[("invg", 1.3), ("const", 1.1)]),
    ]


def nz_probes(g):
    """The n(z) fixture's probes (make_golden.py, kind "nz")."""
    kde = O.Kde(g["zcat"], g["w"], 0.1, zmax=4.0, gals_per_arcmin2=10)
    fu = O.Fu(0.471, 5.1843, 0.7259, gals_per_arcmin2=30)
    shift = O.Shift(O.Smail(1.0, 2.0, 0.7, 10.0, 10), 0.05)
    return [O.Probe("wl", [fu, kde, shift], sigma_e=0.26), O.Probe("nc", [kde], bias=1.2)]


def delta_probes():
    """The single-plane fixture's probes (make_golden.py, kind "delta")."""
    pa = O.Smail(1, 2, 0.5, 10.0, 10)
    return [O.Probe("wl", [pa, O.Delta(1.0, gals_per_arcmin2=5), O.Delta(0.4)], sigma_e=0.26,
                    m=[0.0, 0.01, -0.02]),
            O.Probe("nc", [pa], bias=1.2)]


@pytest.mark.parametrize("name", ["cl_wl2", "cl_mixed", "cl_ia", "cl_nz", "cl_delta"])
def test_angular_cl(golden, name):
    g = golden(name)
    for i, row in enumerate(g["cosmos"]):
        c = O.Cosmo.from_vector(row)
        if name == "cl_wl2":
            pz = [O.Smail(1, 2, 0.5, 4.0, 10), O.Smail(1, 2, 1.0, 4.0, 10)]
            P = [O.Probe("wl", pz, sigma_e=0.26)]
        elif name == "cl_ia":
            P = ia_probes()
        elif name == "cl_nz":
            P = nz_probes(g)
        elif name == "cl_delta":
            P = delta_probes()
        else:
            pz = [O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10)]
            P = [O.Probe("wl", pz, sigma_e=0.26), O.Probe("nc", pz, bias=1.2)]
        cl = O.angular_cl(c, g["ell"], P)
        assert cl.shape == g["cl"][i].shape
        assert rel(cl, g["cl"][i]) < 1e-11


def test_covariance_and_likelihood(golden):
    cv = golden("cov_like")
    c = O.planck15()
    P = [O.Probe("nc", [O.Smail(1, 2, 1.0), O.Smail(1, 2, 0.5)], bias=1.0)]
    mu, cov_sp = O.gaussian_cl_covariance_and_mean(c, cv["nc_ell"], P, sparse=True)
    _, cov_d = O.gaussian_cl_covariance_and_mean(c, cv["nc_ell"], P, sparse=False)
    assert rel(mu, cv["nc_mu"]) < RTOL
    assert rel(cov_sp, cv["nc_cov_sparse"]) < 1e-11
    nz = cv["nc_cov_dense"] != 0
    assert np.array_equal(cov_d.numpy() != 0, nz)
    assert rel(cov_d.numpy()[nz], cv["nc_cov_dense"][nz]) < 1e-11
    assert rel(O.noise_cl(cv["nc_ell"], P), cv["nc_cl_noise"]) < RTOL
    data, mu_t = torch.tensor(cv["nc_data"]), torch.tensor(cv["nc_mu"])
    for inc in (True, False):
        ll = O.gaussian_log_likelihood(data, mu_t, torch.tensor(cv["nc_cov_sparse"]), inc)
        assert rel(ll, cv[f"nc_ll_sparse_{inc}"]) < 1e-10
        for m in ("inverse", "cholesky"):
            ll = O.gaussian_log_likelihood(data, mu_t, torch.tensor(cv["nc_cov_dense"]), inc, m)
            assert rel(ll, cv[f"nc_ll_{m}_{inc}"]) < 1e-10
    sig, noi = torch.tensor(cv["fixed_signal"]), torch.tensor(cv["fixed_noise"])
    d = O.gaussian_cl_covariance(cv["fixed_ell"], 2, sig, noi, 0.3, sparse=False)
    s = O.gaussian_cl_covariance(cv["fixed_ell"], 2, sig, noi, 0.3, sparse=True)
    assert np.array_equal(d.numpy(), cv["fixed_cov_dense"])
    assert np.array_equal(s.numpy(), cv["fixed_cov_sparse"])
    assert np.array_equal(O.to_dense(s).numpy(), d.numpy())


def test_sparse_algebra(golden):
    sp = golden("sparse")
    S = torch.tensor(sp["sparse"])
    assert rel(O.sparse_inv(S), sp["inv"]) < 1e-12
    sign, ld = O.sparse_slogdet(S)
    assert float(sign) == float(sp["sign"])
    assert rel(ld, sp["logdet"]) < 1e-12
    assert np.array_equal(O.to_dense(S).numpy(), sp["dense"])
    assert rel(O.sparse_dot_vec(S, torch.tensor(sp["v"])), sp["dot_vec"]) < 1e-12
    # self-consistency with the dense matrix (tests/test_sparse.py pattern)
    dense = O.to_dense(S)
    assert rel(torch.linalg.slogdet(dense)[1], sp["logdet"]) < 1e-12


def test_interp_quirks():
    """Nearest-node + side rule of scipy/interpolate.py:34-59 on hand cases."""
    xp = torch.tensor([0.0, 1.0, 2.0, 4.0, 8.0], dtype=torch.float64)
    fp = torch.tensor([0.0, 10.0, 20.0, 30.0, 70.0], dtype=torch.float64)
    # below xp[1]: segment [1, 2] extrapolated (segment [0, 1] is never used)
    assert float(O.interp(torch.tensor([0.5], dtype=torch.float64), xp, fp)) == 5.0
    assert float(O.interp(torch.tensor([-1.0], dtype=torch.float64), xp, fp)) == -10.0
    # interior: plain linear interpolation on the bracketing segment
    assert float(O.interp(torch.tensor([3.0], dtype=torch.float64), xp, fp)) == 25.0
    # above xp[-2]: segment [n-2, n-1]
    assert float(O.interp(torch.tensor([10.0], dtype=torch.float64), xp, fp)) == 90.0
    # decreasing table: side is always -1 below the last-but-one node
    xd = torch.tensor([8.0, 4.0, 2.0, 1.0, 0.0], dtype=torch.float64)
    v = float(O.interp(torch.tensor([2.2], dtype=torch.float64), xd, fp))
    assert v == pytest.approx(10.0 + (2.2 - 4.0) * (20.0 - 10.0) / (2.0 - 4.0))


PHYSICS_VARIANTS = (("eisenhu_osc", "smith2003"), ("eisenhu_osc", "linear"), ("eisenhu", "takahashi2012"))


def physics_probes():
    pa, pb = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10)
    return [O.Probe("wl", [pa, pb], sigma_e=0.26), O.Probe("nc", [pb], bias=1.2)]


def test_power_operator_points(golden):
    """Eisenstein_Hu type "eisenhu" (transfer.py:99-105), halofit smith2003
    (power.py:182-244) and linear_matter_power as nonlinear_fn."""
    p = golden("power2")
    k = torch.tensor(p["k"])
    for i, row in enumerate(p["cosmos"]):
        cn = O.Cosmo.from_vector(row)
        cn.transfer = "eisenhu"
        assert rel(O.eisenstein_hu(cn, k), p["T_nw"][i]) < RTOL
        assert rel(O.sigmasqr(cn), p["s8_nw"][i]) < RTOL
        c = O.Cosmo.from_vector(row)
        for j, a in enumerate(p["a_list"]):
            at = torch.tensor([a])
            assert rel(O.linear_matter_power(cn, k, a), p["plin_nw"][i][j]) < RTOL
            assert rel(O.halofit(cn, k, at), p["pnl_nw"][i][j]) < 1e-11
            assert rel(O.halofit(c, k, at, "smith2003"), p["pnl_smith"][i][j]) < 1e-11
            assert rel(O.linear_matter_power(c, k, a), p["pnl_lin"][i][j]) < RTOL
        pairs = O.halofit(c, torch.tensor(p["k_pairs"]), torch.tensor(p["a_pairs"]), "smith2003")
        assert rel(pairs, p["pnl_smith_pairs"][i]) < 1e-11


@pytest.mark.parametrize("variant", PHYSICS_VARIANTS, ids=["smith2003", "linear", "nowiggle"])
def test_angular_cl_operator_points(golden, variant):
    g = golden("cl_physics")
    tf, nl = variant
    for i, row in enumerate(g["cosmos"]):
        c = O.Cosmo.from_vector(row)
        c.transfer = tf
        cl = O.angular_cl(c, g["ell"], physics_probes(), nonlinear=nl)
        ref = g["cl_" + "_".join(variant)][i]
        assert cl.shape == ref.shape
        assert rel(cl, ref) < 1e-11


def test_gamma_growth(golden):
    """Cosmology(gamma=...): growth_factor, growth_rate (background.py:515-582) and
    angular_cl with that growth."""
    g = golden("gamma")
    a = torch.tensor(g["a_q"])
    for i, (row, gm) in enumerate(zip(g["cosmos"], g["gammas"])):
        c = O.Cosmo.from_vector(row)
        c.gamma = float(gm)
        assert rel(O.growth_factor(c, a), g["D"][i]) < RTOL
        assert rel(O.growth_rate(c, a), g["f"][i]) < RTOL
        cl = O.angular_cl(c, g["ell"], physics_probes())
        assert rel(cl, g["cl"][i]) < 1e-11
