"""GPU parity: libjcg (through the C ABI, via the Python API) against the golden
fixtures of the unmodified reference and against the float64 oracle.

Tolerances: FP64 path 1e-9 relative (libm vs CUDA transcendental rounding,
summation order); FP32C path 1e-4 relative per C_ell (the stated bound of the
compensated form).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import jax_cosmo_gb300 as jc  # noqa: E402
from oracle import jc_oracle as O  # noqa: E402

RT64 = 1e-9
RT32 = 1e-4

NAMES = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def cosmo_of(row):
    return jc.Cosmology(**{n: float(v) for n, v in zip(NAMES, row)})


def cosmo_batch(rows):
    rows = np.asarray(rows)
    return jc.Cosmology(**{n: torch.tensor(rows[:, i]) for i, n in enumerate(NAMES)})


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.set_device(0)


# ------------------------------------------------------------- background ---
def test_background_points_vs_golden(golden):
    g = golden("background")
    a = g["a_q"]
    for i, row in enumerate(g["cosmos"]):
        c = cosmo_of(row)
        chi = jc.background.radial_comoving_distance(c, a)
        pos = g["chi"][i] > 0
        assert rel(chi[torch.as_tensor(pos)], g["chi"][i][pos]) < RT64
        assert float(chi[torch.as_tensor(~pos)].abs().max()) < 1e-6
        assert rel(jc.background.growth_factor(c, a), g["D"][i]) < RT64
        assert rel(jc.background.H(c, a), g["H"][i]) < RT64
        assert rel(jc.background.dchioverda(c, a), g["dchioverda"][i]) < RT64


def test_background_distances_and_growth_rate_vs_golden(golden):
    """background.py:245-368, 401-512 on the device: curvature branches, the
    reference's interpolation of the decreasing chi table, the growth rate."""
    g = golden("background2")
    for i, row in enumerate(g["cosmos"]):
        c = cosmo_of(row)
        assert rel(jc.background.transverse_comoving_distance(c, g["a_q"]), g["transverse"][i]) < RT64
        assert rel(jc.background.angular_diameter_distance(c, g["a_q"]), g["d_a"][i]) < RT64
        assert rel(jc.background.a_of_chi(c, g["chi_q"]), g["a_of_chi"][i]) < RT64
        assert rel(jc.background.growth_rate(c, g["a_q"]), g["growth_rate"][i]) < RT64
    cb = cosmo_batch(g["cosmos"])
    fk = jc.background.transverse_comoving_distance(cb, g["a_q"])
    assert fk.shape == (len(g["cosmos"]), len(g["a_q"]))


def test_background_batched_matches_single(golden):
    g = golden("background")
    cb = cosmo_batch(g["cosmos"])
    chi = jc.background.radial_comoving_distance(cb, g["a_q"])
    assert chi.shape == (len(g["cosmos"]), len(g["a_q"]))
    for i, row in enumerate(g["cosmos"]):
        assert torch.equal(chi[i], jc.background.radial_comoving_distance(cosmo_of(row), g["a_q"]))


# ------------------------------------------------------------------ power ---
def test_power_points_vs_golden(golden):
    p = golden("power")
    k = p["k"]
    for i, row in enumerate(p["cosmos"]):
        c = cosmo_of(row)
        assert rel(jc.transfer.Eisenstein_Hu(c, k), p["T"][i]) < RT64
        for j, a in enumerate(p["a_list"]):
            assert rel(jc.power.linear_matter_power(c, k, a), p["plin"][i][j]) < RT64
            assert rel(jc.power.nonlinear_matter_power(c, k, a), p["pnl"][i][j]) < RT64
        kn, ne, C = jc.power.halofit_parameters(c, p["a_hf"])
        assert rel(kn, p["k_nl"][i]) < RT64
        assert rel(ne, p["n_eff"][i]) < RT64
        assert rel(C, p["C"][i]) < RT64
        assert rel(jc.power.nonlinear_matter_power(c, p["k_pairs"], p["a_pairs"]), p["pnl_pairs"][i]) < RT64


# ---------------------------------------------------------------- tracers ---
def test_probe_kernels_vs_golden(golden):
    t = golden("tracers")
    b = golden("background")
    zk = t["z_kernel"]
    for i, row in enumerate(b["cosmos"][:3]):
        c = cosmo_of(row)
        pz = [jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10, zmax=4.0),
              jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10, zmax=4.0)]
        wl = jc.probes.WeakLensing(pz, sigma_e=0.26).kernel(c, zk, 100.0)
        assert rel(wl, t["wl_kernel"][i]) < RT64
        nc = jc.probes.NumberCounts(pz, jc.bias.constant_linear_bias(1.2)).kernel(c, zk, 100.0)
        assert rel(nc, t["nc_kernel"][i]) < RT64


# ------------------------------------------------------------- angular_cl ---
def _wl2():
    pz = [jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10, zmax=4.0),
          jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10, zmax=4.0)]
    return [jc.probes.WeakLensing(pz, sigma_e=0.26)]


def _mixed():
    pz = [jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10),
          jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10)]
    return [jc.probes.WeakLensing(pz, sigma_e=0.26),
            jc.probes.NumberCounts(pz, jc.bias.constant_linear_bias(1.2))]


def _ia():
    """The intrinsic-alignment fixture's probes (tests/golden/make_golden.py, kind "ia")."""
    pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
    pb = jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10)
    pc = jc.redshift.smail_nz(1.0, 2.0, 0.8, gals_per_arcmin2=5, zmax=4.0)
    return [
        jc.probes.WeakLensing([pa, pb], ia_bias=[jc.bias.des_y1_ia_bias(1.2, 0.6, 0.62),
                                                 jc.bias.constant_linear_bias(0.8)],
                              multiplicative_bias=[0.01, -0.02], sigma_e=0.26),
        jc.probes.WeakLensing([pc], ia_bias=jc.bias.inverse_growth_linear_bias(0.7), sigma_e=0.3),
        jc.probes.NumberCounts([pa, pc], [jc.bias.inverse_growth_linear_bias(1.3), jc.bias.constant_linear_bias(1.1)]),
    ]


@pytest.mark.parametrize("name,probes", [("cl_wl2", _wl2), ("cl_mixed", _mixed), ("cl_ia", _ia)])
def test_angular_cl_vs_golden(golden, name, probes):
    g = golden(name)
    for i, row in enumerate(g["cosmos"]):
        cl = jc.cl.angular_cl(cosmo_of(row), g["ell"], probes())
        assert cl.shape == g["cl"][i].shape
        assert rel(cl, g["cl"][i]) < RT64
        cl32 = jc.cl.angular_cl(cosmo_of(row), g["ell"], probes(), precision="fp32c")
        assert rel(cl32, g["cl"][i]) < RT32


def _oracle_probes(spec):
    out = []
    for kind, bins, extra in spec:
        out.append(O.Probe(kind, [O.Smail(*b) for b in bins], **extra))
    return out


def _jc_probes(spec):
    out = []
    for kind, bins, extra in spec:
        nz = [jc.redshift.smail_nz(a, b, z0, gals_per_arcmin2=ng, zmax=zm) for a, b, z0, zm, ng in bins]
        if kind == "wl":
            out.append(jc.probes.WeakLensing(nz, sigma_e=extra.get("sigma_e", 0.26),
                                             multiplicative_bias=extra.get("m", 0.0)))
        else:
            out.append(jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(extra["bias"])))
    return out


def _oracle_spec(spec):
    res = []
    for kind, bins, extra in spec:
        e = dict(extra)
        if kind == "wl" and "m" in e:
            pass
        res.append((kind, bins, e))
    return res


C1_SPEC = [("wl", [(1.0, 2.0, 0.5, 4.0, 10), (1.0, 2.0, 1.0, 4.0, 10)], {"sigma_e": 0.26})]
C2_BINS = [(1.0, 2.0, z0, 10.0, 10) for z0 in np.linspace(0.3, 1.5, 5)]
C2_SPEC = [("wl", C2_BINS, {"sigma_e": 0.26}), ("nc", C2_BINS, {"bias": 1.2})]


@pytest.mark.parametrize(
    "spec,ell,n_limber",
    [
        (C1_SPEC, np.logspace(1, np.log10(3000), 50), 256),  # 2 WL bins, N = 256, zmax = 4
        (C2_SPEC, np.logspace(1, np.log10(5000), 24), 512),  # config 2 tracers, 55 spectra
        ([("wl", [(1.0, 2.0, 0.7, 3.0, 5)], {"sigma_e": 0.3, "m": 0.02}),
          ("nc", [(2.0, 1.5, 0.4, 2.5, 3), (1.0, 2.0, 0.9, 5.0, 4)], {"bias": 0.9})],
         np.array([2.0, 7.5, 33.0, 480.0, 2999.0]), 200),   # ragged zmax, m != 0, odd ell
        ([("wl", [(1.0, 2.0, 0.6, 3.0, 8)], {"sigma_e": 0.28}),
          ("wl", [(1.0, 2.0, 1.1, 6.0, 8), (1.0, 2.0, 0.4, 6.0, 6)], {"sigma_e": 0.25})],
         np.logspace(1, 3.5, 9), 128),   # two lensing groups (probe zmax 3 and 6)
    ],
)
def test_angular_cl_vs_oracle(spec, ell, n_limber):
    rows = [[0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0],
            [0.31, 0.045, 0.66, 0.98, 0.72, 0.0, -0.85, 0.15]]
    oracle_probes = []
    for kind, bins, extra in spec:
        e = {}
        if kind == "wl":
            e["sigma_e"] = extra.get("sigma_e", 0.26)
            e["m"] = extra.get("m", 0.0)
        else:
            e["bias"] = extra["bias"]
        oracle_probes.append(O.Probe(kind, [O.Smail(a, b, z0, zm, ng) for a, b, z0, zm, ng in bins], **e))
    cb = cosmo_batch(rows)
    cl = jc.cl.angular_cl(cb, ell, _jc_probes(spec), n_limber=n_limber)
    cl32 = jc.cl.angular_cl(cb, ell, _jc_probes(spec), n_limber=n_limber, precision="fp32c")
    for i, row in enumerate(rows):
        ref = O.angular_cl(O.Cosmo.from_vector(row), ell, oracle_probes, n_limber=n_limber)
        assert rel(cl[i], ref) < RT64
        assert rel(cl32[i], ref) < RT32
        # batch entry == single call, bit for bit
        single = jc.cl.angular_cl(cosmo_of(row), ell, _jc_probes(spec), n_limber=n_limber)
        assert torch.equal(single, cl[i])


def test_angular_cl_edge_cases():
    c = jc.Planck15()
    # one ell, one tracer
    p1 = [jc.probes.NumberCounts([jc.redshift.smail_nz(1.0, 2.0, 0.8)], jc.bias.constant_linear_bias(1.0))]
    cl = jc.cl.angular_cl(c, 100.0, p1)
    ref = O.angular_cl(O.planck15(), [100.0], [O.Probe("nc", [O.Smail(1.0, 2.0, 0.8)], bias=1.0)])
    assert cl.shape == (1, 1) and rel(cl, ref) < RT64
    with pytest.raises(ValueError):
        jc.cl.angular_cl(c, [10.0, 20.0], p1, n_limber=255)  # Simpson needs even N
    with pytest.raises(NotImplementedError):
        jc.cl.angular_cl(c, [10.0], p1, transfer_fn=lambda *a: None)
    # 16 tracers (136 spectra): the maximum request size
    nz = [jc.redshift.smail_nz(1.0, 2.0, z0) for z0 in np.linspace(0.3, 1.5, 8)]
    p16 = [jc.probes.WeakLensing(nz), jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(1.1))]
    ell = np.logspace(1, 3, 6)
    cl16 = jc.cl.angular_cl(c, ell, p16)
    o16 = [O.Probe("wl", [O.Smail(1.0, 2.0, z0) for z0 in np.linspace(0.3, 1.5, 8)]),
           O.Probe("nc", [O.Smail(1.0, 2.0, z0) for z0 in np.linspace(0.3, 1.5, 8)], bias=1.1)]
    ref16 = O.angular_cl(O.planck15(), ell, o16)
    assert cl16.shape == (136, 6) and rel(cl16, ref16) < RT64
    assert torch.isfinite(jc.cl.angular_cl(c, ell, p16, precision="fp32c")).all()


# ------------------------------------------------------ covariance / like ---
def test_covariance_and_likelihood_vs_golden(golden):
    cv = golden("cov_like")
    nz1 = jc.redshift.smail_nz(1.0, 2.0, 1.0)
    nz2 = jc.redshift.smail_nz(1.0, 2.0, 0.5)
    P = [jc.probes.NumberCounts([nz1, nz2], jc.bias.constant_linear_bias(1.0))]
    c = jc.Planck15()
    mu, cov_sp = jc.cl.gaussian_cl_covariance_and_mean(c, cv["nc_ell"], P, sparse=True)
    mu_d, cov_d = jc.cl.gaussian_cl_covariance_and_mean(c, cv["nc_ell"], P, sparse=False)
    assert rel(mu, cv["nc_mu"]) < RT64
    assert rel(cov_sp, cv["nc_cov_sparse"]) < RT64
    nzm = cv["nc_cov_dense"] != 0
    assert np.array_equal(cov_d.cpu().numpy() != 0, nzm)
    assert rel(cov_d.cpu().numpy()[nzm], cv["nc_cov_dense"][nzm]) < RT64
    assert rel(jc.cl.noise_cl(cv["nc_ell"], P), cv["nc_cl_noise"]) < 1e-14
    data = torch.as_tensor(cv["nc_data"])
    mu_g = torch.as_tensor(cv["nc_mu"])
    for inc in (True, False):
        ll = jc.likelihood.gaussian_log_likelihood(data, mu_g, torch.as_tensor(cv["nc_cov_sparse"]), inc)
        assert rel(ll, cv[f"nc_ll_sparse_{inc}"]) < 1e-10
        for m in ("inverse", "cholesky"):
            ll = jc.likelihood.gaussian_log_likelihood(data, mu_g, torch.as_tensor(cv["nc_cov_dense"]), inc, m)
            assert rel(ll, cv[f"nc_ll_{m}_{inc}"]) < 1e-10
    # fixed signal / noise (tests/test_angular_cl.py:201-213 pattern): exact
    sig, noi = cv["fixed_signal"], cv["fixed_noise"]
    d = jc.cl.gaussian_cl_covariance(cv["fixed_ell"], P, sig, noi, f_sky=0.3, sparse=False)
    s = jc.cl.gaussian_cl_covariance(cv["fixed_ell"], P, sig, noi, f_sky=0.3, sparse=True)
    assert np.array_equal(d.cpu().numpy(), cv["fixed_cov_dense"])
    assert np.array_equal(s.cpu().numpy(), cv["fixed_cov_sparse"])
    assert torch.equal(jc.sparse.to_dense(s), d)


def test_likelihood_unstructured_dense_and_batched():
    torch.manual_seed(0)
    N = 12
    A = torch.randn(N, N, dtype=torch.float64)
    C = A @ A.T + N * torch.eye(N, dtype=torch.float64)
    mu = torch.randn(N, dtype=torch.float64)
    data = torch.randn(N, dtype=torch.float64)
    ll = jc.likelihood.gaussian_log_likelihood(data, mu, C)
    ref = O.gaussian_log_likelihood(data, mu, C)
    assert rel(ll, ref) < 1e-11
    # batched sparse
    sp = torch.rand(3, 3, 5, dtype=torch.float64)
    sp = torch.einsum("ijl,kjl->ikl", sp, sp) + 3 * torch.eye(3, dtype=torch.float64)[:, :, None]
    spb = torch.stack([sp, 2 * sp])
    mub = torch.randn(2, 15, dtype=torch.float64)
    db = torch.randn(2, 15, dtype=torch.float64)
    llb = jc.likelihood.gaussian_log_likelihood(db, mub, spb)
    for i in range(2):
        assert rel(llb[i], O.gaussian_log_likelihood(db[i], mub[i], spb[i])) < 1e-11


# ----------------------------------------------------------------- sparse ---
def test_sparse_vs_golden(golden):
    sp = golden("sparse")
    S = torch.as_tensor(sp["sparse"])
    assert rel(jc.sparse.inv(S), sp["inv"]) < 1e-11
    sign, ld = jc.sparse.slogdet(S)
    assert float(sign) == float(sp["sign"]) and rel(ld, sp["logdet"]) < 1e-12
    assert np.array_equal(jc.sparse.to_dense(S).cpu().numpy(), sp["dense"])
    assert rel(jc.sparse.dot(S, sp["v"]), sp["dot_vec"]) < 1e-12
    assert rel(jc.sparse.dot(sp["v"], S), sp["vec_dot"]) < 1e-12
    assert rel(jc.sparse.dot(sp["v"].reshape(1, -1), S, sp["v"].reshape(-1, 1)), sp["bilinear"]) < 1e-12


def test_sparse_known_answers():
    """The integer known-answer cases of the reference's tests/test_sparse.py."""
    X = torch.tensor([[[1, 2, 3], [4, 5, 6], [-1, -2, -3]], [[1, 2, 3], [-4, -5, -6], [7, 8, 9]]],
                     dtype=torch.float64)
    D = jc.sparse.to_dense(X).cpu()
    assert D.shape == (6, 9)
    assert D[0, 3] == 4 and D[1, 4] == 5 and D[5, 8] == 9 and D[3, 3] == -4 and D[0, 1] == 0
    with pytest.raises(ValueError):
        jc.sparse.to_dense([1, 2, 3])
    Xi = torch.tensor([[[1.0, 1.0], [1.0, 1.0]], [[1.0, 1.0], [2.0, 2.0]]], dtype=torch.float64)
    ans = torch.tensor([[[2.0, 2.0], [-1.0, -1.0]], [[-1.0, -1.0], [1.0, 1.0]]], dtype=torch.float64)
    assert rel(jc.sparse.inv(Xi), ans) < 1e-14
    Xd = torch.tensor([[[1, 2, 3], [4, 5, 6], [-1, 7, -2]], [[1, 2, 3], [-4, -5, -6], [2, -3, 9]],
                       [[7, 8, 9], [5, -4, 6], [-3, -2, -1]]], dtype=torch.float64)
    assert float(-jc.sparse.det(-Xd)) == pytest.approx(float(jc.sparse.det(Xd)), rel=1e-12)
    assert float(jc.sparse.det(Xd)) == pytest.approx(float(np.linalg.det(jc.sparse.to_dense(Xd).cpu().numpy())), rel=1e-6)


def test_sparse_products_known_answers():
    """The product and bilinear-form cases of the reference's
    tests/test_sparse.py (test_dot, test_bilinear), every product in libjcg,
    against the dense products of to_dense."""
    X1 = torch.tensor([[[1.0, 2], [3, 4], [5, 6]], [[4, 5], [6, 7], [8, 9]]], dtype=torch.float64)
    X2 = torch.tensor([[[1.0, -2], [3, -4]], [[5, 4], [6, -7]], [[5, 6], [9, 8]]], dtype=torch.float64)
    X1d, X2d = jc.sparse.to_dense(X1).cpu(), jc.sparse.to_dense(X2).cpu()
    v1, v2 = torch.arange(6, dtype=torch.float64), torch.arange(4, dtype=torch.float64)
    sp = jc.sparse
    assert rel(sp.dot(X2, v2), X2d @ v2) < 1e-15
    assert rel(sp.dot(X1, v1), X1d @ v1) < 1e-15
    assert rel(sp.dot(v2, X1), v2 @ X1d) < 1e-15
    assert rel(sp.dot(v1, X2), v1 @ X2d) < 1e-15
    assert rel(sp.dot(X1, X2d), X1d @ X2d) < 1e-15
    assert rel(sp.dot(X1d, X2), X1d @ X2d) < 1e-15
    assert rel(sp.to_dense(sp.dot(X1, X2)), X1d @ X2d) < 1e-15
    assert rel(sp.to_dense(sp.dot(X2, X1)), X2d @ X1d) < 1e-15
    X12, X21 = sp.dot(X2, X1), sp.dot(X1, X2)
    assert rel(sp.dot(X1d, X12, X2d), X1d @ (X2d @ X1d) @ X2d) < 1e-14
    assert rel(sp.dot(X2d, X21, X1d), X2d @ (X1d @ X2d) @ X1d) < 1e-14


def test_sparse_products_random_and_batched_inverse():
    """Random float64 operands at covariance sizes: every product against the
    dense product, the batched inverse against per-matrix inverses, and an
    inverse at the 16-tracer block size (136) against torch.linalg.inv."""
    def nrel(a, b):  # max error over the largest magnitude: entries cancel to ~0
        a = a.detach().cpu() if isinstance(a, torch.Tensor) else torch.as_tensor(a)
        b = b.detach().cpu()
        return float((a - b).abs().max() / b.abs().max())

    g = torch.Generator().manual_seed(5)
    A = torch.randn(15, 9, 50, generator=g, dtype=torch.float64)
    B = torch.randn(9, 7, 50, generator=g, dtype=torch.float64)
    Ad, Bd = jc.sparse.to_dense(A).cpu(), jc.sparse.to_dense(B).cpu()
    D = torch.randn(9 * 50, 33, generator=g, dtype=torch.float64)
    E = torch.randn(21, 15 * 50, generator=g, dtype=torch.float64)
    assert nrel(jc.sparse.dot(A, D), Ad @ D) < 1e-12
    assert nrel(jc.sparse.dot(E, A), E @ Ad) < 1e-12
    assert nrel(jc.sparse.to_dense(jc.sparse.dot(A, B)), Ad @ Bd) < 1e-12
    Z = torch.randn(7 * 50, 11, generator=g, dtype=torch.float64)
    assert nrel(jc.sparse.dot(E, jc.sparse.dot(A, B), Z), E @ (Ad @ Bd) @ Z) < 1e-11
    # SPD blocks: batched inverse == one inverse per matrix; n = 136 vs torch
    M = torch.randn(3, 20, 20, 8, generator=g, dtype=torch.float64)
    S = torch.einsum("bikl,bjkl->bijl", M, M) + 20 * torch.eye(20, dtype=torch.float64)[None, :, :, None]
    inv_b = jc.sparse.inv_batched(S).cpu()
    for b in range(3):
        assert torch.equal(inv_b[b], jc.sparse.inv(S[b]).cpu())
        assert nrel(inv_b[b].permute(2, 0, 1), torch.linalg.inv(S[b].permute(2, 0, 1))) < 1e-12
    M = torch.randn(136, 136, 4, generator=g, dtype=torch.float64)
    S = torch.einsum("ikl,jkl->ijl", M, M) + 136 * torch.eye(136, dtype=torch.float64)[:, :, None]
    assert nrel(jc.sparse.inv(S).cpu().permute(2, 0, 1), torch.linalg.inv(S.permute(2, 0, 1))) < 1e-11
    sign, ld = jc.sparse.slogdet(S)
    s_ref, ld_ref = torch.linalg.slogdet(jc.sparse.to_dense(S).cpu())
    assert float(sign) == float(s_ref) and abs(float(ld) - float(ld_ref)) < 1e-10 * abs(float(ld_ref))


def test_fast_moments_match_full_moments():
    """fp32c mode evaluates the halofit moments with exp only where it matters
    (Taylor prefix sums below y^2 = 1, terms under 1e-20 dropped above
    y^2 = 60), the exp terms in float32 from a float pair y^2.  k_nl comes
    from the float64 sigma^2 table and root find: equal to ~1e-12; n_eff and C
    carry the float32 terms' rounding (a few 1e-7 relative)."""
    import ctypes

    from jax_cosmo_gb300 import _geometry, _lib

    rows = [[0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0],
            [0.35, 0.04, 0.60, 1.00, 1.00, 0.0, -1.3, 0.0],
            [0.20, 0.06, 0.80, 0.90, 0.60, 0.0, -0.7, 0.0]]
    probes = _wl2()
    ell = np.logspace(1, 3, 4)
    params = torch.as_tensor(np.asarray(rows), device="cuda")
    out = {}
    for prec in (_lib.FP64, _lib.FP32C):
        g, geo, _ = _geometry.get_geometry(probes, ell, 512, params.device)
        wsz = ctypes.c_size_t()
        _lib.call("jcg_workspace_size", ctypes.byref(g), 3, prec, ctypes.byref(wsz))
        ws = _lib.workspace(wsz.value, params.device)
        cl = torch.empty(3, 3, 4, dtype=torch.float64, device="cuda")
        st = _lib.stream_of(params.device)
        _lib.call("jcg_angular_cl", ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params), 3, prec,
                  _lib.ptr(cl), _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
        na = g.n_limber + 1
        r = torch.empty(3, na, 24, dtype=torch.float64, device="cuda")
        for i in range(3):
            _lib.call("jcg_workspace_read", ctypes.byref(g), 3, prec, _lib.ptr(ws), i, 3,
                      _lib.ptr(r[i]), ctypes.c_size_t(na * 24), st)
        out[prec] = r
    full, fast = out[_lib.FP64], out[_lib.FP32C]
    for col, tol in ((2, 1e-12), (3, 2e-6), (4, 2e-5)):  # k_nl, n_eff, C
        err = ((fast[..., col] - full[..., col]).abs() / full[..., col].abs()).max().item()
        assert err < tol, (col, err)


def _nz_probes(g):
    """The tabulated n(z) fixture's probes (tests/golden/make_golden.py, kind "nz")."""
    kde = jc.redshift.kde_nz(g["zcat"], g["w"], bw=0.1, gals_per_arcmin2=10, zmax=4.0)
    fu = jc.redshift.fu_nz(0.471, 5.1843, 0.7259, gals_per_arcmin2=30)
    shift = jc.redshift.systematic_shift(jc.redshift.smail_nz(1.0, 2.0, 0.7, gals_per_arcmin2=10), 0.05)
    return [jc.probes.WeakLensing([fu, kde, shift], sigma_e=0.26),
            jc.probes.NumberCounts([kde], jc.bias.constant_linear_bias(1.2))]


def test_tabulated_nz_vs_golden(golden):
    """fu_nz, kde_nz and systematic_shift bins: pz_fn evaluated on the device at
    libjcg's points, against the unmodified reference's C_ell; the Jacobian
    with tabulated bins against the oracle's autograd."""
    g = golden("cl_nz")
    cb = cosmo_batch(g["cosmos"])
    cl = jc.cl.angular_cl(cb, g["ell"], _nz_probes(g))
    cl32 = jc.cl.angular_cl(cb, g["ell"], _nz_probes(g), precision="fp32c")
    for i in range(len(g["cosmos"])):
        assert rel(cl[i], g["cl"][i]) < RT64
        assert rel(cl32[i], g["cl"][i]) < RT32
    # kernels at arbitrary redshifts go through the same tabulation
    zq = np.linspace(0.05, 2.5, 7)
    kq = _nz_probes(g)[1].kernel(cosmo_of(g["cosmos"][0]), zq, 100.0)
    kde = O.Kde(g["zcat"], g["w"], 0.1, zmax=4.0, gals_per_arcmin2=10)
    kref = O.probe_kernel(O.Cosmo.from_vector(g["cosmos"][0]), O.Probe("nc", [kde], bias=1.2),
                          torch.tensor(zq), 100.0)
    assert rel(kq, kref) < RT64
    ell = g["ell"][::3]
    oprobes = [O.Probe("wl", [O.Fu(0.471, 5.1843, 0.7259, gals_per_arcmin2=30), kde,
                              O.Shift(O.Smail(1.0, 2.0, 0.7, 10.0, 10), 0.05)], sigma_e=0.26),
               O.Probe("nc", [kde], bias=1.2)]
    row = list(g["cosmos"][1])

    def f(v):
        return O.angular_cl(O.Cosmo.from_vector(v), ell, oprobes, n_limber=128)

    J_o = torch.autograd.functional.jacobian(f, torch.tensor(row, dtype=torch.float64), strategy="forward-mode",
                                             vectorize=True)
    _, J = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, _nz_probes(g), 128)
    err = max(float((J[..., d].cpu() - J_o[..., d]).abs().max() / J_o[..., d].abs().max().clamp_min(1e-300))
              for d in range(8))
    assert err < 1e-8, err


def _delta_probes():
    """The single-plane fixture's probes (tests/golden/make_golden.py, kind "delta")."""
    pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
    return [jc.probes.WeakLensing([pa, jc.redshift.delta_nz(1.0, gals_per_arcmin2=5), jc.redshift.delta_nz(0.4)],
                                  multiplicative_bias=[0.0, 0.01, -0.02], sigma_e=0.26),
            jc.probes.NumberCounts([pa], jc.bias.constant_linear_bias(1.2))]


def test_single_plane_nz_vs_golden(golden):
    """delta_nz WeakLensing bins (probes.py:53-64) beside an extended bin,
    against the unmodified reference's C_ell, FP64 and fp32c; the Jacobian
    against the oracle's autograd in both precisions."""
    g = golden("cl_delta")
    cb = cosmo_batch(g["cosmos"])
    cl = jc.cl.angular_cl(cb, g["ell"], _delta_probes())
    cl32 = jc.cl.angular_cl(cb, g["ell"], _delta_probes(), precision="fp32c")
    for i in range(len(g["cosmos"])):
        assert rel(cl[i], g["cl"][i]) < RT64
        assert rel(cl32[i], g["cl"][i]) < RT32
    ell = g["ell"][::3]
    pa = O.Smail(1, 2, 0.5, 10.0, 10)
    oprobes = [O.Probe("wl", [pa, O.Delta(1.0, gals_per_arcmin2=5), O.Delta(0.4)], sigma_e=0.26,
                       m=[0.0, 0.01, -0.02]),
               O.Probe("nc", [pa], bias=1.2)]
    row = list(g["cosmos"][1])

    def f(v):
        return O.angular_cl(O.Cosmo.from_vector(v), ell, oprobes, n_limber=128)

    J_o = torch.autograd.functional.jacobian(f, torch.tensor(row, dtype=torch.float64), strategy="forward-mode",
                                             vectorize=True)
    for prec, tol in (("fp64", 1e-8), ("fp32c", 1e-4)):
        _, J = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, _delta_probes(), 128, prec)
        err = max(float((J[..., d].cpu() - J_o[..., d]).abs().max() / J_o[..., d].abs().max().clamp_min(1e-300))
                  for d in range(8))
        assert err < tol, (prec, err)


# ---------------------------------------------- non-default operator points --
PHYSICS_VARIANTS = (("eisenhu_osc", "smith2003"), ("eisenhu_osc", "linear"), ("eisenhu", "takahashi2012"))


def _fns(variant):
    import functools

    tf_type, nl = variant
    tf = functools.partial(jc.transfer.Eisenstein_Hu, type=tf_type)
    if nl == "linear":
        return tf, jc.power.linear_matter_power
    return tf, functools.partial(jc.power.halofit, prescription=nl)


def _physics_probes():
    pa = jc.redshift.smail_nz(1.0, 2.0, 0.5, gals_per_arcmin2=10)
    pb = jc.redshift.smail_nz(1.0, 2.0, 1.0, gals_per_arcmin2=10)
    return [jc.probes.WeakLensing([pa, pb], sigma_e=0.26),
            jc.probes.NumberCounts([pb], jc.bias.constant_linear_bias(1.2))]


def test_power_operator_points_vs_golden(golden):
    """Eisenstein_Hu type "eisenhu", halofit smith2003 and linear_matter_power as
    nonlinear_fn at (k, a) points against the unmodified reference."""
    import functools

    p = golden("power2")
    k = p["k"]
    nw = functools.partial(jc.transfer.Eisenstein_Hu, type="eisenhu")
    smith = functools.partial(jc.power.halofit, prescription="smith2003")
    for i, row in enumerate(p["cosmos"]):
        c = cosmo_of(row)
        assert rel(jc.transfer.Eisenstein_Hu(c, k, type="eisenhu"), p["T_nw"][i]) < RT64
        for j, a in enumerate(p["a_list"]):
            assert rel(jc.power.linear_matter_power(c, k, a, transfer_fn=nw), p["plin_nw"][i][j]) < RT64
            assert rel(jc.power.nonlinear_matter_power(c, k, a, transfer_fn=nw), p["pnl_nw"][i][j]) < RT64
            assert rel(jc.power.nonlinear_matter_power(c, k, a, nonlinear_fn=smith), p["pnl_smith"][i][j]) < RT64
            lin = jc.power.nonlinear_matter_power(c, k, a, nonlinear_fn=jc.power.linear_matter_power)
            assert rel(lin, p["pnl_lin"][i][j]) < RT64
        pairs = jc.power.nonlinear_matter_power(c, p["k_pairs"], p["a_pairs"], nonlinear_fn=smith)
        assert rel(pairs, p["pnl_smith_pairs"][i]) < RT64


@pytest.mark.parametrize("variant", PHYSICS_VARIANTS, ids=["smith2003", "linear", "nowiggle"])
def test_angular_cl_operator_points_vs_golden(golden, variant):
    """angular_cl with the non-default transfer_fn / nonlinear_fn against the
    unmodified reference (FP64 and fp32c, batched), and the Jacobian in both
    precisions against the oracle's autograd."""
    g = golden("cl_physics")
    tf, nl = _fns(variant)
    ref = g["cl_" + "_".join(variant)]
    cb = cosmo_batch(g["cosmos"])
    cl = jc.cl.angular_cl(cb, g["ell"], _physics_probes(), tf, nl)
    cl32 = jc.cl.angular_cl(cb, g["ell"], _physics_probes(), tf, nl, precision="fp32c")
    for i in range(len(g["cosmos"])):
        assert rel(cl[i], ref[i]) < RT64
        assert rel(cl32[i], ref[i]) < RT32
    # the default operator points give a different answer (the switch is live)
    assert rel(jc.cl.angular_cl(cb, g["ell"], _physics_probes())[0], ref[0]) > 1e-6
    ell = g["ell"][::3]
    pa, pb = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10)
    oprobes = [O.Probe("wl", [pa, pb], sigma_e=0.26), O.Probe("nc", [pb], bias=1.2)]
    row = list(g["cosmos"][1])

    def f(v):
        c = O.Cosmo.from_vector(v)
        c.transfer = variant[0]
        return O.angular_cl(c, ell, oprobes, n_limber=128, nonlinear=variant[1])

    J_o = torch.autograd.functional.jacobian(f, torch.tensor(row, dtype=torch.float64), strategy="forward-mode",
                                             vectorize=True)
    for prec, tol in (("fp64", 1e-8), ("fp32c", 1e-4)):
        _, J = jc.autodiff.angular_cl_jacobian(cosmo_of(row), ell, _physics_probes(), 128, prec, tf, nl)
        err = max(float((J[..., d].cpu() - J_o[..., d]).abs().max() / J_o[..., d].abs().max().clamp_min(1e-300))
                  for d in range(8))
        assert err < tol, (prec, err)


def test_gamma_growth_vs_golden(golden):
    """Cosmology(gamma=...) (background.py:515-582): growth_factor / growth_rate
    points and angular_cl (FP64 and fp32c, batched) against the unmodified
    reference; the Jacobian (gamma held fixed) against the oracle's autograd."""
    g = golden("gamma")
    rows, gms = g["cosmos"], g["gammas"]
    cb = jc.Cosmology(**{n: torch.tensor(rows[:, i]) for i, n in enumerate(NAMES)}, gamma=torch.tensor(gms))
    assert rel(jc.background.growth_factor(cb, g["a_q"]), g["D"]) < RT64
    assert rel(jc.background.growth_rate(cb, g["a_q"]), g["f"]) < RT64
    cl = jc.cl.angular_cl(cb, g["ell"], _physics_probes())
    cl32 = jc.cl.angular_cl(cb, g["ell"], _physics_probes(), precision="fp32c")
    for i in range(len(rows)):
        assert rel(cl[i], g["cl"][i]) < RT64
        assert rel(cl32[i], g["cl"][i]) < RT32
    ell = g["ell"][::3]
    pa, pb = O.Smail(1, 2, 0.5, 10.0, 10), O.Smail(1, 2, 1.0, 10.0, 10)
    oprobes = [O.Probe("wl", [pa, pb], sigma_e=0.26), O.Probe("nc", [pb], bias=1.2)]
    row, gm = list(rows[1]), float(gms[1])

    def f(v):
        c = O.Cosmo.from_vector(v[:8])
        c.gamma = v[8]
        return O.angular_cl(c, ell, oprobes, n_limber=128)

    J_o = torch.autograd.functional.jacobian(f, torch.tensor(row + [gm], dtype=torch.float64),
                                             strategy="forward-mode", vectorize=True)
    c1 = jc.Cosmology(**{n: float(v) for n, v in zip(NAMES, row)}, gamma=gm)
    for prec, tol in (("fp64", 1e-8), ("fp32c", 1e-4)):
        _, J = jc.autodiff.angular_cl_jacobian(c1, ell, _physics_probes(), 128, prec)
        assert J.shape[-1] == 9  # the 8 parameters, then gamma
        err = max(float((J[..., d].cpu() - J_o[..., d]).abs().max() / J_o[..., d].abs().max().clamp_min(1e-300))
                  for d in range(9))
        assert err < tol, (prec, err)
    # autograd through angular_cl with a gamma tensor that requires grad
    gt = torch.tensor(gm, dtype=torch.float64, requires_grad=True)
    c2 = jc.Cosmology(**{n: float(v) for n, v in zip(NAMES, row)}, gamma=gt)
    jc.cl.angular_cl(c2, ell, _physics_probes(), n_limber=128).sum().backward()
    ref = float(J_o[..., 8].sum())
    assert abs(float(gt.grad) - ref) < 1e-8 * abs(ref)


def test_fp32c_float_pair_tables_match_fp64():
    """fp32c builds the per-cosmology tables in float-pair arithmetic (the
    chi and growth right-hand sides, the sigma8 Romberg integrand and
    P(k) k^3 by pair exp / log / sin / cube root, about 48 bits) instead of
    float64: the tables the halofit root find decides on (sigma^2(R), growth,
    P(k) k^3) and chi agree with the FP64 build to 1e-12 relative, over the
    batched workload's box corners and a w0-wa cosmology."""
    import ctypes

    from jax_cosmo_gb300 import _geometry, _lib

    rows = [[0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0],
            [0.35, 0.04, 0.60, 1.00, 1.00, 0.0, -1.3, 0.0],
            [0.20, 0.06, 0.80, 0.90, 0.60, 0.0, -0.7, 0.0],
            [0.30, 0.05, 0.70, 0.95, 0.80, 0.02, -0.9, 0.3]]
    probes = _wl2()
    ell = np.logspace(1, 3, 4)
    params = torch.as_tensor(np.asarray(rows), device="cuda")
    B = len(rows)
    out = {}
    for prec in (_lib.FP64, _lib.FP32C):
        g, geo, _ = _geometry.get_geometry(probes, ell, 512, params.device)
        wsz = ctypes.c_size_t()
        _lib.call("jcg_workspace_size", ctypes.byref(g), B, prec, ctypes.byref(wsz))
        ws = _lib.workspace(wsz.value, params.device)
        st = _lib.stream_of(params.device)
        _lib.call("jcg_stage_cosmo_tables", ctypes.byref(g), _lib.ptr(params), B, prec, _lib.ptr(ws),
                  ctypes.c_size_t(ws.numel()), st)
        tabs = {}
        for what, n in ((0, 256), (1, 128), (2, 40), (5, 257), (6, 256)):
            r = torch.empty(B, n, dtype=torch.float64, device="cuda")
            for i in range(B):
                _lib.call("jcg_workspace_read", ctypes.byref(g), B, prec, _lib.ptr(ws), i, what, _lib.ptr(r[i]),
                          ctypes.c_size_t(n), st)
            tabs[what] = r
        out[prec] = tabs
    for what, name in ((0, "chi"), (1, "growth"), (5, "P(k) k^3"), (6, "sigma^2(R)")):
        a, b = out[_lib.FP32C][what], out[_lib.FP64][what]
        # relative per entry, except where the table is rounding noise around
        # zero (chi at a = 1 is a difference of two equal prefix sums)
        mask = b.abs() > 1e-9 * b.abs().amax(dim=1, keepdim=True)
        err = float(((a - b).abs()[mask] / b.abs()[mask]).max())
        print(name, "fp32c float-pair vs fp64: max rel err %.2e" % err)
        assert err < 1e-12, (name, err)
    s32, s64 = out[_lib.FP32C][2], out[_lib.FP64][2]
    for idx in (24, 25):  # sigmasqr(8), sigma8^2 / sigmasqr(8)
        assert float(((s32[:, idx] - s64[:, idx]) / s64[:, idx]).abs().max()) < 1e-12
