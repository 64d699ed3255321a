"""Host-side logic of the Python API (no GPU): descriptors, orderings, batching."""
import ctypes
import functools

import numpy as np
import pytest
import torch

import jax_cosmo_gb300 as jc
from jax_cosmo_gb300 import _geometry, _lib
from oracle import jc_oracle as O


def _probes():
    nz = [jc.redshift.smail_nz(1.0, 2.0, z0, gals_per_arcmin2=10 + i) for i, z0 in enumerate((0.5, 1.0))]
    return [
        jc.probes.WeakLensing(nz, sigma_e=0.3, multiplicative_bias=[0.01, -0.02]),
        jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(1.2)),
    ]


def test_describe_fills_descriptor():
    g = _geometry.describe(_probes(), 7, 256)
    assert g.n_tracers == 4 and g.n_ell == 7 and g.n_limber == 256 and g.zmax == 10.0
    assert list(g.kind)[:4] == [_lib.TRACER_WL] * 2 + [_lib.TRACER_NC] * 2
    assert g.mult[0] == 0.01 and g.mult[1] == -0.02 and g.mult[2] == 0.0
    assert g.bias[2] == 1.2 and g.bias[0] == 0.0
    # noise of probes.py:210-223 and 274-281
    assert g.noise[0] == pytest.approx(0.3**2 / (10 * 11818102.86004228), rel=1e-15)
    assert g.noise[3] == pytest.approx(1.0 / (11 * 11818102.86004228), rel=1e-15)
    assert _geometry.n_cls_of(g) == 10


def test_describe_bias_models():
    nz = [jc.redshift.smail_nz(1.0, 2.0, 1.0), jc.redshift.smail_nz(1.0, 2.0, 0.5)]
    P = [jc.probes.WeakLensing(nz, ia_bias=[jc.bias.des_y1_ia_bias(1.2, 0.6, 0.62),
                                            jc.bias.constant_linear_bias(0.8)], multiplicative_bias=[0.01, 0.0]),
         jc.probes.WeakLensing(nz[:1]),
         jc.probes.NumberCounts(nz, jc.bias.inverse_growth_linear_bias(1.3))]
    g = _geometry.describe(P, 3)
    assert list(g.bias_kind)[:5] == [_lib.BIAS_DES_Y1, _lib.BIAS_CONSTANT, _lib.BIAS_NONE,
                                     _lib.BIAS_INV_GROWTH, _lib.BIAS_INV_GROWTH]
    assert (g.bias[0], g.bias_eta[0], g.bias_z0[0]) == (1.2, 0.6, 0.62)
    assert g.bias[1] == 0.8 and g.bias[3] == 1.3 and g.mult[0] == 0.01
    sz = ctypes.c_size_t()
    assert _lib.load().jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == 0
    # the library validates the bias descriptors
    g.bias_kind[0] = 9
    assert _lib.load().jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_ARG
    g.bias_kind[0] = _lib.BIAS_DES_Y1
    g.bias_z0[0] = -2.0
    assert _lib.load().jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_VALUE
    with pytest.raises(ValueError):
        _geometry.describe([jc.probes.NumberCounts(nz, [jc.bias.constant_linear_bias(1.0)])], 3)


def test_describe_rejects_unsupported():
    nz = [jc.redshift.smail_nz(1.0, 2.0, 1.0)]

    class other_bias(jc.jax_utils.container):
        pass

    with pytest.raises(NotImplementedError):
        _geometry.describe([jc.probes.NumberCounts(nz, other_bias(1.0))], 3)

    class other_nz(jc.redshift.redshift_distribution):
        def pz_fn(self, z):
            return z

    # any redshift_distribution is tabulated; single-plane bins on WeakLensing only
    g = _geometry.describe([jc.probes.WeakLensing([other_nz(zmax=3.0), jc.redshift.smail_nz(1, 2, 1)])], 3)
    assert list(g.nz_kind)[:2] == [_lib.NZ_TABLE, _lib.NZ_SMAIL] and g.nz_zmax[0] == 3.0
    gd = _geometry.describe([jc.probes.WeakLensing([jc.redshift.delta_nz(1.5)])], 3)
    assert gd.nz_kind[0] == _lib.NZ_DELTA and gd.nz_z0[0] == 1.5 and gd.nz_zmax[0] == 10.0
    sz = ctypes.c_size_t()
    assert _lib.load().jcg_geometry_size(ctypes.byref(gd), ctypes.byref(sz)) == 0
    with pytest.raises(NotImplementedError):
        _geometry.describe([jc.probes.NumberCounts([jc.redshift.delta_nz(1.0)], jc.bias.constant_linear_bias(1.0))], 3)
    gd.kind[0] = _lib.TRACER_NC  # the library refuses a single plane on NumberCounts too
    assert _lib.load().jcg_geometry_size(ctypes.byref(gd), ctypes.byref(sz)) == _lib.ERR_ARG
    # the point list has 257 + na (+ na x 257 for lensing) entries per tracer
    cnt = ctypes.c_size_t()
    assert _lib.load().jcg_geometry_nz_points(ctypes.byref(g), None, None, ctypes.byref(cnt), None) == 0
    assert cnt.value == 2 * (257 + 513 + 513 * 257)
    with pytest.raises(ValueError):
        _geometry.describe([jc.probes.WeakLensing([jc.redshift.smail_nz(1, 2, 1)] * 17)], 3)


def test_orderings_match_reference_rules():
    P = _probes()
    assert jc.cl._get_cl_ordering(P) == O.cl_ordering(4)
    assert jc.cl._get_cov_blocks_ordering(P) == O.cov_blocks_ordering(4)


def test_cosmology_batching():
    c = jc.Planck15()
    assert c.batch_size is None
    p = c.param_tensor("cpu")
    assert p.shape == (1, 8) and p.dtype == torch.float64
    assert p[0, 0].item() == 0.2589 and p[0, 6].item() == -1.0
    cb = jc.Planck15(Omega_c=torch.linspace(0.2, 0.3, 5), sigma8=np.full(5, 0.8))
    assert cb.batch_size == 5
    pb = cb.param_tensor("cpu")
    assert pb.shape == (5, 8)
    assert torch.allclose(pb[:, 0], torch.linspace(0.2, 0.3, 5, dtype=torch.float64))
    assert (pb[:, 2] == 0.6774).all()
    with pytest.raises(ValueError):
        jc.Planck15(Omega_c=torch.ones(3), h=torch.ones(4)).batch_size
    with pytest.raises(ValueError):
        jc.Planck15(Omega_c=float("nan")).param_tensor("cpu")
    assert jc.Planck15().Omega_m == pytest.approx(0.3075)
    assert jc.Cosmology.tree_unflatten(*reversed(c.tree_flatten())).h == 0.6774


def test_physics_codes():
    """The operator points of angular_cl map to the descriptor's physics word
    (transfer.py:10-156, power.py:144-272)."""
    tf, hf = jc.transfer.Eisenstein_Hu, jc.power.halofit
    nw = functools.partial(tf, type="eisenhu")
    assert jc.cl.physics_code(tf, hf) == 0
    assert jc.cl.physics_code(functools.partial(tf, type="eisenhu_osc"), functools.partial(hf)) == 0
    assert jc.cl.physics_code(tf, functools.partial(hf, prescription="smith2003")) == _lib.PK_SMITH2003
    assert jc.cl.physics_code(tf, jc.power.linear_matter_power) == _lib.PK_LINEAR
    assert jc.cl.physics_code(nw, hf) == _lib.TF_NOWIGGLE
    assert jc.cl.physics_code(nw, jc.power.linear_matter_power) == _lib.TF_NOWIGGLE | _lib.PK_LINEAR
    g = _geometry.describe([jc.probes.WeakLensing([jc.redshift.smail_nz(1.0, 2.0, 0.5)])], 4, physics=0x11)
    assert g.physics == 0x11
    # the library validates the physics word (host-side, no GPU needed)
    sz = ctypes.c_size_t()
    lib = _lib.load()
    for ok in (0, _lib.PK_SMITH2003, _lib.PK_LINEAR | _lib.TF_NOWIGGLE, _lib.GROWTH_GAMMA | _lib.PK_SMITH2003):
        g.physics = ok
        assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == 0
    for bad in (3, 0x40, 0x100):
        g.physics = bad
        assert lib.jcg_geometry_size(ctypes.byref(g), ctypes.byref(sz)) == _lib.ERR_UNSUPPORTED


def test_smail_nz_host_evaluation_matches_oracle():
    nz = jc.redshift.smail_nz(1.0, 2.0, 0.5, zmax=4.0)
    z = torch.linspace(0, 4, 41, dtype=torch.float64)
    ref = O.Smail(1.0, 2.0, 0.5, 4.0)(z)
    assert torch.allclose(nz(z), ref, rtol=1e-14, atol=0)


def test_unsupported_options_raise():
    c = jc.Planck15()
    with pytest.raises(NotImplementedError):
        jc.cl.physics_code(lambda *a: None, jc.power.halofit)
    with pytest.raises(NotImplementedError):
        jc.cl.physics_code(jc.transfer.Eisenstein_Hu, lambda *a: None)
    with pytest.raises(NotImplementedError):
        jc.cl.physics_code(functools.partial(jc.transfer.Eisenstein_Hu, type="bbks"), jc.power.halofit)
    with pytest.raises(NotImplementedError):
        jc.cl.physics_code(jc.transfer.Eisenstein_Hu, functools.partial(jc.power.halofit, prescription="x"))
    with pytest.raises(ValueError):
        jc.cl._precision_code("fp16")
    # gamma growth: the parameter rows carry gamma as a 9th column and the
    # descriptor's physics word the GROWTH_GAMMA bit
    cg = jc.Cosmology(0.25, 0.05, 0.7, 0.96, 0.8, 0.0, -1.0, 0.0, gamma=0.55)
    pg = cg.param_tensor("cpu")
    assert pg.shape == (1, 9) and float(pg[0, 8]) == 0.55
    assert cg.physics_bits() == _lib.GROWTH_GAMMA and c.physics_bits() == 0
