"""ORACLE — test infrastructure, not product code.

CPU float64 restatement of jax_cosmo's angular-power-spectrum path, written with
torch on the CPU so that autograd gives the gradient oracle (``jax.grad`` of the
reference is not available in this environment).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs may
import this module, and only to check results against it or as the timed CPU
baseline.

Every function follows the reference file and line it names (paths relative to
the jax_cosmo project root).  It reproduces the reference's numerical quirks:

* ``interp`` takes the nearest node by ``argmin((x - xp)**2)`` (first index on
  ties), clips it to ``[1, n-2]`` and picks the side by
  ``sign(clip(x, xp[1], xp[-2]) - xp[ind])`` (scipy/interpolate.py:34-59);
* RK4 ``odeint`` steps on the output grid, first step h = 0 (scipy/ode.py:6-22);
* ``sigmasqr`` integrates ln k over [log10 kmin, log10 kmax] = [-4, 3] with a
  7-level Romberg rule (power.py:56-78, scipy/integrate.py:67-159);
* the halofit non-linear scale is the quirky ``interp`` of a 256-node
  sigma^2(R) table (power.py:93-115);
* ``gaussian_log_likelihood`` returns ``-0.5 * (r^T C^-1 r - logdet)``
  (likelihood.py:61), i.e. ``+0.5 logdet``.

Grid sizes that the reference hard-codes are keyword arguments with the
reference's defaults (``n_limber=512``: angular_cl.py:96).  Grids are built with
NumPy exactly as the reference builds them (``np.linspace`` / ``np.logspace``),
so that the oracle sees the same nodes as the reference run under NumPy.

Parity pin: ``tests/test_oracle_golden.py`` checks this module against
fixtures produced by the unmodified reference source
(``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

DT = torch.float64

# jax_cosmo/constants.py:9-27, jax_cosmo/redshift.py:10
C_KMS = 299792.458
TCMB = 2.726
RH = 2997.92458
H0 = 100.0
RHOCRIT = 2.7750 * 1e11  # constants.py:30
STERADIAN_TO_ARCMIN2 = 11818102.86004228

PARAM_NAMES = ("Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa")


def _t(x):
    if isinstance(x, torch.Tensor):
        return x.to(DT)
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


@dataclass
class Cosmo:
    """Cosmological parameters (core.py:11-198); each is a 0-d float64 tensor."""

    Omega_c: torch.Tensor
    Omega_b: torch.Tensor
    h: torch.Tensor
    n_s: torch.Tensor
    sigma8: torch.Tensor
    Omega_k: torch.Tensor
    w0: torch.Tensor
    wa: torch.Tensor
    cache: dict = field(default_factory=dict)
    # the transfer_fn type of every call on this object ("eisenhu_osc" or
    # "eisenhu", transfer.py:10): the sigma_8 normalisation and the sigma^2(R)
    # table cached here depend on it
    transfer: str = "eisenhu_osc"
    # growth-rate index (core.py:13, 52-54): None -> growth ODE, else
    # f = Omega_m(a)^gamma (background.py:515-582)
    gamma: object = None

    @classmethod
    def from_vector(cls, v):
        v = _t(v)
        return cls(*[v[i] for i in range(8)])

    def vector(self):
        return torch.stack([getattr(self, n) for n in PARAM_NAMES])

    @property
    def Omega_m(self):  # core.py:157
        return self.Omega_b + self.Omega_c

    @property
    def Omega(self):  # core.py:145
        return 1.0 - self.Omega_k

    @property
    def Omega_de(self):  # core.py:161
        return self.Omega - self.Omega_m


def planck15():
    """parameters.py:10-20"""
    return Cosmo.from_vector([0.2589, 0.04860, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0])


def z2a(z):  # utils.py:2
    return 1.0 / (1.0 + z)


def a2z(a):  # utils.py:7
    return 1.0 / a - 1.0


# ---------------------------------------------------------------- numerics ----
def clip(x, lo=None, hi=None):
    """jnp.clip = minimum(maximum(x, lo), hi)."""
    if lo is not None:
        x = torch.maximum(x, _t(lo) if not isinstance(lo, torch.Tensor) else lo)
    if hi is not None:
        x = torch.minimum(x, _t(hi) if not isinstance(hi, torch.Tensor) else hi)
    return x


def interp(x, xp, fp, chunk=1 << 14):
    """scipy/interpolate.py:34-59, including the nearest-node / side quirks."""
    x = x.reshape(-1)
    n = xp.shape[0]
    xd = x.detach()
    xpd = xp.detach()
    inds = []
    for s in range(0, xd.shape[0], chunk):
        d = xd[s : s + chunk, None] - xpd[None, :]
        inds.append(torch.argmin(d * d, dim=1))
    ind = torch.cat(inds) if inds else torch.zeros(0, dtype=torch.long)
    ind = ind.clamp(1, n - 2)
    xi = xpd[ind]
    side = torch.sign(clip(xd, xpd[1], xpd[n - 2]) - xi)
    step = torch.where(side >= 0, 1, -1)
    j = ind + step
    a = (fp[j] - fp[ind]) / (xp[j] - xp[ind])
    b = fp[ind] - a * xp[ind]
    return a * x + b


def simps_weights_apply(y, dx):
    """Composite Simpson sum of samples y (axis 0): scipy/integrate.py:195-199."""
    return dx / 3 * torch.sum(y[0:-1:2] + 4 * y[1::2] + y[2::2], dim=0)


def simps(f, a, b, N=128):
    """scipy/integrate.py:162-199 (array endpoints allowed)."""
    if N % 2 == 1:
        raise ValueError("N must be an even integer.")
    a_np = a.detach().numpy() if isinstance(a, torch.Tensor) else a
    b_np = b.detach().numpy() if isinstance(b, torch.Tensor) else b
    x = _t(np.linspace(a_np, b_np, N + 1))
    dx = (_t(b) - _t(a)) / N
    return simps_weights_apply(f(x), dx)


def romb(f, a, b, divmax=6):
    """scipy/integrate.py:21-159 (trapezoid refinements + Richardson table)."""
    intrange = b - a
    ordsum = 0.5 * (f(_t(a)) + f(_t(b)))
    result = intrange * ordsum
    state = [result] * (divmax + 1)
    for i in range(1, divmax + 1):
        n = 2**i
        numtosum = n // 2
        h = (1.0 * b - 1.0 * a) / numtosum
        lox = a + 0.5 * h
        points = lox + h * np.arange(0, numtosum)
        ordsum = ordsum + torch.sum(f(_t(points)))
        x = intrange * ordsum / n
        new = [x]
        for k in range(divmax):
            tmp = 4.0 ** (k + 1)
            x = (tmp * x - state[k]) / (tmp - 1.0)
            new.append(x)
        state = new
    return state[divmax]


def odeint_rk4(fn, y0, t):
    """scipy/ode.py:6-22: RK4 on the output grid, first step h = 0."""
    y = y0
    t_prev = t[0]
    ys = []
    for i in range(t.shape[0]):
        ti = t[i]
        h = ti - t_prev
        k1 = fn(y, t_prev)
        k2 = fn(y + h * k1 / 2, t_prev + h / 2)
        k3 = fn(y + h * k2 / 2, t_prev + h / 2)
        k4 = fn(y + h * k3, ti)
        y = y + 1.0 / 6.0 * h * (k1 + 2 * k2 + 2 * k3 + k4)
        t_prev = ti
        ys.append(y)
    return torch.stack(ys)


# -------------------------------------------------------------- background ----
def w(c, a):  # background.py:25-53
    return c.w0 + (1.0 - a) * c.wa


def f_de(c, a):  # background.py:56-90
    return -3.0 * (1.0 + c.w0 + c.wa) * torch.log(a) + 3.0 * c.wa * (a - 1.0)


def Esqr(c, a):  # background.py:93-126
    return (
        c.Omega_m * torch.pow(a, -3)
        + c.Omega_k * torch.pow(a, -2)
        + c.Omega_de * torch.exp(f_de(c, a))
    )


def H(c, a):  # background.py:129-142
    return H0 * torch.sqrt(Esqr(c, a))


def Omega_m_a(c, a):  # background.py:145-168
    return c.Omega_m * torch.pow(a, -3) / Esqr(c, a)


def Omega_de_a(c, a):  # background.py:171-196
    return c.Omega_de * torch.exp(f_de(c, a)) / Esqr(c, a)


def dchioverda(c, a):  # background.py:270-294
    return RH / (a**2 * torch.sqrt(Esqr(c, a)))


def chi_table(c, log10_amin=-3, steps=256):
    """background.py:223-236: RK4 of dchi/dln a on logspace(-3, 0, 256)."""
    key = ("chi", log10_amin, steps)
    if key not in c.cache:
        atab = _t(np.logspace(log10_amin, 0.0, steps))

        def dchioverdlna(y, x):
            xa = torch.exp(x)
            return dchioverda(c, xa) * xa

        chitab = odeint_rk4(dchioverdlna, _t(0.0), torch.log(atab))
        chitab = chitab[-1] - chitab
        c.cache[key] = (atab, chitab)
    return c.cache[key]


def radial_comoving_distance(c, a):
    """background.py:199-242"""
    atab, chitab = chi_table(c)
    a = torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)
    return clip(interp(a, atab, chitab), 0.0)


def growth_table(c, log10_amin=-3, steps=128):
    """background.py:443-487: RK4 of the growth ODE in a on logspace(-3, 0, 128);
    with c.gamma, background.py:515-552: RK4 in ln a of Omega_m(a)^gamma."""
    key = ("growth", log10_amin, steps)
    if key not in c.cache and c.gamma is not None:
        atab = _t(np.logspace(log10_amin, 0.0, steps))

        def integrand(y, loga):
            return Omega_m_a(c, torch.exp(loga)) ** c.gamma

        gtab = torch.exp(odeint_rk4(integrand, torch.log(atab[0]), torch.log(atab)))
        c.cache[key] = (atab, gtab / gtab[-1])
    if key not in c.cache:
        atab = _t(np.logspace(log10_amin, 0.0, steps))

        def D_derivs(y, x):
            q = (
                2.0
                - 0.5 * (Omega_m_a(c, x) + (1.0 + 3.0 * w(c, x)) * Omega_de_a(c, x))
            ) / x
            r = 1.5 * Omega_m_a(c, x) / x / x
            return torch.stack([y[1], -q * y[1] + r * y[0]])

        y0 = torch.stack([atab[0], _t(1.0)])
        y = odeint_rk4(D_derivs, y0, atab)
        y1 = y[:, 0]
        gtab = y1 / y1[-1]
        # dlnD/dlna = a / D dD/da (background.py:484-485)
        ftab = y[:, 1] / y1[-1] * atab / gtab
        c.cache[key] = (atab, gtab)
        c.cache[("growth_rate",) + key[1:]] = (atab, ftab)
    return c.cache[key]


def growth_factor(c, a):
    """background.py:371-398, 488"""
    atab, gtab = growth_table(c)
    a = torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)
    return clip(interp(a, atab, gtab), 0.0, 1.0)


def growth_rate(c, a):
    """background.py:401-440, 491-512: interp(a, atab, ftab) of the ODE growth, no clip;
    with c.gamma, Omega_m(a)^gamma (background.py:555-582)."""
    if c.gamma is not None:
        return Omega_m_a(c, torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)) ** c.gamma
    growth_table(c)
    atab, ftab = c.cache[("growth_rate", -3, 128)]
    a = torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)
    return interp(a, atab, ftab)


def a_of_chi(c, chi):
    """background.py:245-267: interp(chi, chi table, a table) (the decreasing chi table)."""
    atab, chitab = chi_table(c)
    chi = torch.atleast_1d(_t(chi) if not isinstance(chi, torch.Tensor) else chi)
    return interp(chi, chitab, atab)


def transverse_comoving_distance(c, a):
    """background.py:297-344: branch by k = -sign(Omega_k) (core.py:169-174)."""
    chi = radial_comoving_distance(c, a)
    ok = c.Omega_k
    ok_v = float(ok.detach()) if isinstance(ok, torch.Tensor) else float(ok)
    if ok_v == 0.0:
        return chi
    sk = torch.sqrt(torch.abs(_t(ok) if not isinstance(ok, torch.Tensor) else ok))
    if ok_v > 0.0:
        return RH / sk * torch.sinh(sk * chi / RH)
    return RH / sk * torch.sin(sk * chi / RH)


def angular_diameter_distance(c, a):
    """background.py:347-368: a f_k(a)."""
    a_t = torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)
    return a_t * transverse_comoving_distance(c, a_t)


# ---------------------------------------------------------------- transfer ----
def eisenstein_hu(c, k):
    """transfer.py:10-156, type c.transfer ('eisenhu_osc' or 'eisenhu')."""
    T_2_7_sqr = (TCMB / 2.7) ** 2
    h2 = c.h**2
    w_m = c.Omega_m * h2
    w_b = c.Omega_b * h2
    fb = c.Omega_b / c.Omega_m
    fc = (c.Omega_m - c.Omega_b) / c.Omega_m
    k_eq = 7.46e-2 * w_m / T_2_7_sqr / c.h
    z_eq = 2.50e4 * w_m / (T_2_7_sqr) ** 2
    b1 = 0.313 * torch.pow(w_m, -0.419) * (1.0 + 0.607 * torch.pow(w_m, 0.674))
    b2 = 0.238 * torch.pow(w_m, 0.223)
    z_d = (
        1291.0
        * torch.pow(w_m, 0.251)
        / (1.0 + 0.659 * torch.pow(w_m, 0.828))
        * (1.0 + b1 * torch.pow(w_b, b2))
    )
    R_d = 31.5 * w_b / (T_2_7_sqr) ** 2 * (1.0e3 / z_d)
    R_eq = 31.5 * w_b / (T_2_7_sqr) ** 2 * (1.0e3 / z_eq)
    sh_d = (
        2.0
        / (3.0 * k_eq)
        * torch.sqrt(6.0 / R_eq)
        * torch.log((torch.sqrt(1.0 + R_d) + torch.sqrt(R_eq + R_d)) / (1.0 + torch.sqrt(R_eq)))
    )
    k_silk = (
        1.6
        * torch.pow(w_b, 0.52)
        * torch.pow(w_m, 0.73)
        * (1.0 + torch.pow(10.4 * w_m, -0.95))
        / c.h
    )
    if c.transfer == "eisenhu":
        # transfer.py:88-105: zero-baryon fit with the effective shape gamma_eff(k)
        alpha_gamma = (
            1.0
            - 0.328 * torch.log(431.0 * w_m) * w_b / w_m
            + 0.38 * torch.log(22.3 * w_m) * (c.Omega_b / c.Omega_m) ** 2
        )
        gamma_eff = c.Omega_m * c.h * (alpha_gamma + (1.0 - alpha_gamma) / (1.0 + (0.43 * k * sh_d) ** 4))
        q = k * (TCMB / 2.7) ** 2 / gamma_eff
        L = torch.log(2.0 * math.exp(1.0) + 1.8 * q)
        C = 14.2 + 731.0 / (1.0 + 62.5 * q)
        return L / (L + C * q * q)
    if c.transfer != "eisenhu_osc":
        raise NotImplementedError(c.transfer)
    a1 = torch.pow(46.9 * w_m, 0.670) * (1.0 + torch.pow(32.1 * w_m, -0.532))
    a2 = torch.pow(12.0 * w_m, 0.424) * (1.0 + torch.pow(45.0 * w_m, -0.582))
    alpha_c = torch.pow(a1, -fb) * torch.pow(a2, -(fb**3))
    b1 = 0.944 / (1.0 + torch.pow(458.0 * w_m, -0.708))
    b2 = torch.pow(0.395 * w_m, -0.0266)
    beta_c = 1.0 + b1 * (torch.pow(fc, b2) - 1.0)
    beta_c = 1.0 / beta_c

    def T_tilde(k1, alpha, beta):
        q = k1 / (13.41 * k_eq)
        L = torch.log(math.exp(1.0) + 1.8 * beta * q)
        C = 14.2 / alpha + 386.0 / (1.0 + 69.9 * torch.pow(q, 1.08))
        return L / (L + C * q * q)

    f = 1.0 / (1.0 + (k * sh_d / 5.4) ** 4)
    Tc = f * T_tilde(k, 1.0, beta_c) + (1.0 - f) * T_tilde(k, alpha_c, beta_c)
    y = (1.0 + z_eq) / (1.0 + z_d)
    x = torch.sqrt(1.0 + y)
    G_EH98 = y * (-6.0 * x + (2.0 + 3.0 * y) * torch.log((x + 1.0) / (x - 1.0)))
    alpha_b = 2.07 * k_eq * sh_d * torch.pow(1.0 + R_d, -0.75) * G_EH98
    beta_node = 8.41 * torch.pow(w_m, 0.435)
    tilde_s = sh_d / torch.pow(1.0 + (beta_node / (k * sh_d)) ** 3, 1.0 / 3.0)
    beta_b = 0.5 + fb + (3.0 - 2.0 * fb) * torch.sqrt((17.2 * w_m) ** 2 + 1.0)
    xs = k * tilde_s / math.pi
    sinc = torch.sin(math.pi * xs) / (math.pi * xs)  # np.sinc, k > 0
    Tb = (
        T_tilde(k, 1.0, 1.0) / (1.0 + (k * sh_d / 5.2) ** 2)
        + alpha_b / (1.0 + (beta_b / (k * sh_d)) ** 3) * torch.exp(-torch.pow(k / k_silk, 1.4))
    ) * sinc
    return fb * Tb + fc * Tc


# ------------------------------------------------------------------- power ----
def primordial_matter_power(c, k):  # power.py:14-18
    return k**c.n_s


def sigmasqr(c, R=8.0, kmin=0.0001, kmax=1000.0):
    """power.py:56-78 (romb over [log10 kmin, log10 kmax] with k = exp(logk))."""
    key = ("sigmasqr", R)
    if key not in c.cache:

        def int_sigma(logk):
            k = torch.exp(logk)
            x = k * R
            wf = 3.0 * (torch.sin(x) - x * torch.cos(x)) / (x * x * x)
            pk = eisenstein_hu(c, k) ** 2 * primordial_matter_power(c, k)
            return k * (k * wf) ** 2 * pk

        y = romb(int_sigma, math.log10(kmin), math.log10(kmax), divmax=7)
        c.cache[key] = 1.0 / (2.0 * math.pi**2.0) * y
    return c.cache[key]


def linear_matter_power(c, k, a=1.0):
    """power.py:21-53"""
    k = torch.atleast_1d(_t(k) if not isinstance(k, torch.Tensor) else k)
    a = torch.atleast_1d(_t(a) if not isinstance(a, torch.Tensor) else a)
    g = growth_factor(c, a)
    t = eisenstein_hu(c, k)
    pknorm = c.sigma8**2 / sigmasqr(c, 8.0)
    pk = primordial_matter_power(c, k) * t**2 * g**2
    pk = pk * pknorm
    return pk.squeeze()


def _halofit_k_grid():
    # power.py:111 / :136: simps(..., log(1e-4), log(1e4), 256)
    logk = np.linspace(np.log(1e-4), np.log(1e4), 257)
    return _t(logk), (np.log(1e4) - np.log(1e-4)) / 256


def sigma_r_table(c):
    """sigma^2(R) at a = 1 on the 256 log-R nodes of power.py:93, without g(a)^2.

    power.py:98-111 builds ``pk*k^3 * exp(-(kR)^2) / (2 pi^2) * g^2`` and
    integrates over ln k; g^2 is a common factor, applied by the caller.
    """
    key = "sigma_r"
    if key not in c.cache:
        logr = _t(np.linspace(np.log(1e-4), np.log(1e1), 256))
        logk, dx = _halofit_k_grid()
        k = torch.exp(logk)
        r = torch.exp(logr)
        y = torch.outer(k, r)
        pk = linear_matter_power(c, k)
        integ = (pk * k**3)[:, None] * torch.exp(-(y**2)) / (2.0 * math.pi**2)
        c.cache[key] = (logr, simps_weights_apply(integ, dx))
    return c.cache[key]


def interp_rows(x, xp, fp):
    """``interp`` of one query per row of ``xp`` ([n, m]) with shared ``fp`` ([m]).

    Same arithmetic as :func:`interp`, batched over the rows; used for the
    halofit root find (power.py:112), where the table changes with a.
    """
    n = xp.shape[1]
    xpd = xp.detach()
    d = x[:, None] - xpd
    ind = torch.argmin(d * d, dim=1).clamp(1, n - 2)
    rows = torch.arange(xp.shape[0])
    xi = xpd[rows, ind]
    side = torch.sign(clip(x, xpd[:, 1], xpd[:, n - 2]) - xi)
    j = ind + torch.where(side >= 0, 1, -1)
    a = (fp[j] - fp[ind]) / (xp[rows, j] - xp[rows, ind])
    b = fp[ind] - a * xp[rows, ind]
    return a * x + b


def halofit_parameters(c, a):
    """power.py:86-141 -> (k_nl, n_eff, C) at each scale factor in ``a``."""
    a = torch.atleast_1d(a)
    key = ("halofit_params", a.shape[0], float(a.detach()[0]), float(a.detach()[-1]))
    if key in c.cache and torch.equal(c.cache[key][0], a.detach()):
        return c.cache[key][1]
    g = growth_factor(c, a)
    logr, s0 = sigma_r_table(c)
    sigma = s0[None, :] * (g**2)[:, None]
    one = torch.ones(a.shape[0], dtype=DT)
    roots = interp_rows(one, sigma, logr)
    R_nl = clip(torch.exp(roots), 1e-6)
    k_nl = 1.0 / R_nl
    logk, dx = _halofit_k_grid()
    k = torch.exp(logk)
    y = torch.outer(k, 1.0 / k_nl)
    pk = linear_matter_power(c, k)
    res = (pk * k**3)[:, None] * torch.exp(-(y**2)) * (g**2)[None, :] / (2.0 * math.pi**2)
    dneff = simps_weights_apply(2 * res * y**2, dx)
    dC = simps_weights_apply(4 * res * (y**2 - y**4), dx)
    n_eff = dneff - 3.0
    C = dneff**2 + dC
    out = (k_nl, n_eff, C)
    c.cache[key] = (a.detach().clone(), out)
    return out


def halofit_coefs(n, C, om_m, om_de, ww, prescription="takahashi2012"):
    """power.py:177-244 -> (a_n, b_n, c_n, gamma_n, alpha_n, beta_n, mu_n, nu_n, f1, f2, f3)."""
    if prescription == "smith2003":
        # eq C9 to C18 (power.py:182-198)
        a_n = 10 ** (1.4861 + 1.8369 * n + 1.6762 * n**2 + 0.7940 * n**3 + 0.1670 * n**4 - 0.6206 * C)
        b_n = 10 ** (0.9463 + 0.9466 * n + 0.3084 * n**2 - 0.9400 * C)
        c_n = 10 ** (-0.2807 + 0.6669 * n + 0.3214 * n**2 - 0.0793 * C)
        gamma_n = 0.8649 + 0.2989 * n + 0.1631 * C
        alpha_n = 1.3884 + 0.3700 * n - 0.1452 * n**2
        beta_n = 0.8291 + 0.9854 * n + 0.3401 * n**2
        mu_n = 10 ** (-3.5442 + 0.1908 * n)
        nu_n = 10 ** (0.9585 + 1.2857 * n)
    elif prescription == "takahashi2012":
        a_n = 10 ** (
            1.5222 + 2.8553 * n + 2.3706 * n**2 + 0.9903 * n**3 + 0.2250 * n**4
            - 0.6038 * C + 0.1749 * om_de * (1 + ww)
        )
        b_n = 10 ** (-0.5642 + 0.5864 * n + 0.5716 * n**2 - 1.5474 * C + 0.2279 * om_de * (1 + ww))
        c_n = 10 ** (0.3698 + 2.0404 * n + 0.8161 * n**2 + 0.5869 * C)
        gamma_n = 0.1971 - 0.0843 * n + 0.8460 * C
        alpha_n = torch.abs(6.0835 + 1.3373 * n - 0.1959 * n**2 - 5.5274 * C)
        beta_n = (
            2.0379 - 0.7354 * n + 0.3157 * n**2 + 1.2490 * n**3 + 0.3980 * n**4 - 0.1682 * C
        )
        mu_n = 0.0
        nu_n = 10 ** (5.2105 + 3.6902 * n)
    else:
        raise NotImplementedError(prescription)
    f1b, f2b, f3b = om_m ** (-0.0307), om_m ** (-0.0585), om_m ** (0.0743)
    if prescription == "takahashi2012":
        f1, f2, f3 = f1b, f2b, f3b
    else:
        # power.py:180, 227-242
        frac = om_de / (1.0 - om_m)
        f1 = frac * f1b + (1 - frac) * om_m ** (-0.0732)
        f2 = frac * f2b + (1 - frac) * om_m ** (-0.1423)
        f3 = frac * f3b + (1 - frac) * om_m**0.0725
    return a_n, b_n, c_n, gamma_n, alpha_n, beta_n, mu_n, nu_n, f1, f2, f3


def _halofit_from(k, pklin, k_nl, coefs):
    """power.py:246-260"""
    a_n, b_n, c_n, gamma_n, alpha_n, beta_n, mu_n, nu_n, f1, f2, f3 = coefs
    d2l = k**3 * pklin / (2.0 * math.pi**2)
    y = k / k_nl
    fy = y / 4.0 + y**2 / 8.0
    d2q = d2l * ((1.0 + d2l) ** beta_n / (1 + alpha_n * d2l)) * torch.exp(-fy)
    d2hprime = a_n * y ** (3 * f1) / (1.0 + b_n * y**f2 + (c_n * f3 * y) ** (3.0 - gamma_n))
    d2h = d2hprime / (1.0 + mu_n / y + nu_n / y**2)
    return 2.0 * math.pi**2 / k**3 * (d2q + d2h)


def halofit(c, k, a, prescription="takahashi2012"):
    """power.py:144-262"""
    a = torch.atleast_1d(a)
    pklin = linear_matter_power(c, k, a)
    k_nl, n, C = halofit_parameters(c, a)
    coefs = halofit_coefs(n, C, Omega_m_a(c, a), Omega_de_a(c, a), w(c, a), prescription)
    return _halofit_from(k, pklin, k_nl, coefs).squeeze()


# ----------------------------------------------------------------- tracers ----
@dataclass
class Smail:
    """redshift.py:15-77: n(z) = z^a exp(-(z/z0)^b) / simps(0, zmax, 256)."""

    a: float
    b: float
    z0: float
    zmax: float = 10.0
    gals_per_arcmin2: float = 1.0

    def pz_fn(self, z):
        return z**self.a * torch.exp(-((z / self.z0) ** self.b))

    @property
    def norm(self):
        return simps(self.pz_fn, 0.0, self.zmax, 256)

    def __call__(self, z):
        return self.pz_fn(z) / self.norm

    @property
    def gals_per_steradian(self):
        return self.gals_per_arcmin2 * STERADIAN_TO_ARCMIN2


class _NZ:
    """Normalised n(z) of a pz_fn (redshift.py:15-58): pz_fn(z) / simps(pz_fn, 0, zmax, 256)."""

    zmax = 10.0
    gals_per_arcmin2 = 1.0

    @property
    def norm(self):
        return simps(self.pz_fn, 0.0, self.zmax, 256)

    def __call__(self, z):
        return self.pz_fn(z) / self.norm

    @property
    def gals_per_steradian(self):
        return self.gals_per_arcmin2 * STERADIAN_TO_ARCMIN2


class Fu(_NZ):
    """redshift.py:80-105: (z^a + z^(a b)) / (z^b + c)."""

    def __init__(self, a, b, c, zmax=10.0, gals_per_arcmin2=1.0):
        self.a, self.b, self.c, self.zmax, self.gals_per_arcmin2 = a, b, c, zmax, gals_per_arcmin2

    def pz_fn(self, z):
        return (z**self.a + z ** (self.a * self.b)) / (z**self.b + self.c)


class Kde(_NZ):
    """redshift.py:125-156: Gaussian KDE of a weighted catalog."""

    def __init__(self, zcat, w, bw, zmax=10.0, gals_per_arcmin2=1.0):
        self.zcat, self.w, self.bw = _t(zcat), _t(w), bw
        self.zmax, self.gals_per_arcmin2 = zmax, gals_per_arcmin2

    def pz_fn(self, z):
        shape = z.shape
        zf = z.reshape(-1)
        X = self.zcat[:, None]
        k = (1.0 / math.sqrt(2 * math.pi) / self.bw) * torch.exp(-((X - zf[None, :]) ** 2) / (self.bw**2 * 2.0))
        return (k.T @ self.w / torch.sum(self.w)).reshape(shape)


class Shift(_NZ):
    """redshift.py:159-171: parent pz_fn at clip(z - bias, 0)."""

    def __init__(self, parent, bias, zmax=10.0, gals_per_arcmin2=1.0):
        self.parent, self.bias, self.zmax, self.gals_per_arcmin2 = parent, bias, zmax, gals_per_arcmin2

    def pz_fn(self, z):
        return self.parent.pz_fn(clip(z - self.bias, 0.0))


class Delta(_NZ):
    """redshift.py:108-122: a single plane at z0, norm 1, pz_fn = (z == z0)."""

    def __init__(self, z0, zmax=10.0, gals_per_arcmin2=1.0):
        self.z0, self.zmax, self.gals_per_arcmin2 = z0, zmax, gals_per_arcmin2

    @property
    def norm(self):
        return 1.0

    def pz_fn(self, z):
        return torch.where(z == self.z0, 1.0, 0.0).to(torch.float64)


@dataclass
class Probe:
    """A WeakLensing ('wl') or NumberCounts ('nc') probe (probes.py:132-281).

    ``bias`` (NC galaxy bias) and ``ia`` (WL NLA bias, None = no intrinsic
    alignment) are a number (constant_linear_bias), a bias spec tuple
    ("const", b) / ("invg", b) / ("desy1", A, eta, z0) (bias.py:10-57), or a
    list of those, one per bin.
    """

    kind: str
    bins: list
    sigma_e: float = 0.26
    bias: object = 1.0
    m: float = 0.0
    ia: object = None

    @property
    def n_tracers(self):
        return len(self.bins)

    @property
    def zmax(self):
        return max(b.zmax for b in self.bins)

    def noise(self):
        ng = _t([b.gals_per_steradian for b in self.bins])
        if self.kind == "wl":
            return self.sigma_e**2 / ng
        return 1.0 / ng


def weak_lensing_kernel(c, pzs, z, ell):
    """probes.py:16-74 -> [n_bins, len(z)]."""
    z = torch.atleast_1d(z)
    rk = _wl_radial(c, pzs, z)
    constant_factor = 3.0 * H0**2 * c.Omega_m / 2.0 / C_KMS
    ell = _t(ell)
    ell_factor = torch.sqrt((ell - 1) * (ell) * (ell + 1) * (ell + 2)) / (ell + 0.5) ** 2
    return constant_factor * ell_factor * rk


def _mult(probe):
    """1 + m, m a number or one value per bin (probes.py:204-207)."""
    if isinstance(probe.m, (list, tuple)):
        return 1.0 + _t(np.asarray(probe.m, dtype=np.float64))[..., None]
    return 1.0 + probe.m


def bias_eval(c, spec, z):
    """b(cosmo, z) of one bias model (bias.py:10-57)."""
    if not isinstance(spec, tuple):
        spec = ("const", spec)
    if spec[0] == "const":  # bias.py:21-22
        return spec[1] * torch.ones_like(z)
    if spec[0] == "invg":  # bias.py:38-39
        return spec[1] / growth_factor(c, z2a(z))
    if spec[0] == "desy1":  # bias.py:56-57
        A, eta, z0 = spec[1:]
        return A * ((1.0 + z) / (1.0 + z0)) ** eta
    raise ValueError(spec)


def _bias_stack(c, bias, z, n):
    """probes.py:89-93 / 113-117: a list gives one bias per bin."""
    if isinstance(bias, list):
        return torch.stack([bias_eval(c, b, z) for b in bias], dim=0)
    return bias_eval(c, bias, z)


def density_kernel(c, pzs, bias, z):
    """probes.py:77-99"""
    dndz = torch.stack([pz(z) for pz in pzs], dim=0)
    b = _bias_stack(c, bias, z, len(pzs))
    return 1.0 * 1.0 * (dndz * b * H(c, z2a(z)))


def nla_radial(c, pzs, bias, z):
    """The ell-independent part of nla_kernel (probes.py:102-129)."""
    dndz = torch.stack([pz(z) for pz in pzs], dim=0)
    b = _bias_stack(c, bias, z, len(pzs))
    rk = dndz * b * H(c, z2a(z))
    return rk * (-(5e-14 * RHOCRIT) * c.Omega_m / growth_factor(c, z2a(z)))


def probe_kernel(c, probe, z, ell):
    """probes.py:188-208 / 260-272."""
    if probe.kind == "wl":
        k = weak_lensing_kernel(c, probe.bins, z, ell)
        if probe.ia is not None:
            ell_t = _t(ell)
            ef = torch.sqrt((ell_t - 1) * (ell_t) * (ell_t + 1) * (ell_t + 2)) / (ell_t + 0.5) ** 2
            k = k + 1.0 * ef * nla_radial(c, probe.bins, probe.ia, torch.atleast_1d(z))
        return k * _mult(probe)
    return density_kernel(c, probe.bins, probe.bias, z)


def _wl_radial(c, pzs, z):
    """The ell-independent part of probes.py:24-68 (radial_kernel): Simpson
    over z' in [z, zmax] for extended bins, the single-plane ratio at z0 for
    delta_nz bins (probes.py:53-64), in the bins' order."""
    zmax = max(pz.zmax for pz in pzs)
    chi = radial_comoving_distance(c, z2a(z))
    ext = [i for i, pz in enumerate(pzs) if not isinstance(pz, Delta)]
    out = [None] * len(pzs)
    if ext:
        zp = _t(np.linspace(z.detach().numpy(), zmax, 257))
        dx = (zmax - z) / 256
        chi_p = radial_comoving_distance(c, z2a(zp.reshape(-1))).reshape(zp.shape)
        dndz = torch.stack([pzs[i](zp) for i in ext], dim=1)
        integ = dndz * (clip(chi_p - chi[None, :], 0.0) / clip(chi_p, 1.0))[:, None, :]
        rk = simps_weights_apply(integ, dx) * (1.0 + z) * chi
        for j, i in enumerate(ext):
            out[i] = rk[j]
    for i, pz in enumerate(pzs):
        if isinstance(pz, Delta):
            chi0 = radial_comoving_distance(c, z2a(_t([pz.z0])))
            out[i] = clip(chi0 - chi, 0.0) / clip(chi0, 1.0) * (1.0 + z) * chi
    return torch.stack(out, dim=0)


def probe_kernels_all_ell(c, probe, z, ell):
    """probe_kernel for every ell at once -> [n_ell, n_bins, len(z)].

    The radial part is computed once; the ell factor is applied with the same
    operation order as probes.py:71-74, 207.
    """
    ell = _t(ell).reshape(-1)
    if probe.kind == "wl":
        rk = _wl_radial(c, probe.bins, z)
        constant_factor = 3.0 * H0**2 * c.Omega_m / 2.0 / C_KMS
        ef = torch.sqrt((ell - 1) * (ell) * (ell + 1) * (ell + 2)) / (ell + 0.5) ** 2
        k = (constant_factor * ef)[:, None, None] * rk[None]
        if probe.ia is not None:
            k = k + (1.0 * ef)[:, None, None] * nla_radial(c, probe.bins, probe.ia, z)[None]
        return k * _mult(probe)
    k = density_kernel(c, probe.bins, probe.bias, z)
    return k[None].expand(ell.shape[0], -1, -1)


# -------------------------------------------------------------- angular_cl ----
def cl_ordering(n_tracers):
    """angular_cl.py:15-25"""
    return [(i, j) for i in range(n_tracers) for j in range(i, n_tracers)]


def cov_blocks_ordering(n_tracers):
    """angular_cl.py:28-46"""
    idx = cl_ordering(n_tracers)
    pos = {p: n for n, p in enumerate(idx)}

    def find(a, b):
        return pos[(a, b)] if (a, b) in pos else pos[(b, a)]

    return [
        (find(i, m), find(j, n), find(i, n), find(j, m)) for i, j in idx for m, n in idx
    ]


def limber_nodes(zmax, n_limber=512):
    """The scale-factor nodes of angular_cl.py:96: linspace(z2a(zmax), 1, N+1)."""
    a0 = 1.0 / (1.0 + zmax)
    return np.linspace(a0, 1.0, n_limber + 1), (1.0 - a0) / n_limber


def halofit_nodes(c, k, a, nonlinear="takahashi2012"):
    """nonlinear_fn (power.py:144-262 halofit with prescription ``nonlinear``, or
    linear_matter_power for nonlinear="linear") on a [n_ell, n_a] grid of k
    with a per column."""
    a = torch.atleast_1d(a)
    g = growth_factor(c, a)
    t = eisenstein_hu(c, k)
    pknorm = c.sigma8**2 / sigmasqr(c, 8.0)
    pklin = primordial_matter_power(c, k) * t**2 * g**2
    pklin = pklin * pknorm
    if nonlinear == "linear":
        return pklin
    k_nl, n, C = halofit_parameters(c, a)
    coefs = halofit_coefs(n, C, Omega_m_a(c, a), Omega_de_a(c, a), w(c, a), nonlinear)
    return _halofit_from(k, pklin, k_nl, coefs)


def angular_cl(c, ell, probes, n_limber=512, nonlinear="takahashi2012"):
    """angular_cl.py:49-98 -> [n_cls, n_ell]; nonlinear: the halofit
    prescription of nonlinear_fn, or "linear" for linear_matter_power.

    The reference evaluates the integrand once per ell (vmap); ell-independent
    intermediates (tables, halofit parameters, radial kernels) give identical
    values for every ell, so they are computed once here and the integrand is
    evaluated on the whole [n_ell, n_a] grid.
    """
    ell = _t(ell).reshape(-1)
    zmax = max(p.zmax for p in probes)
    a_np, _ = limber_nodes(zmax, n_limber)
    a = _t(a_np)
    dx = (1.0 - z2a(zmax)) / n_limber
    chi = radial_comoving_distance(c, a)
    z = a2z(a)
    k = (ell[:, None] + 0.5) / clip(chi, 1.0)[None, :]
    pk = halofit_nodes(c, k, a, nonlinear)  # [n_ell, n_a]
    kern = torch.cat([probe_kernels_all_ell(c, p, z, ell) for p in probes], dim=1)
    pairs = cl_ordering(kern.shape[1])
    ii = torch.tensor([p[0] for p in pairs])
    jj = torch.tensor([p[1] for p in pairs])
    kk = kern[:, ii] * kern[:, jj]  # [n_ell, n_cls, n_a]
    res = pk[:, None, :] * kk * dchioverda(c, a) / clip(chi**2, 1.0)
    cl = simps_weights_apply(res.permute(2, 1, 0), dx) / C_KMS**2  # [n_cls, n_ell]
    return cl


def noise_cl(ell, probes):
    """angular_cl.py:101-117"""
    n_ell = len(ell)
    noise = torch.cat([p.noise() for p in probes])
    rows = []
    for i, j in cl_ordering(noise.shape[0]):
        delta = 1.0 - min(abs(i - j), 1)
        rows.append(noise[i] * delta * torch.ones(n_ell, dtype=DT))
    return torch.stack(rows)


def gaussian_cl_covariance(ell, n_tracers, cl_signal, cl_noise, f_sky=0.25, sparse=True):
    """angular_cl.py:120-163"""
    ell_np = np.atleast_1d(np.asarray(ell, dtype=np.float64))
    n_ell = len(ell_np)
    cl_obs = cl_signal + cl_noise
    n_cls = cl_obs.shape[0]
    norm = _t((2 * ell_np + 1) * np.gradient(ell_np) * f_sky)
    blocks = cov_blocks_ordering(n_tracers)
    ia = torch.tensor([b[0] for b in blocks])
    ib = torch.tensor([b[1] for b in blocks])
    ic = torch.tensor([b[2] for b in blocks])
    id_ = torch.tensor([b[3] for b in blocks])
    cov = (cl_obs[ia] * cl_obs[ib] + cl_obs[ic] * cl_obs[id_]) / norm
    cov = cov.reshape(n_cls, n_cls, n_ell)
    if sparse:
        return cov
    return to_dense(cov)


def gaussian_cl_covariance_and_mean(c, ell, probes, f_sky=0.25, sparse=False, n_limber=512,
                                    nonlinear="takahashi2012"):
    """angular_cl.py:166-196"""
    cl_signal = angular_cl(c, ell, probes, n_limber=n_limber, nonlinear=nonlinear)
    cl_noise = noise_cl(np.atleast_1d(ell), probes)
    n_tr = sum(p.n_tracers for p in probes)
    cov = gaussian_cl_covariance(ell, n_tr, cl_signal, cl_noise, f_sky, sparse)
    return cl_signal.flatten(), cov


# ------------------------------------------------------------------ sparse ----
def to_dense(sp):
    """sparse.py:52-68: (n, m, d) block diagonals -> (n d, m d)."""
    n, m, d = sp.shape
    eye = torch.eye(d, dtype=sp.dtype)
    return (sp[:, :, None, :] * eye[None, None]).permute(0, 2, 1, 3).reshape(n * d, m * d)


def sparse_inv(sp):
    """sparse.py:295-315: per-diagonal inverse."""
    return torch.linalg.inv(sp.permute(2, 0, 1)).permute(1, 2, 0)


def sparse_slogdet(sp):
    """sparse.py:322-366: Schur-complement log-determinant (eq. 2.2 of 1112.4379)."""
    N, _, P = sp.shape
    sign = torch.prod(torch.sign(sp[-1, -1]))
    logdet = torch.sum(torch.log(torch.abs(sp[-1, -1])))
    for k in range(N - 1):
        u = sp[k : k + 1, k + 1 : N]
        S = sp[k + 1 : N, k + 1 : N]
        v = sp[k + 1 : N, k : k + 1]
        Sinv_v = torch.einsum("ijl,jkl->ikl", sparse_inv(S), v)
        M = sp[k, k] - torch.einsum("ijl,jkl->ikl", u, Sinv_v)[0, 0]
        sign = sign * torch.prod(torch.sign(M))
        logdet = logdet + torch.sum(torch.log(torch.abs(M)))
    return sign, logdet


def sparse_dot_vec(sp, v):
    """sparse.py: A @ v with A sparse (n, m, d), v of length m d."""
    n, m, d = sp.shape
    return torch.einsum("ijl,jl->il", sp, v.reshape(m, d)).reshape(n * d)


def gaussian_log_likelihood(data, mu, C, include_logdet=True, inverse_method="inverse"):
    """likelihood.py:9-61 (note the +0.5 logdet of likelihood.py:61)."""
    r = mu - data
    if C.dim() == 3:
        rT_Cinv_r = torch.dot(r, sparse_dot_vec(sparse_inv(C), r))
    else:
        if inverse_method == "inverse":
            y = torch.linalg.inv(C) @ r
        elif inverse_method == "cholesky":
            L = torch.linalg.cholesky(C)
            y = torch.cholesky_solve(r[:, None], L)[:, 0]
        else:
            raise NotImplementedError
        rT_Cinv_r = torch.dot(r, y)
    if not include_logdet:
        return -0.5 * rT_Cinv_r
    if C.dim() == 3:
        _, logdet = sparse_slogdet(C)
    else:
        _, logdet = torch.linalg.slogdet(C)
    return -0.5 * (rT_Cinv_r - logdet)
