"""Cosmology parameter container (jax_cosmo/core.py:11-198).

Same constructor, properties and pytree leaf order as the reference.  Each
parameter may be a Python float (one cosmology) or a 1-D tensor / array of
length B (a batch of B cosmologies evaluated in one launch); scalars broadcast.
A parameter tensor with ``requires_grad`` makes the angular_cl path
differentiable through libjcg's tangent kernels.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from jax_cosmo_gb300 import _lib

__all__ = ["Cosmology"]

PARAM_NAMES = ("Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa")


class Cosmology:
    def __init__(self, Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa, gamma=None):
        self._Omega_c = Omega_c
        self._Omega_b = Omega_b
        self._h = h
        self._n_s = n_s
        self._sigma8 = sigma8
        self._Omega_k = Omega_k
        self._w0 = w0
        self._wa = wa
        self._flags = {}
        self._gamma = gamma
        self._flags["gamma_growth"] = gamma is not None
        self._workspace = {}

    def __str__(self):
        return (
            "Cosmological parameters: \n"
            + "    h:        " + str(self.h) + " \n"
            + "    Omega_b:  " + str(self.Omega_b) + " \n"
            + "    Omega_c:  " + str(self.Omega_c) + " \n"
            + "    Omega_k:  " + str(self.Omega_k) + " \n"
            + "    w0:       " + str(self.w0) + " \n"
            + "    wa:       " + str(self.wa) + " \n"
            + "    n:        " + str(self.n_s) + " \n"
            + "    sigma8:   " + str(self.sigma8)
        )

    def __repr__(self):
        return self.__str__()

    # pytree leaves in the order of core.py:98-116
    def tree_flatten(self):
        params = (
            self._Omega_c, self._Omega_b, self._h, self._n_s,
            self._sigma8, self._Omega_k, self._w0, self._wa,
        )
        if self._flags["gamma_growth"]:
            params += (self._gamma,)
        return params, self._flags

    @classmethod
    def tree_unflatten(cls, aux_data, children):
        Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa = children[:8]
        gamma = children[8] if aux_data.get("gamma_growth") and len(children) > 8 else None
        return cls(Omega_c=Omega_c, Omega_b=Omega_b, h=h, n_s=n_s, sigma8=sigma8,
                   Omega_k=Omega_k, w0=w0, wa=wa, gamma=gamma)

    # ---------------------------------------------------------------- batch --
    def param_list(self):
        """The 8 parameters, then gamma when the growth is parametrised by it."""
        ps = [getattr(self, "_" + n) for n in PARAM_NAMES]
        if self._flags["gamma_growth"]:
            ps.append(self._gamma)
        return ps

    def physics_bits(self):
        """libjcg physics bits of this cosmology: JCG_GROWTH_GAMMA when gamma is set."""
        return _lib.GROWTH_GAMMA if self._flags["gamma_growth"] else 0

    @property
    def batch_size(self):
        """None for a single cosmology, else the batch length B."""
        b = None
        for v in self.param_list():
            if isinstance(v, (torch.Tensor, np.ndarray)) and np.ndim(v) >= 1:
                n = int(v.shape[0])
                if b is not None and n != b:
                    raise ValueError("Cosmology parameters have inconsistent batch lengths")
                b = n
        return b

    def requires_grad(self):
        return any(isinstance(v, torch.Tensor) and v.requires_grad for v in self.param_list())

    def param_tensor(self, device, differentiable=False):
        """[B, 8] float64 tensor on ``device`` (B = 1 for a single cosmology);
        [B, 9] with gamma last when the growth is parametrised by gamma."""
        B = self.batch_size or 1
        cols = []
        for v in self.param_list():
            if isinstance(v, torch.Tensor):
                t = v.to(device=device, dtype=torch.float64)
                if not differentiable:
                    t = t.detach()
            else:
                t = torch.as_tensor(np.asarray(v, dtype=np.float64), device=device)
            if t.dim() == 0:
                t = t.expand(B)
            cols.append(t.reshape(B))
        p = torch.stack(cols, dim=1).contiguous()
        if p.device.type == "cpu":
            if not bool(torch.isfinite(p.detach()).all()):
                raise ValueError("Cosmology parameters must be finite")
        # device tensors are checked by libjcg's kernels: non-finite parameters
        # give NaN outputs for that cosmology without a host synchronisation
        return p

    # ------------------------------------------------------- reference API --
    @property
    def Omega(self):
        return 1.0 - self._Omega_k

    @property
    def Omega_b(self):
        return self._Omega_b

    @property
    def Omega_c(self):
        return self._Omega_c

    @property
    def Omega_m(self):
        return self._Omega_b + self._Omega_c

    @property
    def Omega_de(self):
        return self.Omega - self.Omega_m

    @property
    def Omega_k(self):
        return self._Omega_k

    @property
    def k(self):
        ok = self._Omega_k
        if isinstance(ok, torch.Tensor):
            return -torch.sign(ok).to(torch.int8)
        return -int(np.sign(ok))

    @property
    def sqrtk(self):
        ok = self._Omega_k
        if isinstance(ok, torch.Tensor):
            return torch.sqrt(torch.abs(ok))
        return math.sqrt(abs(ok))

    @property
    def h(self):
        return self._h

    @property
    def w0(self):
        return self._w0

    @property
    def wa(self):
        return self._wa

    @property
    def n_s(self):
        return self._n_s

    @property
    def sigma8(self):
        return self._sigma8

    @property
    def gamma(self):
        return self._gamma
