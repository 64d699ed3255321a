"""NumPy-backed stand-in for the subset of ``jax`` that jax_cosmo imports.

JAX is not installed in this environment and there is no network, so the golden
fixtures are produced by running the *unmodified* jax_cosmo source on top of this
module, in float64 on the CPU.  ``install()`` registers fake ``jax``, ``jax.numpy``,
``jax.lax``, ``jax.tree_util``, ``jax.scipy``, ``jax.scipy.linalg`` and
``jax.experimental.ode`` modules in ``sys.modules``.

Semantics kept from JAX where jax_cosmo depends on them:
  * ``vmap`` maps over the given axes one element at a time and stacks the
    results (``in_axes`` / ``out_axes`` honoured, pytrees of tuples supported).
  * ``jit`` is the identity (with or without ``static_argnums``).
  * ``lax.scan`` / ``lax.map`` / ``lax.switch`` are plain Python loops.
  * ``jnp.clip`` is ``minimum(maximum(x, lo), hi)`` and accepts a missing bound,
    which is what ``jax.numpy.clip`` does (the order matters for the decreasing
    table in the halofit root find, jax_cosmo/scipy/interpolate.py:54).
  * ``argmin`` ties resolve to the first index (same in NumPy and XLA).
Everything is float64 (``jax_enable_x64`` behaviour).

This file is test infrastructure only: it is used by ``make_golden.py`` to
generate the committed ``.npz`` fixtures and never by the library.
"""
import sys
import types

import numpy as _np
import scipy.linalg as _sla


def _clip(a, a_min=None, a_max=None, *args, **kwargs):
    out = _np.asarray(a)
    if a_min is not None:
        out = _np.maximum(out, a_min)
    if a_max is not None:
        out = _np.minimum(out, a_max)
    return out


def _take(x, axis, i):
    return _np.take(_np.asarray(x), i, axis=axis)


def _axis_size(args, in_axes):
    for a, ax in zip(args, in_axes):
        if ax is not None:
            return _np.asarray(a).shape[ax]
    raise ValueError("vmap: no mapped argument")


def _stack_tree(outs, out_axes):
    first = outs[0]
    if isinstance(first, tuple):
        axes = out_axes if isinstance(out_axes, tuple) else (out_axes,) * len(first)
        return tuple(
            _stack_tree([o[k] for o in outs], axes[k]) for k in range(len(first))
        )
    return _np.stack([_np.asarray(o) for o in outs], axis=out_axes)


def vmap(fun=None, in_axes=0, out_axes=0):
    if fun is None:
        return lambda f: vmap(f, in_axes=in_axes, out_axes=out_axes)

    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = _axis_size(args, axes)
        outs = []
        for i in range(n):
            call = [a if ax is None else _take(a, ax, i) for a, ax in zip(args, axes)]
            outs.append(fun(*call))
        return _stack_tree(outs, out_axes)

    return mapped


def jit(fun=None, static_argnums=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _scan(f, init, xs, length=None):
    carry = init
    ys = []
    n = len(xs) if xs is not None else length
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    return carry, _stack_tree(ys, 0) if ys else None


def _lmap(f, xs):
    return _stack_tree([f(x) for x in xs], 0)


def _switch(index, branches, *operands):
    i = int(_np.clip(int(index), 0, len(branches) - 1))
    return branches[i](*operands)


def register_pytree_node_class(cls):
    return cls


def _make_numpy_module():
    jnp = types.ModuleType("jax.numpy")
    for name in dir(_np):
        if not name.startswith("__"):
            setattr(jnp, name, getattr(_np, name))
    jnp.clip = _clip
    jnp.float64 = _np.float64
    jnp.linalg = _np.linalg
    return jnp


def install():
    """Register the stand-in modules; idempotent."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_is_standin", False):
        return sys.modules["jax"]
    jax = types.ModuleType("jax")
    jax._is_standin = True
    jnp = _make_numpy_module()
    lax = types.ModuleType("jax.lax")
    lax.scan = _scan
    lax.map = _lmap
    lax.switch = _switch
    tree_util = types.ModuleType("jax.tree_util")
    tree_util.register_pytree_node_class = register_pytree_node_class
    jscipy = types.ModuleType("jax.scipy")
    jlinalg = types.ModuleType("jax.scipy.linalg")
    jlinalg.cho_factor = _sla.cho_factor
    jlinalg.cho_solve = _sla.cho_solve
    jscipy.linalg = jlinalg
    experimental = types.ModuleType("jax.experimental")
    ode = types.ModuleType("jax.experimental.ode")
    ode.odeint = None
    experimental.ode = ode

    jax.numpy = jnp
    jax.lax = lax
    jax.tree_util = tree_util
    jax.scipy = jscipy
    jax.experimental = experimental
    jax.vmap = vmap
    jax.jit = jit

    sys.modules.update(
        {
            "jax": jax,
            "jax.numpy": jnp,
            "jax.lax": lax,
            "jax.tree_util": tree_util,
            "jax.scipy": jscipy,
            "jax.scipy.linalg": jlinalg,
            "jax.experimental": experimental,
            "jax.experimental.ode": ode,
        }
    )
    return jax
