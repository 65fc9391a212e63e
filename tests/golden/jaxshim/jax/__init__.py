"""A NumPy stand-in for the small part of JAX that jqmc's per-walker functions use.

Used only by tests/golden/make_golden.py to execute the reference's own Python
functions in a container where JAX is not installed.  Tracing, autodiff and
device placement are absent: ``jit`` is the identity, ``vmap`` loops in Python,
``lax`` control flow runs eagerly, and the autodiff entry points raise when
called.  ``jax.numpy`` is NumPy with float64 defaults.
"""
import types as _types

import numpy as _np

from . import numpy, lax, scipy, random, tree_util, typing, nn, ops  # noqa: F401

Array = _np.ndarray


class _Config:
    def update(self, *a, **k):
        pass


config = _Config()


def jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _take(x, axis, i):
    if axis is None:
        return x
    return _np.take(_np.asarray(x), i, axis=axis)


def _stack_out(outs):
    first = outs[0]
    if isinstance(first, tuple):
        return tuple(_stack_out([o[k] for o in outs]) for k in range(len(first)))
    if isinstance(first, list):
        return [_stack_out([o[k] for o in outs]) for k in range(len(first))]
    return _np.stack([_np.asarray(o) for o in outs], axis=0)


def _empty_like_out(o):
    if isinstance(o, tuple):
        return tuple(_empty_like_out(x) for x in o)
    o = _np.asarray(o)
    return _np.zeros((0,) + o.shape, dtype=o.dtype)


def vmap(fun, in_axes=0, out_axes=0, **kwargs):
    def wrapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _np.asarray(a).shape[ax]
                break
        if n == 0:
            dummy = [a if ax is None else _np.zeros(_np.delete(_np.asarray(a).shape, ax), dtype=_np.asarray(a).dtype)
                     for a, ax in zip(args, axes)]
            return _empty_like_out(fun(*dummy))
        outs = [fun(*[_take(a, ax, i) for a, ax in zip(args, axes)]) for i in range(n)]
        return _stack_out(outs)
    return wrapped


def _no_autodiff(*a, **k):
    def f(*args, **kwargs):
        raise NotImplementedError("autodiff is not available in the NumPy stand-in")
    return f


grad = hessian = jacrev = jacfwd = value_and_grad = _no_autodiff


def vjp(*a, **k):
    raise NotImplementedError("autodiff is not available in the NumPy stand-in")


jvp = vjp


class custom_vjp:
    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun

    def defvjp(self, fwd, bwd):
        return None

    def __call__(self, *a, **k):
        return self.fun(*a, **k)


custom_jvp = custom_vjp


def block_until_ready(x):
    return x


def devices():
    return []


debug = _types.SimpleNamespace(print=lambda *a, **k: None)
experimental = _types.SimpleNamespace()
