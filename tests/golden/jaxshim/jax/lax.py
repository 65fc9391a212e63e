"""jax.lax control flow, run eagerly."""
import numpy as _np


def cond(pred, true_fun, false_fun, *operands, operand=None):
    ops = operands if operands else (operand,)
    return true_fun(*ops) if bool(pred) else false_fun(*ops)


def switch(index, branches, *operands):
    return branches[int(index)](*operands)


def fori_loop(lower, upper, body, init):
    val = init
    for i in range(int(lower), int(upper)):
        val = body(i, val)
    return val


def while_loop(cond_fun, body_fun, init):
    val = init
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def scan(f, init, xs=None, length=None):
    carry = init
    ys = []
    n = length if xs is None else len(xs)
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    return carry, ys


def stop_gradient(x):
    return x


def select(pred, a, b):
    return _np.where(pred, a, b)
