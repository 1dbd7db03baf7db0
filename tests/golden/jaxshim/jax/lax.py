"""jax.lax control flow as Python control flow."""
import numpy as np

from ._array import wrap, tree_wrap


def fori_loop(lower, upper, body_fun, init_val, **_):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val


def while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def cond(pred, true_fun, false_fun, *operands, **_):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def switch(index, branches, *operands):
    i = int(np.clip(int(index), 0, len(branches) - 1))
    return branches[i](*operands)


def scan(f, init, xs, length=None, **_):
    carry = init
    ys = []
    n = length if xs is None else len(xs)
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    return carry, (tree_wrap(np.stack(ys)) if ys and ys[0] is not None else None)


def stop_gradient(x):
    return x


def with_sharding_constraint(x, *_a, **_k):
    return x


def slice_in_dim(operand, start_index, limit_index, stride=1, axis=0):
    sl = [slice(None)] * np.ndim(operand)
    sl[axis] = slice(start_index, limit_index, stride)
    return wrap(np.asarray(operand)[tuple(sl)])


def dynamic_slice_in_dim(operand, start_index, slice_size, axis=0):
    return slice_in_dim(operand, int(start_index), int(start_index) + slice_size, 1, axis)


def concatenate(operands, dimension):
    return wrap(np.concatenate(operands, axis=dimension))


def select(pred, on_true, on_false):
    return wrap(np.where(pred, on_true, on_false))
