"""NumPy stand-in for the parts of JAX that soundersim's kernel modules use.

Test infrastructure only: it lets the UNMODIFIED reference source
(``soundersim/kernels/coherent.py``, ``kernels/multilayer.py``,
``roughness.py``, ``refraction.py``, ``refraction_joint.py``, ``antenna.py``,
``kernels/geometry.py``) execute on the CPU in this container, where JAX is
not installed, so that ``make_golden.py`` can freeze the reference's own
outputs as fixtures. Semantics follow NumPy (NEP 50 promotion): float32
inputs stay float32, float64 stays float64, which mirrors JAX's
``enable_x64`` / default-f32 split closely enough for the tolerances the
fixtures are used with. ``jit`` is the identity, ``vmap`` a Python loop plus
stack, ``lax.scan``/``fori_loop`` plain loops, ``segment_sum`` an
``np.add.at``.
"""

import contextlib
import sys
import types

import numpy as np
import scipy.special


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        arr = self._arr

        class _Set:
            def set(self_inner, value):
                out = np.array(arr, copy=True).view(_Arr)
                out[idx] = value
                return out

        return _Set()


class _Arr(np.ndarray):
    """ndarray with JAX's functional ``.at[idx].set(v)`` update."""

    @property
    def at(self):
        return _AtIndexer(self)


def _tree_map(fn, *trees):
    t0 = trees[0]
    if t0 is None:
        return None
    if isinstance(t0, (tuple, list)):
        out = [_tree_map(fn, *[t[i] for t in trees]) for i in range(len(t0))]
        if hasattr(t0, "_fields"):
            return type(t0)(*out)
        return type(t0)(out)
    return fn(*trees)


def _stack_tree(items):
    if items[0] is None:
        return None
    if isinstance(items[0], (tuple, list)):
        out = [_stack_tree([it[i] for it in items])
               for i in range(len(items[0]))]
        if hasattr(items[0], "_fields"):
            return type(items[0])(*out)
        return type(items[0])(out)
    return np.stack([np.asarray(x) for x in items])


def _index_tree(tree, i):
    return _tree_map(lambda a: np.asarray(a)[i], tree)


def _tree_len(tree):
    if isinstance(tree, (tuple, list)):
        for t in tree:
            n = _tree_len(t)
            if n is not None:
                return n
        return None
    if tree is None:
        return None
    return np.asarray(tree).shape[0]


def jit(fn=None, **_kw):
    if fn is None:
        return lambda f: f
    return fn


def vmap(fn, in_axes=0, **_kw):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (
            (in_axes,) * len(args))
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _tree_len(a)
                break
        outs = []
        for i in range(n):
            sl = [(_index_tree(a, i) if ax is not None else a)
                  for a, ax in zip(args, axes)]
            outs.append(fn(*sl))
        return _stack_tree(outs)
    return mapped


@contextlib.contextmanager
def enable_x64(*_a, **_k):
    yield


# --- jax.lax -------------------------------------------------------------
lax = types.ModuleType("jax.lax")


def _scan(f, init, xs=None, length=None, reverse=False, **_kw):
    n = length if xs is None else _tree_len(xs)
    idx = range(n - 1, -1, -1) if reverse else range(n)
    carry = init
    ys = [None] * n
    for i in idx:
        x = None if xs is None else _index_tree(xs, i)
        carry, y = f(carry, x)
        ys[i] = y
    if n == 0 or ys[0] is None:
        return carry, None
    return carry, _stack_tree(ys)


def _fori_loop(lo, hi, body, init):
    val = init
    for i in range(lo, hi):
        val = body(i, val)
    return val


def _rsqrt(x):
    return 1.0 / np.sqrt(x)


def _dynamic_index_in_dim(x, index, axis=0, keepdims=True):
    x = np.asarray(x)
    out = np.take(x, int(index), axis=axis)
    if keepdims:
        out = np.expand_dims(out, axis)
    return out


lax.scan = _scan
lax.fori_loop = _fori_loop
lax.rsqrt = _rsqrt
lax.dynamic_index_in_dim = _dynamic_index_in_dim

# --- jax.ops ---------------------------------------------------------------
ops = types.ModuleType("jax.ops")


def _segment_sum(data, segment_ids, num_segments):
    data = np.asarray(data)
    out = np.zeros((num_segments,) + data.shape[1:], data.dtype)
    np.add.at(out, np.asarray(segment_ids), data)
    return out


ops.segment_sum = _segment_sum

# --- jax.numpy -------------------------------------------------------------
jnp = types.ModuleType("jax.numpy")
for _name in dir(np):
    if not _name.startswith("_"):
        setattr(jnp, _name, getattr(np, _name))


def _zeros_like(a, dtype=None):
    return np.zeros_like(np.asarray(a), dtype=dtype).view(_Arr)


jnp.zeros_like = _zeros_like
jnp.asarray = lambda a, dtype=None: np.asarray(a, dtype=dtype)
jnp.linalg = np.linalg

# --- jax.scipy.special -----------------------------------------------------
jscipy = types.ModuleType("jax.scipy")
jspecial = types.ModuleType("jax.scipy.special")
jspecial.gammaln = scipy.special.gammaln
jscipy.special = jspecial

# --- the package -----------------------------------------------------------
jax = types.ModuleType("jax")
jax.jit = jit
jax.vmap = vmap
jax.enable_x64 = enable_x64
jax.lax = lax
jax.ops = ops
jax.numpy = jnp
jax.scipy = jscipy


def install():
    """Register the stand-in as ``jax`` (and its submodules) in sys.modules."""
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.lax"] = lax
    sys.modules["jax.ops"] = ops
    sys.modules["jax.scipy"] = jscipy
    sys.modules["jax.scipy.special"] = jspecial
