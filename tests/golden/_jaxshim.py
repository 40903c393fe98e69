"""A numpy stand-in for the small part of the jax API that trot's hot-path
modules touch, so that those modules can be imported and run unmodified on a
machine without jax (fixture generation only; see make_golden.py).

Semantics follow jax with x64 enabled: float64 / complex128 defaults,
``jax.vmap`` as a loop over the mapped axis, ``lax.scan`` / ``lax.map`` as
loops.  Random draws are not reproduced: ``jax.random.normal`` and
``jax.random.uniform`` pop pre-set arrays from ``INJECT`` (fields and SR zeta
are injected, exactly as in the CUDA path's tests).
"""
from __future__ import annotations

import sys
import types
from collections import deque

import numpy as np
import scipy.linalg

INJECT: deque = deque()


def _is_leaf(x):
    return not isinstance(x, (tuple, list, dict)) or x is None


def tree_leaves(tree):
    if tree is None:
        return []
    if isinstance(tree, dict):
        out = []
        for k in sorted(tree):
            out += tree_leaves(tree[k])
        return out
    if isinstance(tree, (tuple, list)):
        out = []
        for t in tree:
            out += tree_leaves(t)
        return out
    return [tree]


def tree_map(f, tree, *rest):
    if tree is None:
        return None
    if isinstance(tree, dict):
        return {k: tree_map(f, tree[k], *[r[k] for r in rest]) for k in tree}
    if isinstance(tree, tuple) and hasattr(tree, "_fields"):
        return type(tree)(*[tree_map(f, t, *[r[i] for r in rest]) for i, t in enumerate(tree)])
    if isinstance(tree, (tuple, list)):
        return type(tree)(tree_map(f, t, *[r[i] for r in rest]) for i, t in enumerate(tree))
    return f(tree, *rest)


def _stack(outs):
    first = outs[0]
    return tree_map(lambda *xs: np.stack([np.asarray(x) for x in xs]), first, *outs[1:])


def vmap(fn, in_axes=0, out_axes=0):
    def wrapped(*args):
        axes = in_axes if isinstance(in_axes, tuple) else (in_axes,) * len(args)
        mapped = [i for i, a in enumerate(axes) if a == 0]
        n = tree_leaves(args[mapped[0]])[0].shape[0]
        outs = []
        for b in range(n):
            call = [tree_map(lambda x: x[b], a) if ax == 0 else a for a, ax in zip(args, axes)]
            outs.append(fn(*call))
        return _stack(outs)

    return wrapped


def _scan(f, init, xs=None, length=None):
    carry = init
    ys = []
    if xs is None:
        for _ in range(length):
            carry, y = f(carry, None)
            ys.append(y)
    else:
        n = tree_leaves(xs)[0].shape[0]
        for i in range(n):
            carry, y = f(carry, tree_map(lambda a: a[i], xs))
            ys.append(y)
    if ys and ys[0] is not None:
        return carry, _stack(ys)
    return carry, None


def _map(f, xs, batch_size=None):
    n = tree_leaves(xs)[0].shape[0]
    return _stack([f(tree_map(lambda a: a[i], xs)) for i in range(n)])


def _split(key, num=2):
    key = np.asarray(key, dtype=np.uint32)
    base = int(key[-1]) * 1000003 + int(key[0])
    return np.array([[base % 2**32, (base + 1 + i) % 2**32] for i in range(num)], dtype=np.uint32)


def _normal(key, shape=(), dtype=np.float64):
    x = np.asarray(INJECT.popleft())
    assert x.shape == tuple(shape), (x.shape, shape)
    return x.astype(dtype)


def _uniform(key, shape=(), dtype=np.float64, minval=0.0, maxval=1.0):
    x = np.asarray(INJECT.popleft(), dtype=dtype)
    assert x.shape == tuple(shape), (x.shape, shape)
    return x


def _array_result(obj):
    """numpy returns numpy scalars (float subclasses) where jax returns 0-d
    arrays; keep array semantics so ``.astype`` etc. work as under jax."""
    if isinstance(obj, type) or not callable(obj):
        return obj

    def f(*a, **k):
        r = obj(*a, **k)
        return np.asarray(r) if isinstance(r, np.generic) else r

    f.__name__ = getattr(obj, "__name__", "f")
    return f


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v):
        out = np.array(self.arr, copy=True).view(JArr)
        out[self.idx] = v
        return out

    def add(self, v):
        out = np.array(self.arr, copy=True).view(JArr)
        out[self.idx] += v
        return out


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


class JArr(np.ndarray):
    """ndarray with jax's functional ``x.at[idx].set(v)`` update syntax."""

    @property
    def at(self):
        return _At(self)


def _jarr(fn):
    def f(*a, **k):
        r = fn(*a, **k)
        return r.view(JArr) if isinstance(r, np.ndarray) else r

    f.__name__ = getattr(fn, "__name__", "f")
    return f


class _Dummy:
    def __init__(self, *a, **k):
        self.args = a
        self.size = 1


def install():
    """Register the stand-in modules under the ``jax`` names."""
    jax = types.ModuleType("jax")
    jnp = types.ModuleType("jax.numpy")
    for k in dir(np):
        if not k.startswith("__"):
            setattr(jnp, k, _array_result(getattr(np, k)))
    jnp.linalg = np.linalg
    jnp.ndarray = np.ndarray
    for name in ("zeros", "zeros_like", "ones", "eye", "array", "asarray", "full"):
        setattr(jnp, name, _jarr(getattr(np, name)))
    lax = types.ModuleType("jax.lax")
    lax.complex = lambda a, b: np.asarray(a) + 1.0j * np.asarray(b)
    lax.scan = _scan
    lax.map = _map
    lax.with_sharding_constraint = lambda x, s: x
    tu = types.ModuleType("jax.tree_util")
    tu.register_pytree_node_class = lambda cls: cls
    tu.tree_map = tree_map
    tu.tree_leaves = tree_leaves
    sh = types.ModuleType("jax.sharding")
    sh.Mesh = _Dummy
    sh.NamedSharding = _Dummy
    sh.PartitionSpec = _Dummy
    ex = types.ModuleType("jax.experimental")
    mu = types.ModuleType("jax.experimental.mesh_utils")
    mu.create_device_mesh = lambda shape: np.zeros(shape)
    ex.mesh_utils = mu
    ex.io_callback = lambda *a, **k: None
    rnd = types.ModuleType("jax.random")
    rnd.PRNGKey = lambda seed: np.array([0, int(seed) % 2**32], dtype=np.uint32)
    rnd.split = _split
    rnd.normal = _normal
    rnd.uniform = _uniform
    sp = types.ModuleType("jax.scipy")
    spl = types.ModuleType("jax.scipy.linalg")
    spl.expm = scipy.linalg.expm
    sp.linalg = spl
    jax.numpy = jnp
    jax.lax = lax
    jax.tree_util = tu
    jax.sharding = sh
    jax.experimental = ex
    jax.random = rnd
    jax.scipy = sp
    jax.vmap = vmap
    jax.Array = np.ndarray
    jax.local_device_count = lambda: 1
    jax.jit = lambda f, *a, **k: f
    mods = {
        "jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.tree_util": tu,
        "jax.sharding": sh, "jax.experimental": ex, "jax.experimental.mesh_utils": mu,
        "jax.random": rnd, "jax.scipy": sp, "jax.scipy.linalg": spl,
    }
    sys.modules.update(mods)
    return jax
