"""Host stand-ins that let dLux's own, unmodified modules run under NumPy.

dLux is pure Python on JAX, Equinox and Zodiax, none of which can be installed
in this image. The golden-fixture generator (make_ref_golden.py) puts the small
modules below into ``sys.modules`` under those names and then imports dLux
from its source tree without executing ``dLux/__init__.py`` (which asks
importlib.metadata for an installed version). dLux's arithmetic then runs on
NumPy in float64/complex128, i.e. as dLux runs with ``jax_enable_x64``.

What the stand-ins provide, and nothing more:
  * ``jax.numpy``: NumPy, with every array it returns viewed as ``JArray``,
    an ndarray whose augmented assignments (``x /= y``) bind a new array
    instead of writing in place -- JAX arrays are immutable, and dLux's code
    relies on that (e.g. ``shift /= pixel_scale_out`` in its MFT);
  * ``jax.vmap`` / ``equinox.filter_vmap``: a loop over the mapped axis whose
    outputs (arrays or module trees) are stacked leaf by leaf;
  * ``jax.lax``: pow, cond, switch, reduce, bitwise_or, exp, lgamma;
  * ``jax.tree``: map / flatten / leaves over lists, tuples, dicts and modules;
  * ``jax.scipy``: the SciPy functions of the same names;
  * ``equinox``: Module, field (static fields become plain attributes),
    filter_jit (identity), filter_vmap, partition;
  * ``zodiax.Base``: get / set / add / subtract / multiply / divide / power by
    attribute path, returning
    shallow copies, as zodiax does for its immutable modules;
  * ``abcdLux`` and ``interpax``: empty modules (dLux imports them at module
    level; the paths fixtures are made for never call into them).

Only the fixture generator imports this file, and only in a container that
holds dLux's source tree.
"""

from __future__ import annotations

import functools
import importlib
import os
import sys
import types

import numpy as np
import scipy.signal
import scipy.special
import scipy.stats


# ----------------------------------------------------------------------------
# Arrays with JAX's value semantics
# ----------------------------------------------------------------------------
class JArray(np.ndarray):
    """ndarray whose augmented assignments rebind instead of mutating."""

    def __iadd__(self, o):
        return np.add(self, o)

    def __isub__(self, o):
        return np.subtract(self, o)

    def __imul__(self, o):
        return np.multiply(self, o)

    def __itruediv__(self, o):
        return np.true_divide(self, o)

    def __ifloordiv__(self, o):
        return np.floor_divide(self, o)

    def __imod__(self, o):
        return np.mod(self, o)

    def __ipow__(self, o):
        return np.power(self, o)

    def __imatmul__(self, o):
        return np.matmul(self, o)

    def __iand__(self, o):
        return np.bitwise_and(self, o)

    def __ior__(self, o):
        return np.bitwise_or(self, o)

    def __ixor__(self, o):
        return np.bitwise_xor(self, o)


def J(x):
    """View every ndarray in x (arrays, tuples, lists) as a JArray."""
    if type(x) is np.ndarray:
        return x.view(JArray)
    if isinstance(x, tuple):
        return tuple(J(v) for v in x)
    if isinstance(x, list):
        return [J(v) for v in x]
    return x


def _wrap_fn(fn):
    @functools.wraps(fn)
    def wrapped(*args, **kwargs):
        return J(fn(*args, **kwargs))
    return wrapped


class _UfuncProxy:
    def __init__(self, uf):
        self._uf = uf

    def __call__(self, *args, **kwargs):
        return J(self._uf(*args, **kwargs))

    def __getattr__(self, name):
        attr = getattr(self._uf, name)
        return _wrap_fn(attr) if callable(attr) else attr


def _wrapped_namespace(name, src):
    m = types.ModuleType(name)
    for k in dir(src):
        if k.startswith("__"):
            continue
        v = getattr(src, k)
        if isinstance(v, np.ufunc):
            v = _UfuncProxy(v)
        elif callable(v) and not isinstance(v, type):
            v = _wrap_fn(v)
        setattr(m, k, v)
    return m


# ----------------------------------------------------------------------------
# Trees: modules are nodes whose children are their instance attributes.
# ----------------------------------------------------------------------------
class Module:
    """Stand-in for equinox.Module: a plain object whose attributes are its fields."""


def _shallow(obj):
    """A copy of a module sharing its fields (no __getattr__ lookups on the way)."""
    new = object.__new__(type(obj))
    new.__dict__.update(obj.__dict__)
    return new


def _is_node(x):
    return isinstance(x, (list, tuple, dict, Module)) or x is None


def _children(x):
    if x is None:
        return [], None
    if isinstance(x, dict):
        keys = list(x.keys())
        return [x[k] for k in keys], ("dict", type(x), keys)
    if isinstance(x, (list, tuple)):
        return list(x), ("seq", type(x), len(x))
    keys = list(vars(x).keys())
    return [getattr(x, k) for k in keys], ("mod", x, keys)


def _rebuild(meta, kids):
    if meta is None:
        return None
    kind, t, keys = meta
    if kind == "dict":
        out = t()
        for k, v in zip(keys, kids):
            out[k] = v
        return out
    if kind == "seq":
        return t(kids)
    new = _shallow(t)
    for k, v in zip(keys, kids):
        object.__setattr__(new, k, v)
    return new


def tree_flatten(tree, is_leaf=None):
    leaves = []

    def rec(x):
        if (is_leaf is not None and is_leaf(x)) or not _is_node(x):
            leaves.append(x)
            return ("leaf",)
        kids, meta = _children(x)
        return ("node", meta, [rec(k) for k in kids])

    return leaves, rec(tree)


def tree_unflatten(treedef, leaves):
    it = iter(leaves)

    def rec(d):
        if d[0] == "leaf":
            return next(it)
        return _rebuild(d[1], [rec(k) for k in d[2]])

    return rec(treedef)


def tree_leaves(tree, is_leaf=None):
    return tree_flatten(tree, is_leaf)[0]


def tree_map(fn, tree, *rest, is_leaf=None):
    leaves, treedef = tree_flatten(tree, is_leaf)
    others = [tree_flatten(r, is_leaf)[0] for r in rest]
    return tree_unflatten(treedef, [fn(*xs) for xs in zip(leaves, *others)])


# ----------------------------------------------------------------------------
# vmap: loop and stack
# ----------------------------------------------------------------------------
def _take(x, i, axis):
    if axis is None:
        return x
    return tree_map(lambda a: J(np.take(np.asarray(a), i, axis=axis))
                    if isinstance(a, np.ndarray) else a, x)


def _stack(outs):
    first = outs[0]
    leaves0, treedef = tree_flatten(first)
    all_leaves = [tree_flatten(o)[0] for o in outs]
    stacked = []
    for j, leaf in enumerate(leaves0):
        col = [ls[j] for ls in all_leaves]
        if isinstance(leaf, (np.ndarray, float, int, complex, np.generic)) and \
                not isinstance(leaf, bool):
            stacked.append(J(np.stack([np.asarray(c) for c in col])))
        else:
            stacked.append(leaf)  # static field: the same in every call
    return tree_unflatten(treedef, stacked)


def vmap(fn, in_axes=0, out_axes=0):
    if out_axes != 0:
        raise NotImplementedError("stand-in vmap maps outputs along axis 0 only")

    def wrapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is None:
                continue
            for leaf in tree_leaves(a):
                if isinstance(leaf, np.ndarray) and leaf.ndim > ax:
                    n = leaf.shape[ax]
                    break
            if n is not None:
                break
        if n is None:
            raise ValueError("stand-in vmap: no mapped array argument")
        outs = [fn(*[_take(a, i, ax) for a, ax in zip(args, axes)]) for i in range(n)]
        return _stack(outs)

    return wrapped


def filter_vmap(fn=None, **kw):
    if fn is None:
        return lambda f: filter_vmap(f, **kw)

    def wrapped(*args):
        axes = tuple(0 if any(isinstance(leaf, np.ndarray) for leaf in tree_leaves(a)) else None
                     for a in args)
        return vmap(fn, in_axes=axes)(*args)

    return wrapped


def filter_jit(fn=None, **kw):
    if fn is None:
        return lambda f: f
    return fn


def field(**kw):
    return kw.get("default", None)


def partition(tree, filter_spec, is_leaf=None):
    spec = tree_flatten(filter_spec, is_leaf)[0]
    leaves, treedef = tree_flatten(tree, is_leaf)
    keep = [leaf if s else None for leaf, s in zip(leaves, spec)]
    drop = [None if s else leaf for leaf, s in zip(leaves, spec)]
    return tree_unflatten(treedef, keep), tree_unflatten(treedef, drop)


# ----------------------------------------------------------------------------
# zodiax.Base
# ----------------------------------------------------------------------------
class Base(Module):
    """Stand-in for zodiax.Base: path-addressed get/set on an immutable module."""

    def get(self, path):
        obj = self
        for key in str(path).split("."):
            obj = obj[key] if isinstance(obj, dict) else getattr(obj, key)
        return obj

    def _set_path(self, keys, value):
        key = keys[0]
        if isinstance(self, dict):
            new = type(self)(self)
            child = self[key]
        else:
            new = _shallow(self)
            child = getattr(self, key)
        if len(keys) > 1:
            value = Base._set_path(child, keys[1:], value)
        if isinstance(new, dict):
            new[key] = value
        else:
            object.__setattr__(new, key, value)
        return new

    def set(self, parameters=None, values=None, **kwargs):
        pairs = []
        if parameters is not None:
            if isinstance(parameters, (list, tuple)):
                pairs += list(zip(parameters, values))
            else:
                pairs.append((parameters, values))
        pairs += list(kwargs.items())
        new = self
        for path, value in pairs:
            new = Base._set_path(new, str(path).split("."), value)
        return new

    def add(self, path, value):
        return self.set(path, self.get(path) + value)

    def multiply(self, path, value):
        return self.set(path, self.get(path) * value)

    def divide(self, path, value):
        return self.set(path, self.get(path) / value)

    def subtract(self, path, value):
        return self.set(path, self.get(path) - value)

    def power(self, path, value):
        return self.set(path, self.get(path) ** value)


# ----------------------------------------------------------------------------
# Module objects
# ----------------------------------------------------------------------------
def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    return m


def _lax_reduce(operands, init, computation, dimensions):
    arr = np.asarray(operands)
    if tuple(dimensions) != (0,):
        raise NotImplementedError("stand-in lax.reduce reduces axis 0 only")
    return functools.reduce(computation, list(arr), np.asarray(init))


def install():
    """Put the stand-ins into sys.modules (idempotent)."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_dlux_standin", False):
        return
    jnp = _wrapped_namespace("jax.numpy", np)
    jnp.fft = _wrapped_namespace("jax.numpy.fft", np.fft)
    jnp.linalg = _wrapped_namespace("jax.numpy.linalg", np.linalg)
    lax = _module(
        "jax.lax",
        pow=lambda x, y: np.power(np.asarray(x, float), y),
        integer_pow=lambda x, n: np.asarray(x) ** n,
        cond=lambda pred, tf, ff, *ops: tf(*ops) if bool(pred) else ff(*ops),
        switch=lambda index, branches, *ops: branches[int(index)](*ops),
        reduce=_lax_reduce,
        bitwise_or=np.bitwise_or,
        exp=np.exp,
        lgamma=scipy.special.gammaln,
    )
    tree = _module("jax.tree", map=tree_map, flatten=tree_flatten, leaves=tree_leaves,
                   unflatten=tree_unflatten)
    jsp = _module("jax.scipy",
                  stats=_module("jax.scipy.stats", norm=scipy.stats.norm,
                                multivariate_normal=scipy.stats.multivariate_normal),
                  special=scipy.special,
                  signal=_module("jax.scipy.signal", convolve=scipy.signal.convolve))
    jax = _module("jax", numpy=jnp, lax=lax, tree=tree, scipy=jsp, vmap=vmap,
                  Array=np.ndarray, jit=filter_jit, _dlux_standin=True)
    eqx = _module("equinox", Module=Module, field=field, filter_jit=filter_jit,
                  filter_vmap=filter_vmap, partition=partition)
    zdx = _module("zodiax", Base=Base)
    abcd = _module("abcdLux", abcd=_module("abcdLux.abcd"), lct=_module("abcdLux.lct"),
                   asm=_module("abcdLux.asm"), mft=_module("abcdLux.mft", mft_kernels=None))
    ipx = _module("interpax")
    mods = {"jax": jax, "jax.numpy": jnp, "jax.numpy.fft": jnp.fft,
            "jax.numpy.linalg": jnp.linalg, "jax.lax": lax, "jax.tree": tree,
            "jax.scipy": jsp, "jax.scipy.stats": jsp.stats, "jax.scipy.special": jsp.special,
            "jax.scipy.signal": jsp.signal, "equinox": eqx, "zodiax": zdx, "abcdLux": abcd,
            "abcdLux.abcd": abcd.abcd, "abcdLux.lct": abcd.lct, "abcdLux.asm": abcd.asm,
            "abcdLux.mft": abcd.mft, "interpax": ipx}
    sys.modules.update(mods)


def load_dlux(src_root):
    """Import dLux from ``src_root`` (the directory that contains ``dLux/``)
    under the stand-ins; returns the package with its submodules attached."""
    install()
    if "dLux" not in sys.modules:
        pkg = types.ModuleType("dLux")
        pkg.__path__ = [os.path.join(src_root, "dLux")]
        pkg.__package__ = "dLux"
        sys.modules["dLux"] = pkg
    pkg = sys.modules["dLux"]
    for name in ("utils", "coordinates", "psfs", "wavefronts", "parametric", "polynomials",
                 "layers", "spectra", "sources", "optical_systems", "detectors",
                 "instruments"):
        setattr(pkg, name, importlib.import_module(f"dLux.{name}"))
    return pkg
