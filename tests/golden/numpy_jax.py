"""A float64 NumPy stand-in for the few JAX names the reference renderer uses (TEST INFRASTRUCTURE).

JAX is installed on neither machine this project runs on. The reference's pure-JAX renderer
(``baseline/fm_render.py``, ``baseline/util_render.py``) only needs a small slice of JAX:

* ``jax.numpy``: ``triu exp log abs prod diag nan_to_num tile stack array where eye pi``;
* ``jax.lax.map(f, xs, batch_size=...)`` over an array or a ``{0: .., 1: .., 2: ..}`` dict;
* ``jax.vmap(f)(*args)`` (``render_func_idx_quattrans[_flow]``, ``log_likelihood``);
* ``jax.lax.min`` / ``jax.lax.max`` and ``jax.scipy.special.logsumexp``.

``install()`` puts modules with those names into ``sys.modules`` so that the reference files
can be imported unmodified and run in float64 (the ``jax_enable_x64`` semantics).

``lax.map`` and ``vmap`` are evaluated the way ``vmap`` defines them, vectorised: the mapped
function is called once with :class:`Batched` values, arrays whose leading axes are batch axes
(one per active map, ordered by nesting level) and whose trailing axes are what the function
sees. Indexing, ``.T``, ``@``, reductions and ``len``/iteration act on the trailing axes only;
elementwise operations broadcast batch axes by level and the trailing axes NumPy-style. The
``batch_size`` argument of ``lax.map`` only changes how JAX schedules the work, not its result,
so it is accepted and ignored.

Nothing here is specific to the renderer; ``tests/test_oracle.py`` checks the stand-in's map
semantics against plain Python loops.
"""

from __future__ import annotations

import contextlib
import itertools
import sys
import types

import numpy as np

__all__ = ["Batched", "JArray", "install", "installed", "lax_map", "vmap"]

_level_counter = itertools.count(1)


class JArray(np.ndarray):
    """A plain array that can be indexed by a :class:`Batched` integer index (a traced gather,
    as ``rot_mats[pose_idx]`` is under ``vmap``)."""

    def __getitem__(self, key):
        k = key if isinstance(key, tuple) else (key,)
        if any(isinstance(x, Batched) for x in k):
            if not isinstance(k[0], Batched) or any(isinstance(x, Batched) for x in k[1:]):
                raise NotImplementedError("a batched index is supported on the first axis only")
            idx = k[0]
            out = Batched(np.asarray(self)[idx.data], idx.levels)
            return out[k[1:]] if len(k) > 1 else out
        return super().__getitem__(key)


def _j(x):
    """Wrap a plain result as :class:`JArray` (Batched values pass through)."""
    if isinstance(x, Batched):
        return x
    return np.asarray(x, dtype=None).view(JArray) if not np.isscalar(x) else x


def _parts(x):
    """(data, levels) of a Batched or plain value."""
    if isinstance(x, Batched):
        return x.data, x.levels
    return np.asarray(x), ()


def _lift(xs, align_logical=True):
    """Bring values to a common set of batch levels.

    Returns ``(datas, levels)``: each data has one axis per level (size 1 where the value does not
    depend on that level) followed by its own trailing axes, which are left-padded with size-1
    axes to a common rank when ``align_logical`` is set (NumPy broadcasting of the trailing
    axes)."""
    parts = [_parts(x) for x in xs]
    levels = tuple(sorted(set().union(*[set(lv) for _, lv in parts])))
    lnd = max(d.ndim - len(lv) for d, lv in parts)
    out = []
    for d, lv in parts:
        lshape = d.shape[len(lv):]
        shape = [d.shape[lv.index(L)] if L in lv else 1 for L in levels]
        if align_logical:
            shape += [1] * (lnd - len(lshape))
        shape += list(lshape)
        out.append(d.reshape(shape))
    return out, levels


def _wrap(data, levels):
    return Batched(data, levels) if levels else _j(data)


def _elementwise(fn, *xs):
    datas, levels = _lift(xs)
    return _wrap(fn(*datas), levels)


class Batched:
    """A value inside ``vmap``/``lax.map``: leading batch axes (``levels``), trailing axes seen by
    the mapped function."""

    __array_ufunc__ = None        # NumPy operators defer to the reflected methods below

    def __init__(self, data, levels):
        self.data = np.asarray(data)
        self.levels = tuple(levels)
        assert self.data.ndim >= len(self.levels)

    # --- shape -----------------------------------------------------------------------------
    @property
    def nb(self):
        return len(self.levels)

    @property
    def shape(self):
        return self.data.shape[self.nb:]

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def dtype(self):
        return self.data.dtype

    def __len__(self):
        if not self.shape:
            raise TypeError("len() of a scalar")
        return self.shape[0]

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]

    @property
    def T(self):
        nb = self.nb
        axes = list(range(nb)) + list(range(self.data.ndim - 1, nb - 1, -1))
        return Batched(self.data.transpose(axes), self.levels)

    def astype(self, dt):
        if dt is int:
            dt = np.int64
        return Batched(self.data.astype(dt), self.levels)

    # --- indexing --------------------------------------------------------------------------
    def __getitem__(self, key):
        k = key if isinstance(key, tuple) else (key,)
        if any(isinstance(x, Batched) for x in k):
            raise NotImplementedError("indexing a batched value by a batched index")
        return _wrap(self.data[(slice(None),) * self.nb + k], self.levels)

    # --- reductions over the trailing axes ---------------------------------------------------
    def _reduce(self, fn, axis):
        if axis is None:
            axes = tuple(range(self.nb, self.data.ndim))
        else:
            ax = axis if isinstance(axis, tuple) else (axis,)
            axes = tuple(self.nb + (a % self.ndim) for a in ax)
        return _wrap(fn(self.data, axis=axes), self.levels)

    def sum(self, axis=None):
        return self._reduce(np.sum, axis)

    def max(self, axis=None):
        return self._reduce(np.max, axis)

    def min(self, axis=None):
        return self._reduce(np.min, axis)

    def prod(self, axis=None):
        return self._reduce(np.prod, axis)

    def mean(self, axis=None):
        return self._reduce(np.mean, axis)

    def ravel(self):
        return Batched(self.data.reshape(self.data.shape[:self.nb] + (-1,)), self.levels)

    # --- arithmetic ----------------------------------------------------------------------------
    def __add__(self, o): return _elementwise(np.add, self, o)
    def __radd__(self, o): return _elementwise(np.add, o, self)
    def __sub__(self, o): return _elementwise(np.subtract, self, o)
    def __rsub__(self, o): return _elementwise(np.subtract, o, self)
    def __mul__(self, o): return _elementwise(np.multiply, self, o)
    def __rmul__(self, o): return _elementwise(np.multiply, o, self)
    def __truediv__(self, o): return _elementwise(np.true_divide, self, o)
    def __rtruediv__(self, o): return _elementwise(np.true_divide, o, self)
    def __pow__(self, o): return _elementwise(np.power, self, o)
    def __rpow__(self, o): return _elementwise(np.power, o, self)
    def __neg__(self): return Batched(-self.data, self.levels)
    def __abs__(self): return Batched(np.abs(self.data), self.levels)
    def __gt__(self, o): return _elementwise(np.greater, self, o)
    def __ge__(self, o): return _elementwise(np.greater_equal, self, o)
    def __lt__(self, o): return _elementwise(np.less, self, o)
    def __le__(self, o): return _elementwise(np.less_equal, self, o)
    def __matmul__(self, o): return _matmul(self, o)
    def __rmatmul__(self, o): return _matmul(o, self)

    def __bool__(self):
        raise TypeError("the truth value of a batched value depends on the batch")

    def __repr__(self):
        return f"Batched(levels={self.levels}, shape={self.shape}, data_shape={self.data.shape})"


def _matmul(a, b):
    """``a @ b`` on the trailing axes (NumPy matmul rules for 1-D and 2-D operands)."""
    (da, db), levels = _lift((a, b), align_logical=False)
    nb = len(levels)
    ra, rb = da.ndim - nb, db.ndim - nb
    if ra == 2 and rb == 1:
        out = np.matmul(da, db[..., None])[..., 0]
    elif ra == 1 and rb == 2:
        out = np.matmul(da[..., None, :], db)[..., 0, :]
    elif ra == 2 and rb == 2:
        out = np.matmul(da, db)
    elif ra == 1 and rb == 1:
        out = (da * db).sum(-1)
    else:
        raise NotImplementedError(f"matmul of ranks {ra} and {rb}")
    return _wrap(out, levels)


# --- pytrees ---------------------------------------------------------------------------------
def _tree_map(fn, tree):
    if isinstance(tree, dict):
        return {k: _tree_map(fn, v) for k, v in tree.items()}
    if isinstance(tree, (tuple, list)):
        return type(tree)(_tree_map(fn, v) for v in tree)
    if tree is None:
        return None
    return fn(tree)


def _tree_leaves(tree):
    if isinstance(tree, dict):
        return [x for v in tree.values() for x in _tree_leaves(v)]
    if isinstance(tree, (tuple, list)):
        return [x for v in tree for x in _tree_leaves(v)]
    return [] if tree is None else [tree]


def _map_impl(f, args):
    """Evaluate ``f`` mapped over axis 0 of every leaf of ``args`` (a tuple of pytrees)."""
    level = next(_level_counter)
    sizes = {int((x.shape if isinstance(x, Batched) else np.shape(x))[0]) for x in _tree_leaves(args)}
    if len(sizes) != 1:
        raise ValueError(f"mapped axes have different sizes: {sorted(sizes)}")
    n = sizes.pop()

    def enter(x):
        d, lv = _parts(x)
        # the mapped (first trailing) axis becomes the innermost batch axis: no data movement
        return Batched(d, lv + (level,))

    out = f(*_tree_map(enter, args))

    def leave(y):
        d, lv = _parts(y)
        if level in lv:
            assert lv[-1] == level, "the innermost level is the newest"
            return _wrap(d, lv[:-1])
        # a result that does not depend on the mapped value is broadcast along the new axis
        nb = len(lv)
        d = np.broadcast_to(np.expand_dims(d, nb), d.shape[:nb] + (n,) + d.shape[nb:])
        return _wrap(np.array(d), lv)

    return _tree_map(leave, out)


def lax_map(f, xs, batch_size=None):
    """``jax.lax.map``: ``f`` applied to every slice of ``xs`` along axis 0, results stacked."""
    del batch_size   # a scheduling choice in JAX; the result is the same
    return _map_impl(lambda x: f(x), (xs,))


def vmap(f, in_axes=0, out_axes=0):
    """``jax.vmap`` with every input and output mapped along axis 0."""
    if in_axes != 0 or out_axes != 0:
        raise NotImplementedError("only in_axes=0, out_axes=0")

    def g(*args):
        return _map_impl(f, args)

    return g


# --- jax.numpy ---------------------------------------------------------------------------------
def _unary(fn):
    def g(x, *a, **k):
        if isinstance(x, Batched):
            return Batched(fn(x.data, *a, **k), x.levels)
        return _j(fn(np.asarray(x, dtype=np.float64) if not isinstance(x, np.ndarray) else x, *a, **k))
    return g


def _array(obj, dtype=None):
    """``jnp.array`` of nested lists that may hold Batched values (stacked along a new axis 0)."""
    if isinstance(obj, Batched):
        return obj
    if isinstance(obj, (list, tuple)):
        items = [_array(x) for x in obj]
        if any(isinstance(x, Batched) for x in items):
            datas, levels = _lift(items)
            nb = len(levels)
            shape = np.broadcast_shapes(*[d.shape for d in datas])
            datas = [np.broadcast_to(d, shape) for d in datas]
            return Batched(np.stack(datas, axis=nb), levels)
        return _j(np.array([np.asarray(x) for x in items], dtype=dtype or np.float64))
    return _j(np.array(obj, dtype=dtype))


def _where(c, a, b):
    return _elementwise(np.where, c, a, b)


def _diag(x):
    if isinstance(x, Batched):
        return Batched(np.diagonal(x.data, axis1=-2, axis2=-1), x.levels)
    return _j(np.diag(x))


def _prod(x, axis=None):
    if isinstance(x, Batched):
        return x.prod(axis)
    return np.prod(x, axis=axis)


def _sum(x, axis=None):
    if isinstance(x, Batched):
        return x.sum(axis)
    return np.sum(x, axis=axis)


def _logsumexp(a, axis=None):
    """``log(sum(exp(a)))`` along ``axis`` with the max shifted out (scipy's definition)."""
    a = np.asarray(a, dtype=np.float64)
    m = np.max(a, axis=axis, keepdims=True)
    m = np.where(np.isfinite(m), m, 0.0)
    out = np.log(np.sum(np.exp(a - m), axis=axis, keepdims=True)) + m
    return _j(np.squeeze(out, axis=axis) if axis is not None else out.reshape(()))


def _build_modules():
    jnp = types.ModuleType("jax.numpy")
    jnp.float64 = np.float64
    jnp.float32 = np.float32
    jnp.pi = np.pi
    jnp.inf = np.inf
    jnp.array = _array
    jnp.asarray = _array
    jnp.exp = _unary(np.exp)
    jnp.log = _unary(np.log)
    jnp.abs = _unary(np.abs)
    jnp.sqrt = _unary(np.sqrt)
    jnp.triu = lambda x, k=0: _j(np.triu(np.asarray(x), k))
    jnp.nan_to_num = _unary(np.nan_to_num)
    jnp.tile = lambda x, reps: _j(np.tile(np.asarray(x), reps))
    jnp.stack = lambda xs, axis=0: _j(np.stack([np.asarray(x) for x in xs], axis))
    jnp.where = _where
    jnp.eye = lambda n, dtype=None: _j(np.eye(n))
    jnp.diag = _diag
    jnp.prod = _prod
    jnp.sum = _sum
    jnp.minimum = lambda a, b: _elementwise(np.minimum, a, b)
    jnp.maximum = lambda a, b: _elementwise(np.maximum, a, b)

    lax = types.ModuleType("jax.lax")
    lax.map = lax_map
    lax.min = lambda a, b: _elementwise(np.minimum, a, b)
    lax.max = lambda a, b: _elementwise(np.maximum, a, b)

    special = types.ModuleType("jax.scipy.special")
    special.logsumexp = _logsumexp
    jscipy = types.ModuleType("jax.scipy")
    jscipy.special = special

    debug = types.ModuleType("jax.debug")
    debug.print = lambda *a, **k: None

    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.lax = lax
    jax.scipy = jscipy
    jax.vmap = vmap
    jax.debug = debug
    jax.Array = type("Array", (), {})   # nothing is an instance: other libraries probe for it
    jax.__numpy_standin__ = True
    return {"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.scipy": jscipy,
            "jax.scipy.special": special, "jax.debug": debug}


def install():
    """Put the stand-in into ``sys.modules``; returns the previous entries for ``uninstall``."""
    mods = _build_modules()
    saved = {k: sys.modules.get(k) for k in mods}
    sys.modules.update(mods)
    return saved


def uninstall(saved):
    for k, v in saved.items():
        if v is None:
            sys.modules.pop(k, None)
        else:
            sys.modules[k] = v


@contextlib.contextmanager
def installed():
    saved = install()
    try:
        yield sys.modules["jax"]
    finally:
        uninstall(saved)
