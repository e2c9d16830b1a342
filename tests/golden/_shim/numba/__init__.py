"""Pure-Python stand-in for the subset of numba that the reference imports.

Test infrastructure only: it lets ``tests/golden/make_golden.py`` import and
run the unmodified reference (a numba project) in a container where numba is
not installed.  Decorators return plain Python functions; ``vectorize`` and
``guvectorize`` reproduce numpy-ufunc broadcasting by looping over the
broadcast loop dimensions.  Nothing in the product imports this package.
"""
import re

import numpy as np

__version__ = "0.0-shim"


class _Type:
    """A numba scalar/array type object: ``float64``, ``float64[:]`` ..."""

    def __init__(self, dtype, ndim=0):
        self.dtype = np.dtype(dtype)
        self.ndim = ndim

    def __getitem__(self, key):
        return _Type(self.dtype, len(key) if isinstance(key, tuple) else 1)

    def __call__(self, *args):
        # used both as a signature constructor (``float64(float64[:])``) and as
        # a scalar constructor inside kernels (``complex128(1j)``)
        if len(args) == 1 and not isinstance(args[0], _Type):
            return self.dtype.type(args[0])
        return _Sig(self, args)


class _Sig:
    def __init__(self, ret, args):
        self.ret = ret
        self.args = args


float32 = _Type("float32")
float64 = _Type("float64")
complex64 = _Type("complex64")
complex128 = _Type("complex128")
uint32 = _Type("uint32")
int32 = _Type("int32")
int64 = _Type("int64")
boolean = _Type("bool")

prange = range
_threads = [1]


def set_num_threads(n):
    _threads[0] = int(n)


def get_num_threads():
    return _threads[0]


def _passthrough(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


njit = _passthrough
jit = _passthrough


def _signature_dtypes(sig):
    """Return (input dtypes, output dtype or None) of one declaration."""
    if isinstance(sig, _Sig):
        return [a.dtype for a in sig.args], sig.ret.dtype
    if isinstance(sig, tuple):
        return [a.dtype for a in sig], None
    return None, None


def vectorize(signatures=None, **kwargs):
    def wrap(func):
        nin = func.__code__.co_argcount
        decls = [_signature_dtypes(s) for s in (signatures or [])]

        def ufunc(*args, out=None):
            if len(args) > nin:
                out = args[nin]
                args = args[:nin]
            arrs = [np.asarray(a) for a in args]
            rdt = None
            for cast in ("equiv", "safe", "same_kind"):
                for ins, ret in decls:
                    if ins and all(np.can_cast(a.dtype, t, cast) for a, t in zip(arrs, ins)):
                        rdt = ret
                        arrs = [np.asarray(a, t) for a, t in zip(arrs, ins)]
                        break
                if rdt is not None:
                    break
            b = np.broadcast(*arrs)
            res = np.empty(b.shape, dtype=rdt if rdt is not None else np.result_type(*arrs))
            flat = res.reshape(-1)
            for k, vals in enumerate(b):
                flat[k] = func(*vals)
            if out is not None:
                out[...] = res
                return out
            return res

        ufunc.__name__ = func.__name__
        ufunc.__doc__ = func.__doc__
        return ufunc

    return wrap


def _parse_layout(layout):
    ins, outs = layout.replace(" ", "").split("->")
    group = lambda s: [tuple(x for x in g.split(",") if x) for g in re.findall(r"\(([^)]*)\)", s)]
    return group(ins), group(outs)


class _AnyLayout(np.ndarray):
    """A core argument of a guvectorize kernel.  The reference declares every
    core argument with an any-layout array type (``[:]``, ``[:,:]``), and
    numba's ``ravel`` of such an array is ``flatten`` -- a copy (only arrays
    typed C-contiguous ravel to a view).  numpy would return a view of a
    contiguous core slice, so the stand-in copies here, as numba does."""

    def ravel(self, order="C"):
        return np.array(self, copy=True).reshape(-1)


def guvectorize(signatures, layout, **kwargs):
    core_in, core_out = _parse_layout(layout)
    nin = len(core_in)
    decls = [[t.dtype for t in s] for s in signatures]

    def wrap(func):
        def gufunc(*args, out=None, **kw):
            arrs = [np.asarray(a) for a in args[:nin]]
            if out is None and len(args) > nin:
                out = tuple(args[nin:])
            if out is not None and not isinstance(out, tuple):
                out = (out,)
            if out is not None and all(o is None for o in out):
                out = None
            chosen = None
            for cast in ("equiv", "safe", "same_kind"):
                for d in decls:
                    if all(np.can_cast(a.dtype, t, cast) for a, t in zip(arrs, d[:nin])):
                        chosen = d
                        break
                if chosen is not None:
                    break
            if chosen is None:
                chosen = decls[0]
            arrs = [np.asarray(a, t) for a, t in zip(arrs, chosen[:nin])]
            sizes = {}
            loop_shapes = []
            for a, core in zip(arrs, core_in):
                nc = len(core)
                if a.ndim < nc:
                    raise ValueError("gufunc core dimensions mismatch")
                for name, n in zip(core, a.shape[a.ndim - nc:]):
                    if sizes.setdefault(name, n) != n:
                        raise ValueError("gufunc core dimension %s mismatch" % name)
                loop_shapes.append(a.shape[: a.ndim - nc])
            lshape = np.broadcast_shapes(*loop_shapes)
            if out is None:
                out = tuple(
                    np.empty(lshape + tuple(sizes[n] for n in core), dtype=t)
                    for core, t in zip(core_out, chosen[nin:])
                )
            else:
                lshape = np.broadcast_shapes(
                    lshape, *[o.shape[: o.ndim - len(c)] for o, c in zip(out, core_out)]
                )
            barrs = [np.broadcast_to(a, lshape + a.shape[a.ndim - len(c):]) for a, c in zip(arrs, core_in)]
            bouts = [np.broadcast_to(o, lshape + o.shape[o.ndim - len(c):]) if o.shape[: o.ndim - len(c)] != lshape else o
                     for o, c in zip(out, core_out)]
            for idx in np.ndindex(*lshape):
                iv = [(a[idx] if len(c) else a[idx].reshape(1)).view(_AnyLayout) for a, c in zip(barrs, core_in)]
                ov = [(o[idx] if len(c) else o.reshape(o.shape + (1,))[idx]).view(_AnyLayout)
                      for o, c in zip(bouts, core_out)]
                func(*iv, *ov)
            return out[0] if len(out) == 1 else out

        gufunc.__name__ = func.__name__
        gufunc.__doc__ = func.__doc__
        return gufunc

    return wrap
