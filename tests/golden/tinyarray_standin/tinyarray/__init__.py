"""Minimal numpy-backed stand-in for the ``tinyarray`` package.

Test infrastructure only: it lets the reference Kwant sources (which import
``tinyarray``) run in this container so that golden fixtures can be generated
from the reference itself.  It implements the subset of the tinyarray API the
reference uses on the KPM path: ``array``, ``matrix``, ``dot``, ``zeros``,
``identity`` and the ``ndarray_int/float/complex`` types.

tinyarray arrays are immutable, hashable and compare like tuples (they are
used as site tags, dictionary keys and sort keys); the ndarray subclasses
below reproduce exactly those three properties.
"""

import numpy as np

__all__ = ['array', 'matrix', 'dot', 'zeros', 'identity',
           'ndarray_int', 'ndarray_float', 'ndarray_complex']


def _as_key(a):
    arr = np.asarray(a)
    if arr.ndim == 0:
        return arr.item()
    return tuple(_as_key(x) for x in arr)


class _Tiny(np.ndarray):
    """Hashable ndarray with tuple-style equality and ordering."""

    def __array_finalize__(self, obj):
        pass

    def __hash__(self):
        return hash(_as_key(self))

    def __eq__(self, other):
        try:
            o = np.asarray(other)
        except Exception:
            return False
        if o.shape != self.shape:
            return False
        return bool(np.all(np.asarray(self).view(np.ndarray) == o))

    def __ne__(self, other):
        return not self.__eq__(other)

    def __lt__(self, other):
        return _as_key(self) < _as_key(other)

    def __le__(self, other):
        return _as_key(self) <= _as_key(other)

    def __gt__(self, other):
        return _as_key(self) > _as_key(other)

    def __ge__(self, other):
        return _as_key(self) >= _as_key(other)

    def __repr__(self):
        # tinyarray's repr: 'array(' + nested Python-list repr + ')'.  Site
        # families derive their sort key from it (kwant/lattice.py:389-391,
        # :441-446), so the stand-in must reproduce it for site order.
        return 'array(%r)' % (np.asarray(self).view(np.ndarray).tolist(),)

    def __str__(self):
        return str(np.asarray(self).view(np.ndarray).tolist())

    def __reduce__(self):
        return (array, (np.asarray(self).view(np.ndarray).tolist(),
                        self.dtype.type))


class ndarray_int(_Tiny):
    pass


class ndarray_float(_Tiny):
    pass


class ndarray_complex(_Tiny):
    pass


def _wrap(arr):
    arr = np.ascontiguousarray(arr)
    if arr.dtype.kind in 'iub':
        arr = arr.astype(np.int64, copy=False)
        cls = ndarray_int
    elif arr.dtype.kind == 'f':
        arr = arr.astype(np.float64, copy=False)
        cls = ndarray_float
    elif arr.dtype.kind == 'c':
        arr = arr.astype(np.complex128, copy=False)
        cls = ndarray_complex
    else:
        raise TypeError('unsupported dtype for tinyarray stand-in: %s'
                        % arr.dtype)
    # Left writable: the reference's Cython code takes (non-const) typed
    # memoryviews of these arrays.  Nothing in the reference writes to them.
    return arr.view(cls)


def _dtype_of(dtype):
    if dtype is None:
        return None
    if dtype is int:
        return np.int64
    if dtype is float:
        return np.float64
    if dtype is complex:
        return np.complex128
    return np.dtype(dtype)


def array(obj, dtype=None):
    src = np.asarray(obj.view(np.ndarray) if isinstance(obj, _Tiny) else obj)
    dt = _dtype_of(dtype)
    if dt is not None:
        if np.dtype(dt).kind == 'i' and src.dtype.kind == 'f':
            if not np.all(np.round(src) == src):
                raise TypeError('cannot convert non-integral floats to int')
        src = src.astype(dt)
    return _wrap(src)


def matrix(obj, dtype=None):
    arr = np.asarray(obj.view(np.ndarray) if isinstance(obj, _Tiny) else obj)
    if arr.ndim == 0:
        arr = arr.reshape(1, 1)
    elif arr.ndim == 1:
        arr = arr.reshape(1, -1)
    elif arr.ndim != 2:
        raise ValueError('matrix must be 2-d')
    dt = _dtype_of(dtype)
    if dt is not None:
        arr = arr.astype(dt)
    return _wrap(arr)


def dot(a, b):
    av = a.view(np.ndarray) if isinstance(a, _Tiny) else np.asarray(a)
    bv = b.view(np.ndarray) if isinstance(b, _Tiny) else np.asarray(b)
    res = np.dot(av, bv)
    if np.ndim(res) == 0:
        return np.asarray(res).item()
    return _wrap(res)


def zeros(shape, dtype=float):
    return _wrap(np.zeros(shape, dtype=_dtype_of(dtype)))


def identity(n, dtype=float):
    return _wrap(np.identity(n, dtype=_dtype_of(dtype)))
