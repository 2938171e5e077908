"""``autograd.numpy`` stand-in: numpy for numpy inputs, torch for traced tensors."""

import numpy as _onp
import torch as _torch

from numpy import *  # noqa: F401,F403


def _is_t(x):
    return isinstance(x, _torch.Tensor)


def _promote_numpy_operands():
    """Let traced tensors combine with numpy operands (``tensor + ndarray``)."""
    if getattr(_torch.Tensor, "_xr_shim_patched", False):
        return
    names = (
        "__add__ __radd__ __sub__ __rsub__ __mul__ __rmul__ __truediv__ __rtruediv__ "
        "__pow__ __rpow__ __lt__ __le__ __gt__ __ge__ __eq__ __ne__ __and__ __or__"
    ).split()
    for name in names:
        original = getattr(_torch.Tensor, name)

        def patched(self, other, _original=original):
            if isinstance(other, (_onp.ndarray, _onp.generic)):
                other = _to_tensor(other)
            return _original(self, other)

        setattr(_torch.Tensor, name, patched)
    _torch.Tensor._xr_shim_patched = True


def _to_tensor(x):
    if _is_t(x):
        return x
    if isinstance(x, (list, tuple)) and any(_is_t(v) for v in x):
        return _torch.stack([_to_tensor(v) for v in x])
    arr = _onp.asarray(x)
    if arr.dtype == bool:
        return _torch.as_tensor(arr)
    if arr.dtype.kind in "iu":
        return _torch.as_tensor(arr.astype(_onp.int64))
    return _torch.as_tensor(arr.astype(float), dtype=_torch.float64)


def _any_t(*xs):
    for x in xs:
        if _is_t(x):
            return True
        if isinstance(x, (list, tuple)) and any(_is_t(v) for v in x):
            return True
    return False


def _unary(npf, tf):
    def f(x, *a, **k):
        return tf(x) if _is_t(x) else npf(x, *a, **k)

    return f


exp = _unary(_onp.exp, _torch.exp)
log = _unary(_onp.log, _torch.log)
sqrt = _unary(_onp.sqrt, _torch.sqrt)
sin = _unary(_onp.sin, _torch.sin)
cos = _unary(_onp.cos, _torch.cos)
arccos = _unary(_onp.arccos, _torch.arccos)
abs = _unary(_onp.abs, _torch.abs)  # noqa: A001


def where(c, a, b):
    if not _any_t(c, a, b):
        return _onp.where(c, a, b)
    c = _to_tensor(c).to(_torch.bool) if not _is_t(c) else c
    return _torch.where(c, _to_tensor(a), _to_tensor(b))


def minimum(a, b):
    if not _any_t(a, b):
        return _onp.minimum(a, b)
    return _torch.minimum(_to_tensor(a), _to_tensor(b))


def maximum(a, b):
    if not _any_t(a, b):
        return _onp.maximum(a, b)
    return _torch.maximum(_to_tensor(a), _to_tensor(b))


def clip(x, lo, hi):
    if not _is_t(x):
        return _onp.clip(x, lo, hi)
    return _torch.clamp(x, lo, hi)


def sum(x, axis=None, **k):  # noqa: A001
    if not _is_t(x):
        return _onp.sum(x, axis=axis, **k)
    return _torch.sum(x) if axis is None else _torch.sum(x, dim=axis)


def stack(xs, axis=0):
    if not _any_t(*xs):
        return _onp.stack(xs, axis=axis)
    return _torch.stack([_to_tensor(x) for x in xs], dim=axis)


def concatenate(xs, axis=0):
    if not _any_t(*xs):
        return _onp.concatenate(xs, axis=axis)
    return _torch.cat([_to_tensor(x) for x in xs], dim=axis)


def cross(a, b):
    if not _any_t(a, b):
        return _onp.cross(a, b)
    return _torch.linalg.cross(_to_tensor(a), _to_tensor(b), dim=-1)


def diag(x):
    return _torch.diag(x) if _is_t(x) else _onp.diag(x)


def reshape(x, shape):
    return _torch.reshape(x, shape) if _is_t(x) else _onp.reshape(x, shape)


class _Linalg:
    def __getattr__(self, name):
        return getattr(_onp.linalg, name)

    @staticmethod
    def solve(a, b):
        if not _any_t(a, b):
            return _onp.linalg.solve(a, b)
        try:
            return _torch.linalg.solve(_to_tensor(a), _to_tensor(b))
        except RuntimeError as exc:  # map torch's singular-matrix error to numpy's
            raise _onp.linalg.LinAlgError(str(exc)) from exc

    @staticmethod
    def norm(x, *a, **k):
        return _onp.linalg.norm(x, *a, **k)


linalg = _Linalg()

_promote_numpy_operands()
