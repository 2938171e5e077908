"""Torch-backed stand-in for the HIPS ``autograd`` package (test infrastructure only).

xreac imports ``autograd`` (HIPS, >=1.9.1,<2), which is not installed in this
environment. This package provides the handful of entry points the reference
uses -- ``make_vjp``, ``grad``, ``autograd.numpy``, ``autograd.tracer.getval``,
``autograd.extend.primitive`` and ``defvjp`` -- on top of ``torch.autograd``, so
that the UNMODIFIED reference ``Calculator.evaluate`` runs here and can write
golden fixtures. It is never imported by the product package.

Traced values are CPU float64 torch tensors. Plain numpy inputs stay numpy, so a
call without tracing is bit-identical to running the reference on numpy.
"""

import numpy as _onp
import torch as _torch

from . import numpy  # noqa: F401  (exposes autograd.numpy)
from .numpy import _to_tensor


def make_vjp(fun, argnum=0):
    def wrapped(*args):
        args = list(args)
        x = _torch.tensor(_onp.asarray(args[argnum], dtype=float), dtype=_torch.float64, requires_grad=True)
        args[argnum] = x
        out = fun(*args)
        out_t = _to_tensor(out)

        def backward(g):
            (gx,) = _torch.autograd.grad(
                out_t, x, grad_outputs=_to_tensor(g).reshape(out_t.shape), retain_graph=True, allow_unused=True
            )
            if gx is None:
                return _onp.zeros(x.shape)
            return gx.detach().numpy().copy()

        return backward, out_t.detach().numpy().copy()

    return wrapped


def grad(fun, argnum=0):
    def wrapped(*args):
        backward, value = make_vjp(fun, argnum)(*args)
        return backward(_onp.ones_like(value))

    return wrapped
