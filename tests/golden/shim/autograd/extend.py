"""``autograd.extend`` stand-in: primitives with user-supplied VJPs via torch.autograd.Function."""

import numpy as _onp
import torch as _torch

_VJPS = {}


def _numpy_value(x):
    return x.detach().numpy() if isinstance(x, _torch.Tensor) else x


def primitive(fun):
    def wrapped(*args, **kwargs):
        traced = [k for k, a in enumerate(args) if isinstance(a, _torch.Tensor) and a.requires_grad]
        plain = [_numpy_value(a) for a in args]
        if not traced:
            return fun(*plain, **kwargs)
        makers = _VJPS.get(wrapped, ())

        class _Prim(_torch.autograd.Function):
            @staticmethod
            def forward(ctx, *tensors):
                out = fun(*plain, **kwargs)
                ctx.ans = out
                return _torch.as_tensor(_onp.asarray(out, dtype=float), dtype=_torch.float64)

            @staticmethod
            def backward(ctx, g):
                grads = []
                for k in traced:
                    maker = makers[k] if k < len(makers) else None
                    if maker is None:
                        grads.append(None)
                        continue
                    vjp = maker(ctx.ans, *plain, **kwargs)
                    grads.append(_torch.as_tensor(vjp(g), dtype=_torch.float64))
                return tuple(grads)

        return _Prim.apply(*[args[k] for k in traced])

    wrapped.__name__ = getattr(fun, "__name__", "primitive")
    return wrapped


def defvjp(prim, *makers):
    _VJPS[prim] = makers
