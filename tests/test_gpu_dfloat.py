"""The double-float exp and log of the pair and bond-order kernels (xreac_gb300/csrc/xr_dfloat.cuh)
against CUDA's FP64 exp and log, over the arguments those kernels take and the rest of the domain:
exp within 2e-14 relative, log within 2e-14 absolute (2e-14 relative for |log a| > 1), and the
FP64 functions outside the domain (|x| >= 80, a outside [1e-30, 1e30], non-finite)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _apply(fn, x):
    import torch
    from xreac_gb300 import _native as nat

    lib = nat.load()
    xi = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device="cuda")
    out = torch.empty_like(xi)
    assert lib.xr_test_math(fn, xi.data_ptr(), out.data_ptr(), xi.numel()) == 0
    return out.cpu().numpy()


def test_exp_matches_cuda_exp():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-79.9, 79.9, 400_000), rng.uniform(-3.0, 3.0, 400_000),
                        rng.normal(0.0, 1e-3, 100_000), [0.0, -0.0, 1e-300, -1e-300, 79.99, -79.99],
                        np.log(2.0) / 64 * np.arange(-200, 200) + 1e-12])
    got, want = _apply(0, x), _apply(1, x)
    rel = np.abs(got - want) / want
    assert rel.max() < 2e-14, (rel.max(), x[np.argmax(rel)])


def test_log_matches_cuda_log():
    rng = np.random.default_rng(1)
    a = np.concatenate([10.0 ** rng.uniform(-29.9, 29.9, 400_000), rng.uniform(0.3, 12.0, 400_000),
                        1.0 + rng.normal(0.0, 1e-6, 50_000), 1.0 + rng.normal(0.0, 1e-2, 50_000),
                        [1.0, 2.0, 0.5, 1e-30, 1e30, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)]])
    got, want = _apply(2, a), _apply(3, a)
    err = np.abs(got - want) / np.maximum(1.0, np.abs(want))
    assert err.max() < 2e-14, (err.max(), a[np.argmax(err)])


def test_outside_the_domain_uses_the_fp64_functions():
    x = np.array([80.0, -80.0, 300.0, -700.0, np.inf, -np.inf, np.nan])
    got, want = _apply(0, x), _apply(1, x)
    np.testing.assert_array_equal(got, want)
    a = np.array([1e-31, 1e31, 1e-300, 1e300, 0.0, -1.0, np.inf, np.nan])
    got, want = _apply(2, a), _apply(3, a)
    np.testing.assert_array_equal(got, want)
