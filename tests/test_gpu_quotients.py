"""The division helpers of the element and nodal kernels against CUDA's IEEE division, on the GPU.

nr_rcp (the Newton-Raphson reciprocal from the hardware seed rcp.approx.ftz.f64) and quot (a / b
as a r plus one residual correction) replace IEEE divisions on the FP64-bound hot path.  Their
documented domain is normal b with 2^-1022 < |b| < 2^1022 and a normal quotient.  Bound held here:
both within one ulp of the IEEE result everywhere in that domain, and each correctly rounded in all
but a small fraction of cases (measured on GB300: equal to the IEEE results on all 1,049,194
inputs; the fractions are printed)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulps(x, y):
    """|x - y| in units in the last place of y (finite, same-sign doubles)."""
    xi = x.view(np.int64).astype(np.float64)
    yi = y.view(np.int64).astype(np.float64)
    return np.abs(xi - yi)


def inputs(seed=0, n=1 << 20):
    rng = np.random.default_rng(seed)
    # random significands across the whole documented exponent range, both signs
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-1000, 1000, n).astype(np.float64))
    b *= np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    a = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 20, n).astype(np.float64))
    # edges: powers of two, 1 +- a few ulps, the domain's ends, values the kernels divide by
    edge = [2.0 ** k for k in range(-1021, 1022, 7)]
    one = np.nextafter(1.0, 2.0)
    edge += [1.0, one, np.nextafter(1.0, 0.0), np.nextafter(one, 2.0), 3.0, 7.0, 1.0 / 3.0, 0.1,
             2.0 ** -1021 * 1.5, 2.0 ** 1021 * 1.999, 1e-10, 1e10, 0.649984, 1.0 - 0.350016,
             8930.0 * 1e-9, 3.2e-3, 1.6e-5]
    edge = np.array(edge)
    a_edge = np.ones_like(edge) * 1.2345678901234567
    return np.concatenate([a, a_edge, -a_edge]), np.concatenate([b, edge, edge])


def test_reciprocal_and_quotient_vs_ieee_division(gpu_lib):
    a, b = inputs()
    r = gpu_lib.check_quotients(a, b)
    assert np.all(np.isfinite(r["rcp"])) and np.all(np.isfinite(r["quot"]))
    ur = ulps(r["rcp"], r["ieee_rcp"])
    uq = ulps(r["quot"], r["ieee_quot"])
    exact_r = float(np.mean(ur == 0))
    exact_q = float(np.mean(uq == 0))
    print(f"nr_rcp: max {ur.max():.0f} ulp, exact {exact_r:.6f}; "
          f"quot: max {uq.max():.0f} ulp, exact {exact_q:.6f} (n = {a.size})")
    assert ur.max() <= 1
    assert uq.max() <= 1
    assert exact_r >= 0.999 and exact_q >= 0.999


def test_quotient_of_equal_values_and_exact_cases(gpu_lib):
    """Exact quotients (a multiple of b by a power of two, b a power of two) come out exact."""
    rng = np.random.default_rng(1)
    b = rng.uniform(1.0, 2.0, 4096) * np.exp2(rng.integers(-500, 500, 4096).astype(np.float64))
    k = np.exp2(rng.integers(-30, 30, 4096).astype(np.float64))
    r = gpu_lib.check_quotients(b * k, b)
    assert np.array_equal(r["quot"], k)
    p2 = np.exp2(np.arange(-1000, 1000, 3).astype(np.float64))
    r = gpu_lib.check_quotients(np.ones_like(p2), p2)
    assert np.array_equal(r["rcp"], 1.0 / p2)
    assert np.array_equal(r["quot"], 1.0 / p2)
