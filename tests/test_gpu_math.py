"""Accuracy of the evaluator's compact exp / log / pow (gpr_fastmath.cuh)
against FP64, measured on the GPU through gpr_debug_math.  The evaluator must
stay within a few ulp of the correctly rounded FP32 result so that program
values agree with the reference's libm to the 1e-5 relative tolerance of the
parity tests; special values follow C99 Annex F like the reference's libm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")


@pytest.fixture(scope="module")
def sampler():
    s = g.Sampler(32, program_length=31)
    yield s
    s.close()


def ulp_err(out, ref64):
    """|out - ref| in units of the FP32 spacing at the correctly rounded value
    (subnormal spacing below the normal range)."""
    ref32 = ref64.astype(np.float32)
    sp = np.spacing(np.abs(ref32)).astype(np.float64)
    sp = np.maximum(sp, np.float64(np.finfo(np.float32).smallest_subnormal))
    return np.abs(out.astype(np.float64) - ref64) / sp


def test_exp_accuracy(sampler):
    r = np.random.default_rng(0)
    x = np.concatenate([np.linspace(-103.9, 88.72, 1_000_000), r.uniform(-20, 20, 500_000),
                        r.normal(0, 1e-3, 100_000)]).astype(np.float32)
    out = sampler.math("exp", x)
    ref = np.exp(x.astype(np.float64))
    fin = np.isfinite(ref.astype(np.float32))
    e = ulp_err(out[fin], ref[fin])
    assert e.max() <= 2.0, (e.max(), x[fin][np.argmax(e)])
    assert np.all(np.isinf(out[~fin]))
    sp = np.float32([0.0, -0.0, np.inf, -np.inf, np.nan, 89.0, -110.0])
    o = sampler.math("exp", sp)
    assert o[0] == 1 and o[1] == 1 and o[2] == np.inf and o[3] == 0 and np.isnan(o[4])
    assert o[5] == np.inf and o[6] == 0


def test_log_accuracy(sampler):
    r = np.random.default_rng(1)
    x = np.concatenate([10.0 ** r.uniform(-44, 38.5, 1_000_000), r.uniform(0.5, 2.0, 500_000),
                        1.0 + r.normal(0, 1e-4, 100_000)]).astype(np.float32)
    x = x[(x > 0) & np.isfinite(x)]
    out = sampler.math("log", x)
    e = ulp_err(out, np.log(x.astype(np.float64)))
    assert e.max() <= 2.0, (e.max(), x[np.argmax(e)])
    sp = np.float32([0.0, -0.0, -1.0, np.inf, np.nan, 1.0])
    o = sampler.math("log", sp)
    assert o[0] == -np.inf and o[1] == -np.inf and np.isnan(o[2]) and o[3] == np.inf
    assert np.isnan(o[4]) and o[5] == 0


def test_pow_accuracy(sampler):
    r = np.random.default_rng(2)
    n = 1_000_000
    a = np.concatenate([r.uniform(0, 100, n), 10.0 ** r.uniform(-30, 30, n), -r.uniform(0.1, 10, n)])
    b = np.concatenate([r.uniform(-30, 30, n), r.uniform(-3, 3, n), np.round(r.uniform(-20, 20, n))])
    a, b = a.astype(np.float32), b.astype(np.float32)
    out = sampler.math("pow", a, b)
    with np.errstate(all="ignore"):
        ref = np.power(a.astype(np.float64), b.astype(np.float64))
    fin = np.isfinite(ref.astype(np.float32)) & (np.abs(ref) > np.finfo(np.float32).tiny)
    e = ulp_err(out[fin], ref[fin])
    assert e.max() <= 3.0, (e.max(), a[fin][np.argmax(e)], b[fin][np.argmax(e)])
    big = np.isfinite(ref) & ~np.isfinite(ref.astype(np.float32))
    assert np.all(np.isinf(out[big]))


def test_pow_special_cases(sampler):
    inf, nan = np.inf, np.nan
    cases = [(2.0, 0.0), (nan, 0.0), (1.0, nan), (1.0, inf), (-1.0, inf), (-1.0, -inf), (0.5, inf),
             (0.5, -inf), (2.0, inf), (2.0, -inf), (-2.0, 0.5), (-2.0, 3.0), (-2.0, 2.0), (0.0, -1.0),
             (-0.0, -1.0), (-0.0, -2.0), (0.0, 3.0), (-0.0, 3.0), (-0.0, 2.0), (inf, -1.0), (inf, 2.0),
             (-inf, 3.0), (-inf, 2.0), (-inf, -3.0), (-inf, 0.5), (-inf, -0.5), (nan, 1.0), (2.0, nan),
             (-8.0, 1.0 / 3.0), (3.0, 2.0), (10.0, -2.0)]
    a = np.float32([c[0] for c in cases])
    b = np.float32([c[1] for c in cases])
    out = sampler.math("pow", a, b)
    with np.errstate(all="ignore"):
        ref = np.power(a, b)      # numpy float32 power follows C99 Annex F
    for (ai, bi), o, rr in zip(cases, out, ref):
        if np.isnan(rr):
            assert np.isnan(o), (ai, bi, o, rr)
        else:
            assert o == rr and np.signbit(o) == np.signbit(rr), (ai, bi, o, rr)
