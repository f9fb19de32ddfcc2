"""The reason the kernels issue no FP64 arithmetic in their step loops: on
GB300, FP64 throughput is a small fraction of FP32.  Measured with cuBLAS
GEMMs (DGEMM vs SGEMM without TF32), and with the library's own add kernels,
which also show that an FP64 add issued by a single lane of a warp costs what
a full warp's costs (so confining FP64 work to one lane saves nothing).  The
tests print the figures."""
import time

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _tflops(dtype, n=4096, reps=5):
    a = torch.randn(n, n, device="cuda", dtype=dtype)
    b = torch.randn(n, n, device="cuda", dtype=dtype)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(reps):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    return 2.0 * n ** 3 * reps / (time.perf_counter() - t) / 1e12


def test_fp64_rate_is_a_small_fraction_of_fp32():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        f32 = _tflops(torch.float32)
        f64 = _tflops(torch.float64)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old
    print("SGEMM %.2f TFLOP/s, DGEMM %.2f TFLOP/s, ratio %.1f" % (f32, f64, f32 / f64))
    assert f32 / f64 > 8


def test_fp64_add_issue_cost():
    g = pytest.importorskip("gpuropolis_gb300")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    d32, d1, f32 = g.fp_issue_times(0, 4096)
    print("FP64 adds, 32 lanes: %.3f ms; FP64 adds, 1 lane per warp: %.3f ms; FP32 adds, 32 lanes: %.3f ms; "
          "FP64/FP32 %.0fx" % (d32, d1, f32, d32 / f32))
    assert d32 > 8 * f32          # FP64 is a small fraction of FP32
    assert d1 > 0.5 * d32         # one active lane costs (almost) a whole warp
