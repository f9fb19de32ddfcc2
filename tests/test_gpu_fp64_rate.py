"""The reason the kernel issues no FP64 arithmetic in its step loop: on GB300,
FP64 throughput is a small fraction of FP32.  Measured with cuBLAS GEMMs
(DGEMM vs SGEMM without TF32); the test prints both rates."""
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
