"""GPU parity of the FP64-accurate tensor-core product (modal_gemm_f64: exact
7-bit integer slices on tcgen05, the Ozaki scheme) against numpy's FP64
product.  Error measure: max |C - C_f64| / max(|A| |B|) (|.| elementwise),
which is at most about K * 2^-53 for the FP64 product itself."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(mg):
    c = mg.Context(0)
    yield c
    c.close()


def err(C, A, B, Cref):
    return float(np.max(np.abs(C - Cref)) / np.max(np.abs(A) @ np.abs(B)))


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (7, 5, 3), (128, 128, 64), (130, 250, 511), (300, 200, 513),
                                   (257, 129, 1500), (64, 600, 4100)])
def test_gemm_f64_shapes(ctx, M, N, K):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((K, N))
    C = ctx.gemm_f64(A, B)
    assert err(C, A, B, A @ B) <= 1e-14


def test_gemm_f64_transposes_alpha_beta(ctx):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((400, 300))  # op(A) = A^T: 300 x 400
    B = rng.standard_normal((250, 400))  # op(B) = B^T: 400 x 250
    C0 = rng.standard_normal((300, 250))
    C = ctx.gemm_f64(A, B, transA=True, transB=True, alpha=-0.75, beta=2.0, C=C0)
    ref = -0.75 * (A.T @ B.T) + 2.0 * C0
    assert np.max(np.abs(C - ref)) / (0.75 * np.max(np.abs(A.T) @ np.abs(B.T)) + 2 * np.max(np.abs(C0))) <= 1e-14


def test_gemm_f64_graded_rows(ctx):
    """Entries spanning many binades within a row and column: the error stays
    below 2^-45 of the row maximum times the column maximum."""
    rng = np.random.default_rng(9)
    M, N, K = 200, 180, 700
    A = rng.standard_normal((M, K)) * 10.0 ** rng.uniform(-12, 3, (M, K))
    B = rng.standard_normal((K, N)) * 10.0 ** rng.uniform(-12, 3, (K, N))
    C = ctx.gemm_f64(A, B)
    ref = A @ B
    bound = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * K * 2.0 ** -45
    assert np.all(np.abs(C - ref) <= bound)


@pytest.mark.parametrize("s", [3, 5, 7, 8])
def test_gemm_f64_slices_error_scaling(ctx, s):
    rng = np.random.default_rng(11)
    A = rng.uniform(-1, 1, (256, 1024))
    B = rng.uniform(-1, 1, (1024, 256))
    e = err(ctx.gemm_f64(A, B, slices=s), A, B, A @ B)
    assert e <= max(1e-14, 2.0 ** (-7 * s + 6))
