"""Tensor-core complex GEMM (ia_zgemm_batch, IA_PREC_MIXED): BF16 slices of
the FP64 operands on the tcgen05 pipe (Ozaki scheme), against an FP64
product computed here.

Error bound of the scheme, per output element: at most (4 S + 8) 2^(-6 S)
times |alpha| K max_k |a_ik| max_k |b_kj| for each real product term; a
complex element sums two real products per part, so the test allows four
times that (max over |Re|, |Im| as the magnitudes).  The measured ratio to
that tolerance is printed.  The reference's counterpart is cublasZgemm
(CUDA/ibem.cuh:398)."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu


def _bound(S):
    return (4 * S + 8) * 2.0 ** (-6 * S)


def _op(X, op):
    return {"N": X, "T": X.T, "C": X.conj().T}[op]


def _case(rng, F, M, N, K, opa, opb, spread=0.0):
    """Column-major operands as numpy arrays of shape (F, cols, rows) for the
    C ABI (the transpose of the math matrix), with an optional per-row /
    per-column magnitude spread of 10^spread."""
    def cn(*s):
        return rng.standard_normal(s) + 1j * rng.standard_normal(s)
    A = cn(F, M, K) * 10.0 ** (spread * rng.uniform(-1, 1, (F, M, 1)))     # op(A): M x K
    B = cn(F, K, N) * 10.0 ** (spread * rng.uniform(-1, 1, (F, 1, N)))     # op(B): K x N
    Cin = cn(F, M, N)
    # stored matrices: op(A_st) = A, column-major (F, cols, rows)
    A_st = np.stack([_op(a, opa) for a in A])        # op(op(A)) = A for N, T and C
    B_st = np.stack([_op(b, opb) for b in B])
    colmaj = lambda X: np.ascontiguousarray(np.transpose(X, (0, 2, 1)))
    return A, B, Cin, colmaj(A_st), colmaj(B_st), colmaj(Cin)


def _run(ctx, cuda, opa, opb, M, N, K, S, F=2, alpha=1.0, beta=0.0, spread=0.0, seed=5):
    import torch
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(seed)
    A, B, Cin, Ad, Bd, Cd = _case(rng, F, M, N, K, opa, opb, spread)
    tA, tB, tC = (torch.as_tensor(x, device=cuda) for x in (Ad, Bd, Cd))
    info = torch.zeros(F, dtype=torch.int32, device=cuda)
    api.zgemm_batch(ctx, opa, opb, M, N, K, tA, tB, tC, alpha=alpha, beta=beta, precision=1, slices=S, info=info)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    out = np.transpose(tC.cpu().numpy(), (0, 2, 1))
    ref = alpha * np.einsum("fik,fkj->fij", A, B) + beta * Cin
    mag = lambda X: np.maximum(np.abs(X.real), np.abs(X.imag))
    scale = abs(alpha) * K * mag(A).max(axis=2)[:, :, None] * mag(B).max(axis=1)[:, None, :]
    err = np.maximum(np.abs((out - ref).real), np.abs((out - ref).imag))
    return out, ref, (err / scale).max()


@pytest.mark.parametrize("S", [6, 7, 8])
@pytest.mark.parametrize("opa,opb", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "N")])
def test_tc_gemm_within_the_slicing_bound(cuda, ctx, S, opa, opb):
    # ragged sizes: M not a multiple of 128, N of 32, K of 16
    _, _, ratio = _run(ctx, cuda, opa, opb, 200, 45, 77, S, spread=3.0)
    tol = 4 * _bound(S)
    print(f"\nS={S} {opa}{opb}: max |err| / (|alpha| K max|a_row| max|b_col|) = {ratio:.3e} "
          f"(bound {_bound(S):.1e}); max err / tolerance = {ratio / tol:.3f}")
    assert ratio < tol


def test_tc_gemm_alpha_beta_accumulate(cuda, ctx):
    _, _, ratio = _run(ctx, cuda, "N", "N", 130, 33, 64, 7, alpha=-1.0, beta=1.0)
    assert ratio < 4 * _bound(7)


@pytest.mark.parametrize("S", [7, 8])
def test_tc_gemm_transfer_shape_matches_fp64_gemm(cuda, ctx, S):
    """The shape of the IBEM transfer product (642 x 120 x 642, four bins)
    against the FP64 CUDA-core GEMM of the same library."""
    import torch
    from inverseacoustics_gb300 import api
    rng = np.random.default_rng(11)
    F, M, N, K = 4, 642, 120, 642
    A = np.ascontiguousarray(rng.standard_normal((F, K, M)) + 1j * rng.standard_normal((F, K, M)))
    B = np.ascontiguousarray(rng.standard_normal((F, N, K)) + 1j * rng.standard_normal((F, N, K)))
    tA, tB = torch.as_tensor(A, device=cuda), torch.as_tensor(B, device=cuda)
    C64 = torch.zeros((F, N, M), dtype=torch.complex128, device=cuda)
    Ctc = torch.zeros_like(C64)
    api.zgemm_batch(ctx, "N", "N", M, N, K, tA, tB, C64, precision=0)
    api.zgemm_batch(ctx, "N", "N", M, N, K, tA, tB, Ctc, precision=1, slices=S)
    torch.cuda.synchronize()
    e = relerr(Ctc.cpu().numpy(), C64.cpu().numpy())
    print(f"\n{M}x{N}x{K} x{F}, S={S}: tensor-core vs FP64 GEMM relative error {e:.3e}")
    assert e < (1e-10 if S == 7 else 1e-12)


def test_tc_gemm_refuses_k_beyond_exact_fp32_sums(cuda, ctx):
    """At 7 slices the FP32 level sums stay exact only for 2 K 7 1024 <= 2^24
    (K <= 1170); a longer product is refused, not rounded."""
    import torch
    from inverseacoustics_gb300 import _lib
    M, N, K = 16, 8, 1200
    A = torch.zeros((1, K, M), dtype=torch.complex128, device=cuda)
    B = torch.zeros((1, N, K), dtype=torch.complex128, device=cuda)
    C = torch.zeros((1, N, M), dtype=torch.complex128, device=cuda)
    st = _lib.lib().ia_zgemm_batch(ctx.handle, 0, 0, M, N, K, 1.0, A.data_ptr(), M, A[0].numel(), B.data_ptr(), K,
                                   B[0].numel(), 0.0, C.data_ptr(), M, C[0].numel(), 1, 1, 7, None)
    assert st == 8
    st = _lib.lib().ia_zgemm_batch(ctx.handle, 0, 0, M, N, 64, 1.0, A.data_ptr(), M, A[0].numel(), B.data_ptr(), 64,
                                   B[0].numel(), 0.0, C.data_ptr(), M, C[0].numel(), 1, 1, 9, None)
    assert st == 1
