"""Dense LU on the GPU (Matrice::set_lu / solve) against scipy's LAPACK
getrf/getrs, FP64 and mixed-precision (TF32/FP32 factors + FP64 GMRES-IR)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def make(n, cond, seed):
    rng = np.random.default_rng(seed)
    u, _ = np.linalg.qr(rng.standard_normal((n, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.logspace(0, -np.log10(cond), n)
    return (u * s) @ v.T


@pytest.mark.parametrize("n", [1, 7, 96, 97, 300, 1000])
def test_fp64_lu_solve_matches_lapack(ctx, n):
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_FP64
    A = make(n, 1e6, n)
    b = np.random.default_rng(1).standard_normal(n)
    dA = torch.tensor(A.T.copy(), device="cuda")  # column-major storage
    db = torch.tensor(b, device="cuda")
    lu = DenseLU(ctx)
    lu.factor(dA.data_ptr(), n, n, KD_LU_FP64)
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    xr = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-8
    # transposed solve with the same factors
    db2 = torch.tensor(b, device="cuda")
    lu.solve(db2.data_ptr(), 1)
    xt = db2.cpu().numpy()
    xtr = np.linalg.solve(A.T, b)
    assert np.linalg.norm(xt - xtr) / np.linalg.norm(xtr) < 1e-8


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("n", [200, 1100])
def test_mixed_lu_gmres_ir_reaches_fp64(ctx, mode, n):
    from kadath_frontera_gb300.kadath import DenseLU
    A = make(n, 1e4, n + mode)
    b = np.random.default_rng(2).standard_normal(n)
    dA = torch.tensor(A.T.copy(), device="cuda")
    db = torch.tensor(b, device="cuda")
    lu = DenseLU(ctx)
    lu.factor(dA.data_ptr(), n, n, mode)
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    r = A @ x - b
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-12
    st = lu.stats()
    assert st["refine_iters"] >= 1


def test_singular_matrix_reports_status(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300.kadath import DenseLU
    n = 50
    A = np.random.default_rng(3).standard_normal((n, n))
    A[:, 7] = 0.0
    dA = torch.tensor(A.T.copy(), device="cuda")
    lu = DenseLU(ctx)
    with pytest.raises(KadathError) as e:
        lu.factor(dA.data_ptr(), n, n, 0)
    assert e.value.status == 3  # KD_ERR_SINGULAR


@pytest.mark.parametrize("aligned", [False, True])
@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 384, 96), (200, 130, 96), (1000, 777, 64), (33, 257, 17),
                                   (2000, 1500, 128)])
def test_tcgen05_tf32_update_matches_fp64_product(ctx, m, n, k, aligned):
    """C -= A B on the tcgen05 tensor cores (TF32 inputs, FP32 accumulation)
    against the FP64 product; tolerance from the TF32 unit roundoff 2^-11.
    aligned: ldc a multiple of 4 floats, which selects the persistent TMA
    pipeline (edge tiles exercise its clipped stores); otherwise the
    one-tile-per-CTA kernel."""
    import ctypes as C
    lib = ctx.lib
    lib.kd_tf32_gemm_update.restype = C.c_int
    lib.kd_tf32_gemm_update.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p,
                                        C.c_longlong, C.c_void_p, C.c_longlong]
    rng = np.random.default_rng(m * 7 + n + k)
    lda, ldb = m + 3, k + 1
    ldc = ((m + 3) // 4) * 4 + 4 if aligned else m + 5
    A = rng.standard_normal((k, lda)).astype(np.float32)  # column-major storage: column c at A[c]
    B = rng.standard_normal((n, ldb)).astype(np.float32)
    Cm = rng.standard_normal((n, ldc)).astype(np.float32)
    dA = torch.tensor(A, device="cuda")
    dB = torch.tensor(B, device="cuda")
    dC = torch.tensor(Cm, device="cuda")
    torch.cuda.synchronize()
    st = lib.kd_tf32_gemm_update(ctx.h, m, n, k, dA.data_ptr(), lda, dB.data_ptr(), ldb, dC.data_ptr(), ldc)
    assert st == 0, lib.kd_last_error(ctx.h)
    ctx.synchronize()
    got = dC.cpu().numpy()
    Am = A[:, :m].T.astype(np.float64)          # m x k
    Bm = B[:, :k].T.astype(np.float64)          # k x n
    ref = Cm[:, :m].T.astype(np.float64) - Am @ Bm
    err = np.abs(got[:, :m].T - ref).max()
    scale = np.abs(Am).max() * np.abs(Bm).max() * k
    assert err <= 4 * 2.0 ** -11 * scale, (err, scale)
    # padding rows beyond m (ldc > m) untouched
    assert np.array_equal(got[:, m:], Cm[:, m:])


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 384, 96), (200, 130, 96), (1000, 777, 64), (2000, 1500, 96),
                                   (1000, 777, 128), (300, 200, 160), (2000, 1500, 192)])
def test_tcgen05_3xtf32_update_is_fp32_accurate(ctx, m, n, k):
    """3xTF32 (hi/lo split of both operands, three tensor-core products) is
    about FP32 accurate: error bound 2^-17 * max|A| max|B| k, 256 times
    tighter than the plain TF32 bound of the test above."""
    import ctypes as C
    lib = ctx.lib
    lib.kd_tf32x3_gemm_update.restype = C.c_int
    lib.kd_tf32x3_gemm_update.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong,
                                          C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong]
    rng = np.random.default_rng(m * 11 + n + k)
    lda, ldb, ldc = m + 3, k + 1, m + 4
    A = rng.standard_normal((k, lda)).astype(np.float32)
    B = rng.standard_normal((n, ldb)).astype(np.float32)
    Cm = rng.standard_normal((n, ldc)).astype(np.float32)
    dA, dB, dC = (torch.tensor(x, device="cuda") for x in (A, B, Cm))
    torch.cuda.synchronize()
    st = lib.kd_tf32x3_gemm_update(ctx.h, m, n, k, dA.data_ptr(), lda, dB.data_ptr(), ldb, dC.data_ptr(), ldc)
    assert st == 0, lib.kd_last_error(ctx.h)
    ctx.synchronize()
    got = dC.cpu().numpy()
    Am = A[:, :m].T.astype(np.float64)
    Bm = B[:, :k].T.astype(np.float64)
    ref = Cm[:, :m].T.astype(np.float64) - Am @ Bm
    err = np.abs(got[:, :m].T - ref).max()
    scale = np.abs(Am).max() * np.abs(Bm).max() * k
    assert err <= 2.0 ** -17 * scale, (err, scale)
    assert np.array_equal(got[:, m:], Cm[:, m:])


def test_tcgen05_3xtf32_rejects_unaligned(ctx):
    import ctypes as C
    lib = ctx.lib
    lib.kd_tf32x3_gemm_update.restype = C.c_int
    lib.kd_tf32x3_gemm_update.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong,
                                          C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong]
    dA = torch.zeros(64 * 64, device="cuda")
    dC = torch.zeros(64 * 70, device="cuda")
    st = lib.kd_tf32x3_gemm_update(ctx.h, 62, 64, 32, dA.data_ptr(), 64, dA.data_ptr(), 64, dC.data_ptr(), 70)
    assert st == 6  # KD_ERR_UNSUPPORTED: ldc not a multiple of 4
