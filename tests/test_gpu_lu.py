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
