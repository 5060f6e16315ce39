"""Static pivoting in the mixed-precision LU: a factorisation reuses the pivot
order of the last partial-pivoting one (rows gathered in that order, no row
search), GMRES-IR against the FP64 matrix restores the accuracy, and a bad
order falls back to partial pivoting."""
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


def first_pivot_row(A):
    """Row chosen first by partial pivoting of the equilibrated FP32 copy:
    row scales 2^-round(log2 max_j |A_ij|) (powers of two), then the largest
    scaled entry of column 0, lowest row on ties."""
    m = np.abs(A).max(axis=1)
    _, e = np.frexp(m)
    r = np.ldexp(1.0, 1 - e)
    col = np.abs(r * A[:, 0])
    return int(np.argmax(col))


def solve_with(lu, M, b, mode):
    n = M.shape[0]
    dM = torch.tensor(M.T.copy(), device="cuda")
    db = torch.tensor(b, device="cuda")
    lu.factor(dM.data_ptr(), n, n, mode)
    lu.solve(db.data_ptr())
    return db.cpu().numpy(), lu.pivot_info()


@pytest.mark.parametrize("n", [500, 1300])
def test_reused_order_solves_a_nearby_matrix(ctx, n):
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    A = make(n, 1e4, 1)
    B = A + 1e-3 * make(n, 10.0, 2)
    b = np.random.default_rng(3).standard_normal(n)
    lu = DenseLU(ctx)
    lu.set_pivot_reuse(True)
    x, info = solve_with(lu, A, b, KD_LU_TF32_IR)
    assert info == (False, False)  # the first factorisation pivots
    x, info = solve_with(lu, B, b, KD_LU_TF32_IR)
    assert info == (True, False)
    assert np.linalg.norm(B @ x - b) / np.linalg.norm(b) < 1e-12


def test_zero_pivot_in_the_reused_order_falls_back(ctx):
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 700
    A = make(n, 1e3, 4)
    b = np.random.default_rng(5).standard_normal(n)
    lu = DenseLU(ctx)
    lu.set_pivot_reuse(True)
    solve_with(lu, A, b, KD_LU_TF32_IR)
    B = A.copy()
    B[first_pivot_row(A), 0] = 0.0  # the reused order now starts on a zero pivot
    x, info = solve_with(lu, B, b, KD_LU_TF32_IR)
    assert info == (False, True)
    assert np.linalg.norm(B @ x - b) / np.linalg.norm(b) < 1e-12


def test_tiny_pivot_in_the_reused_order_falls_back(ctx):
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 700
    A = make(n, 1e3, 6)
    b = np.random.default_rng(7).standard_normal(n)
    lu = DenseLU(ctx)
    lu.set_pivot_reuse(True)
    solve_with(lu, A, b, KD_LU_TF32_IR)
    B = A.copy()
    B[first_pivot_row(A), 0] *= 1e-30  # no exact zero: the elimination blows up instead
    x, info = solve_with(lu, B, b, KD_LU_TF32_IR)
    assert info[1]
    assert np.linalg.norm(B @ x - b) / np.linalg.norm(b) < 1e-12


def test_newton_with_static_pivots_matches_fp64_iterates(ctx):
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_FP64, KD_LU_TF32_IR
    ref = workloads.star((9, 5, 4))
    mixed = workloads.star((9, 5, 4))
    nd = ref.space.get_nbr_domains()
    used = []
    for it in range(8):
        d_ref, _ = ref.syst.do_newton(1e-10, lu_mode=KD_LU_FP64)
        d_mix, _ = mixed.syst.do_newton(1e-10, lu_mode=KD_LU_TF32_IR)
        assert d_ref == d_mix
        if d_ref:
            break
        used.append(mixed.syst.last_report["static_pivots"])
        for (_, f), (_, g) in zip(ref.unknowns, mixed.unknowns):
            for d in range(nd):
                a, b = g.get_coef(d), f.get_coef(d)
                assert np.linalg.norm(a - b) <= 1e-10 * max(np.linalg.norm(b), 1e-300)
    assert d_ref
    assert used[0] == 0 and all(used[1:]) and len(used) >= 2


def test_static_factors_precondition_as_well_as_pivoted_ones_at_the_timed_size(ctx):
    """The star at (13, 9, 4), N = 12,331, solved three times: every later
    step factors with the kept pivot order (192-column panels, the trailing
    update on a side stream beside the next panel) and its refinement needs
    at most 4 iterations more than the pivoted first step's; factors spoilt
    by a race between the two streams' updates would need many more (and
    the step would then drop the order)."""
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_TF32_IR
    wl = workloads.star(ctx=ctx)
    for _ in range(3):
        wl.restore()
        wl.syst.reset_pivot_order()
        reps = []
        for _ in range(10):
            done, _ = wl.syst.do_newton(1e-10, lu_mode=KD_LU_TF32_IR)
            if done:
                break
            reps.append(dict(wl.syst.last_report))
        assert done and len(reps) >= 2
        first = reps[0]["refine_iters"]
        assert reps[0]["static_pivots"] == 0
        for r in reps[1:]:
            assert r["static_pivots"] == 1
            assert r["refine_iters"] <= first + 4, (first, [x["refine_iters"] for x in reps])
