"""Failure paths of the solver, made to happen without faulting the GPU.

* A grid-barrier wait that runs out: the context's wait limit is set to 1 ms
  and kd_ctx_stall_waits raises every barrier target by one, so that no
  barrier of the LU panel or of the triangular sweeps completes.  The call
  must return KD_ERR_TIMEOUT, and the same context must then factor and
  solve correctly.
* A refinement that does not converge: a matrix with condition number 1e12,
  whose FP32 factors are no preconditioner, and GMRES(2) with two cycles:
  KD_ERR_NOCONV.
* A Newton step whose mixed solve does not converge (one GMRES iteration,
  one cycle) is solved again with the FP64 LU of the same Jacobian, and the
  iterates are those of the FP64 path.
* NaN in the fields: do_newton reports a non-finite residual (KD_ERR_ARG)
  and makes no update; with the fields restored the solve proceeds."""
import math

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


def _status(exc):
    return exc.value.status


def test_panel_barrier_wait_runs_out_and_context_recovers(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300._lib import KD_ERR_TIMEOUT
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_FP64
    n = 700
    A = make(n, 1e4, 3)
    b = np.random.default_rng(4).standard_normal(n)
    lu = DenseLU(ctx)
    dA = torch.tensor(A.T.copy(), device="cuda")
    ctx.set_wait_limit(1e-3)
    ctx.stall_waits(True)
    try:
        with pytest.raises(KadathError) as e:
            lu.factor(dA.data_ptr(), n, n, KD_LU_FP64)
        assert _status(e) == KD_ERR_TIMEOUT
        assert "grid barrier" in str(e.value)
    finally:
        ctx.stall_waits(False)
        ctx.set_wait_limit(2.0)
    dA = torch.tensor(A.T.copy(), device="cuda")
    db = torch.tensor(b, device="cuda")
    lu.factor(dA.data_ptr(), n, n, KD_LU_FP64)
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12


def test_sweep_barrier_wait_runs_out_and_context_recovers(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300._lib import KD_ERR_TIMEOUT
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 900
    A = make(n, 1e4, 5)
    b = np.random.default_rng(6).standard_normal(n)
    lu = DenseLU(ctx)
    dA = torch.tensor(A.T.copy(), device="cuda")
    lu.factor(dA.data_ptr(), n, n, KD_LU_TF32_IR)
    db = torch.tensor(b, device="cuda")
    ctx.set_wait_limit(1e-3)
    ctx.stall_waits(True)
    try:
        with pytest.raises(KadathError) as e:
            lu.solve(db.data_ptr())
        assert _status(e) == KD_ERR_TIMEOUT
    finally:
        ctx.stall_waits(False)
        ctx.set_wait_limit(2.0)
    db = torch.tensor(b, device="cuda")
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12


def test_cluster_panel_exchange_wait_runs_out_and_context_recovers(ctx):
    """The partial-pivoting panel of the mixed modes runs on a thread-block
    cluster and exchanges each column's candidates by asynchronous stores
    that complete on the receivers' mbarriers.  With stall_waits every
    exchange expects bytes that never come: each wait runs out after the
    context's limit, the factorisation reports KD_ERR_TIMEOUT, and the same
    context then factors and solves correctly."""
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300._lib import KD_ERR_TIMEOUT
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 900
    A = make(n, 1e4, 7)
    b = np.random.default_rng(8).standard_normal(n)
    lu = DenseLU(ctx)
    dA = torch.tensor(A.T.copy(), device="cuda")
    ctx.set_wait_limit(1e-3)
    ctx.stall_waits(True)
    try:
        with pytest.raises(KadathError) as e:
            lu.factor(dA.data_ptr(), n, n, KD_LU_TF32_IR)
        assert _status(e) == KD_ERR_TIMEOUT
    finally:
        ctx.stall_waits(False)
        ctx.set_wait_limit(2.0)
    dA = torch.tensor(A.T.copy(), device="cuda")
    db = torch.tensor(b, device="cuda")
    lu.factor(dA.data_ptr(), n, n, KD_LU_TF32_IR)
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12


def test_refinement_that_cannot_converge_reports_noconv(ctx):
    from kadath_frontera_gb300 import KadathError
    from kadath_frontera_gb300._lib import KD_ERR_NOCONV
    from kadath_frontera_gb300.kadath import DenseLU, KD_LU_TF32_IR
    n = 512
    A = make(n, 1e12, 7)
    b = np.random.default_rng(8).standard_normal(n)
    dA = torch.tensor(A.T.copy(), device="cuda")
    db = torch.tensor(b, device="cuda")
    lu = DenseLU(ctx)
    lu.set_refinement(1e-14, 2, 2)
    lu.factor(dA.data_ptr(), n, n, KD_LU_TF32_IR)
    with pytest.raises(KadathError) as e:
        lu.solve(db.data_ptr())
    assert _status(e) == KD_ERR_NOCONV
    assert lu.stats()["rel_residual"] > 1e-10
    # the same LU object solves a well-conditioned system afterwards
    lu.set_refinement()
    B = make(n, 1e3, 9)
    dB = torch.tensor(B.T.copy(), device="cuda")
    lu.factor(dB.data_ptr(), n, n, KD_LU_TF32_IR)
    db = torch.tensor(b, device="cuda")
    lu.solve(db.data_ptr())
    x = db.cpu().numpy()
    assert np.linalg.norm(B @ x - b) / np.linalg.norm(b) < 1e-12


def test_newton_falls_back_to_fp64_when_refinement_fails(ctx):
    from kadath_frontera_gb300 import workloads
    from kadath_frontera_gb300.kadath import KD_LU_FP64, KD_LU_TF32_IR
    ref = workloads.star((9, 5, 4))
    mixed = workloads.star((9, 5, 4))
    nd = ref.space.get_nbr_domains()
    fallbacks = 0
    for it in range(8):
        d_ref, e_ref = ref.syst.do_newton(1e-10, lu_mode=KD_LU_FP64)
        d_mix, e_mix = mixed.syst.do_newton(1e-10, lu_mode=KD_LU_TF32_IR, max_refine=1, gmres_restarts=1)
        assert d_ref == d_mix
        if d_ref:
            break
        fallbacks += mixed.syst.last_report["fp64_fallback"]
        for (_, f), (_, g) in zip(ref.unknowns, mixed.unknowns):
            for d in range(nd):
                a, b = g.get_coef(d), f.get_coef(d)
                assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1.0)
    assert d_ref
    assert fallbacks >= 1


def test_nan_in_the_fields_is_reported_without_update(ctx):
    from kadath_frontera_gb300 import KadathError, workloads
    from kadath_frontera_gb300._lib import KD_ERR_ARG
    wl = workloads.toy()
    psi = wl.unknowns[0][1]
    good = psi.get_domain(1).copy()
    bad = good.copy()
    bad[3, 2, 1] = math.nan
    psi.set_domain(1, bad)
    psi.std_base()
    with pytest.raises(KadathError) as e:
        wl.syst.do_newton(1e-10)
    assert _status(e) == KD_ERR_ARG
    assert "non-finite" in str(e.value)
    assert np.isnan(psi.get_domain(1)[3, 2, 1])  # no update was made
    psi.set_domain(1, good)
    psi.std_base()
    for _ in range(8):
        done, err = wl.syst.do_newton(1e-10)
        if done:
            break
    assert done and err < 1e-10
