"""The residual's value pass and the Jacobian's seed passes replayed from
CUDA graphs: Newton iterates and Jacobians identical to the bit with and
without the graphs, captures only on a state seen before, replays
afterwards (also across solves that clear the tangent cache, as the
benchmark does); a system with an integral equation is never captured."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(make, graph, solves=3, precision=1e-10, clear_cache=False):
    wl = make()
    wl.syst.graph_capture = graph
    errs, sols = [], []
    for _ in range(solves):
        wl.restore()
        if clear_cache:
            wl.syst.cache_tangents(False)
            wl.syst.cache_tangents(True)
        for it in range(20):
            done, err = wl.syst.do_newton(precision)
            errs.append(err)
            if done:
                break
        assert done
        sols.append(wl.download())
    return wl, errs, sols


@pytest.mark.parametrize("which", ["star", "ns_tov", "star_vector"])
def test_graph_replay_is_bitwise_identical(ctx, which):
    from kadath_frontera_gb300 import workloads as W
    res = (9, 5, 4)
    make = {"star": lambda: W.star(res, ctx=ctx), "ns_tov": lambda: W.ns_tov(res, ctx=ctx),
            "star_vector": lambda: W.star_vector(res, ctx=ctx)}[which]
    wa, ea, sa = _run(make, True)
    wb, eb, sb = _run(make, False)
    assert ea == eb
    for xa, xb in zip(sa, sb):
        for fa, fb in zip(xa, xb):
            for a, b in zip(fa, fb):
                assert np.array_equal(a, b)
    captures, replays = wa.syst.graph_stats()
    assert captures >= 1 and replays >= 2
    assert wb.syst.graph_stats() == (0, 0)
    jc, jr = wa.syst.jacobian_graph_stats()
    assert jc >= 1 and jr >= 1
    assert wb.syst.jacobian_graph_stats() == (0, 0)


@pytest.mark.parametrize("which", ["star", "star_vector"])
def test_jacobian_graph_across_solves_that_clear_the_tangent_cache(ctx, which):
    """Four solves from the initial guess, the tangent cache cleared before
    each (the first step of a solve fills it, the later steps use it): the
    graphs of both kinds of pass are captured once and replayed; every
    error and every solution is bitwise the one without graphs."""
    from kadath_frontera_gb300 import workloads as W
    res = (9, 5, 4)
    make = {"star": lambda: W.star(res, ctx=ctx), "star_vector": lambda: W.star_vector(res, ctx=ctx)}[which]
    wa, ea, sa = _run(make, True, solves=4, clear_cache=True)
    wb, eb, sb = _run(make, False, solves=4, clear_cache=True)
    assert ea == eb
    for xa, xb in zip(sa, sb):
        for fa, fb in zip(xa, xb):
            for a, b in zip(fa, fb):
                assert np.array_equal(a, b)
    jc, jr = wa.syst.jacobian_graph_stats()
    assert 1 <= jc <= 3 and jr >= 4


def test_replayed_jacobian_is_bitwise_the_assembled_one(ctx):
    """One state's Jacobian assembled three times into the same device
    buffer (as it is, captured, replayed), twice with the tangent cache
    full, then with it cleared: every copy equals the first to the bit."""
    import torch
    from kadath_frontera_gb300 import kadath as KD
    from kadath_frontera_gb300 import workloads as W
    wl = W.star((9, 5, 4), ctx=ctx)
    wl.syst.graph_capture = True
    wl.syst.do_newton(1e-10)  # turns the graphs on; a non-trivial iterate
    n = wl.syst.get_nbr_unknowns()
    dJ = torch.empty(n * n, dtype=torch.float64, device="cuda")
    out = []
    for clear in (False, False, False, True, True, True):
        if clear:
            wl.syst.cache_tangents(False)
            wl.syst.cache_tangents(True)
        dJ.fill_(float("nan"))
        torch.cuda.synchronize()
        ctx.check(KD._L().kd_system_jacobian_device(wl.syst.h, dJ.data_ptr(), n))
        out.append(dJ.cpu().numpy().copy())
    c, r = wl.syst.jacobian_graph_stats()
    assert c >= 1 and r >= 2
    for j in out[1:]:
        assert np.array_equal(j, out[0])


def test_integral_equation_systems_are_not_captured(ctx):
    import math
    from kadath_frontera_gb300.kadath import CHEB_TYPE, OUTER_BC, Scalar, Space_spheric, System_of_eqs
    space = Space_spheric(CHEB_TYPE, (0, 0, 0), (9, 5, 4), (1.0, 2.0))
    u = Scalar(space)
    for d in range(space.get_nbr_domains()):
        r = space.get_radius(d)
        u.set_domain(d, (1 - 0.9 * r ** 2) if d == 0 else np.zeros_like(r))
    u.std_base()
    syst = System_of_eqs(space, 0, 0)
    syst.add_var("u", u)
    syst.add_var("lam", 9.0)
    syst.add_cst("pi", math.pi)
    syst.add_eq_inside(0, "Lap(u) + lam*u = 0")
    syst.add_eq_bc(0, OUTER_BC, "u = 0")
    syst.add_eq_int_volume(0, 0, "integvolume(u) = 4/pi")
    syst.graph_capture = True
    for it in range(12):
        done, err = syst.do_newton(1e-11)
        if done:
            break
    assert done
    assert abs(syst.get_var_double("lam") - math.pi ** 2) < 1e-9
    assert syst.graph_stats() == (0, 0)
