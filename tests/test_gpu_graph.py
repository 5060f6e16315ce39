"""The residual's value pass replayed from a CUDA graph: Newton iterates
identical to the bit with and without the graph, captures only on a state
seen before, replays afterwards; a system with an integral equation is
never captured."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(make, graph, solves=3, precision=1e-10):
    from kadath_frontera_gb300 import workloads as W
    wl = make()
    wl.syst.graph_capture = graph
    errs, sols = [], []
    for _ in range(solves):
        wl.restore()
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
