"""Save files in Kadath's binary format (GPU): the product's files parsed by
the oracle's restatement of the format, the oracle's files read by the
product, and save -> load round trips of a converged star (space, scalars,
the shift as a Cartesian vector) that resume the Newton iteration where it
stopped."""
import numpy as np
import pytest

from oracle import configs, kadath as K, kadath_io as KIO

pytestmark = pytest.mark.gpu


def test_product_files_match_the_format(ctx, tmp_path):
    from kadath_frontera_gb300 import workloads as W
    from kadath_frontera_gb300.kadath import KadathFile
    wl = W.star((9, 5, 4), ctx=ctx)
    wl.syst.do_newton(1e-10)  # fields now hold coefficients as well
    path = tmp_path / "star.dat"
    with KadathFile(path, "w") as f:
        wl.space.save(f)
        for _, fld in wl.unknowns:
            fld.save(f)
    doms, _, _, _ = configs.star((9, 5, 4))
    with open(path, "rb") as fp:
        sp = KIO.read_space(fp)
        assert len(sp) == len(doms)
        for a, d in zip(sp, doms):
            assert a["type"] == d.type and a["np"] == d.np and a["nc"] == d.nc
            assert a["alpha"] == d.alpha and a["beta"] == d.beta
        for _, fld in wl.unknowns:
            vals = KIO.read_scalar(fp, sp)
            for dd, (base, zero, conf, coef) in enumerate(vals):
                r, t, p = fld.get_base(dd)
                assert np.array_equal(base[0], r) and np.array_equal(base[1], t) and base[2] == p
                assert not zero and (conf is not None or coef is not None)
                # each representation the field holds, as it holds it
                if conf is not None:
                    assert np.array_equal(conf, fld.get_domain(dd))
                if coef is not None:
                    assert np.array_equal(coef.reshape(-1), fld.get_coef(dd).reshape(-1))
        assert fp.read() == b""


def test_oracle_files_are_read(ctx, tmp_path):
    from kadath_frontera_gb300.kadath import KadathFile, Scalar, Space_spheric
    doms = K.space_spheric((9, 5, 4), [1.0, 2.5])
    f = K.scalar_field(doms, lambda d: np.cos(0.3 * d.radius()) if d.type != K.COMPACT else np.zeros(d.np))
    for d in doms:
        f[d.num].coef()
    path = tmp_path / "oracle.dat"
    with open(path, "wb") as fp:
        KIO.write_space(fp, doms)
        KIO.write_scalar(fp, doms, f)
    with KadathFile(path, "r") as kf:
        space = Space_spheric.from_file(kf, ctx=ctx)
        s = Scalar.from_file(space, kf)
    assert space.get_nbr_domains() == 3
    for d in doms:
        info = space.domain_info(d.num)
        assert info["alpha"] == d.alpha and info["beta"] == d.beta
        assert np.array_equal(s.get_coef(d.num).reshape(-1), f[d.num].cf[0].reshape(-1))


def test_save_load_resumes_the_solve(ctx, tmp_path):
    """A vector star stopped after two Newton steps, saved, read back into a
    new system: the next steps give the same iterates as continuing."""
    from kadath_frontera_gb300 import workloads as W
    from kadath_frontera_gb300.kadath import KadathFile, Scalar, Space_spheric, Vector
    res = (9, 5, 4)
    a = W.star_vector(res, ctx=ctx)
    for _ in range(2):
        a.syst.do_newton(1e-12)
    path = tmp_path / "stop.dat"
    P, NP = a.unknowns[0][1], a.unknowns[1][1]
    bet = Vector(a.space)
    bet.cmp = [a.unknowns[2][1], a.unknowns[3][1], a.unknowns[4][1]]
    with KadathFile(path, "w") as f:
        a.space.save(f)
        P.save(f)
        NP.save(f)
        bet.save(f)
    with KadathFile(path, "r") as f:
        space = Space_spheric.from_file(f, ctx=ctx)
        P2 = Scalar.from_file(space, f)
        NP2 = Scalar.from_file(space, f)
        bet2 = Vector.from_file(space, f)
    assert bet2.type_index == 1
    b = W.star_vector(res, ctx=ctx)
    for (_, src), dst in zip(a.unknowns, [P2, NP2] + bet2.cmp):
        for d in range(space.get_nbr_domains()):
            assert np.array_equal(src.get_coef(d), dst.get_coef(d))
    # the loaded fields belong to another space object: copy them through
    # their coefficients into the second system's fields
    for (_, dst), src in zip(b.unknowns, [P2, NP2] + bet2.cmp):
        for d in range(space.get_nbr_domains()):
            dst.set_domain(d, src.get_domain(d))
    for _ in range(3):
        ea = a.syst.do_newton(1e-12)
        eb = b.syst.do_newton(1e-12)
        assert abs(ea[1] - eb[1]) <= 1e-12 * max(1.0, ea[1])
