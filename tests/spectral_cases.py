"""Domain shapes and basis tables shared by the transform tests (the bases of
Domain_{nucleus,shell,compact}::set_cheb_base / set_anti_cheb_base,
src/Domain/Spheric/domain_shell.cpp:288, domain_nucleus.cpp:229-263)."""
import numpy as np

from oracle import spectral as S


def std_base(kind, nc1, nc2, anti=False):
    base_t = []
    base_r = [[0] * nc2 for _ in range(nc1)]
    for k in range(nc2):
        m = k // 2
        if not anti:
            base_t.append(S.COS_EVEN if m % 2 == 0 else S.SIN_ODD)
        else:
            base_t.append(S.COS_ODD if m % 2 == 0 else S.SIN_EVEN)
        for j in range(nc1):
            if kind == "nucleus":
                even = (m % 2 == 0) != anti
                base_r[j][k] = S.CHEB_EVEN if even else S.CHEB_ODD
            else:
                base_r[j][k] = S.CHEB
    return base_r, base_t, S.COSSIN


SHAPES = [("nucleus", (13, 7, 4)), ("shell", (13, 7, 4)), ("compact", (13, 7, 4)),
          ("nucleus", (13, 9, 4)), ("shell", (11, 9, 8)), ("compact", (17, 9, 4)), ("shell", (9, 5, 1))]
