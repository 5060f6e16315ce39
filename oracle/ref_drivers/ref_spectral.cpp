// Golden-vector driver over the reference's 1-D spectral routines.
//
// Test infrastructure only (built by oracle/Makefile.ref into oracle/_ref/).
// Each input line "OP BASE LINE N_IN N_OUT" asks for the matrix of one 1-D
// routine of the reference applied to a work line of LINE doubles:
//   OP 0: coef_1d   (src/Coef/coef_1d.cpp:607)
//   OP 1: coef_i_1d (src/Coef/coef_i_1d.cpp:527)
//   OP 2..12: der_1d, mult_sin_1d, div_sin_1d, mult_cos_1d, div_cos_1d,
//             mult_x_1d, div_x_1d, mult_xm1_1d, div_xm1_1d, div_xp1_1d,
//             div_1mx2_1d (src/Ope_1d/*.cpp)
// Column c is the routine applied to the unit vector e_c (c < N_IN, zero
// padded to LINE), read in its first N_OUT slots.  The output, on stdout, is
// one line per request: the output basis the routine returned (the input
// basis for the transforms) followed by the N_OUT x N_IN matrix, row-major,
// printed with 17 significant digits.
#include <cstdio>
#include <iostream>
#include <string>

#include "kadath.hpp"

namespace Kadath {
void coef_1d(int, Array<double>&);
void coef_i_1d(int, Array<double>&);
int der_1d(int, Array<double>&);
int mult_sin_1d(int, Array<double>&);
int div_sin_1d(int, Array<double>&);
int mult_cos_1d(int, Array<double>&);
int div_cos_1d(int, Array<double>&);
int mult_x_1d(int, Array<double>&);
int div_x_1d(int, Array<double>&);
int mult_xm1_1d(int, Array<double>&);
int div_xm1_1d(int, Array<double>&);
int div_xp1_1d(int, Array<double>&);
int div_1mx2_1d(int, Array<double>&);
}  // namespace Kadath

using namespace Kadath;

int main() {
  int op, base, line, nin, nout;
  while (std::cin >> op >> base >> line >> nin >> nout) {
    if (nin > line || nout > line || op < 0 || op > 12) {
      std::cerr << "ref_spectral: bad request" << std::endl;
      return 2;
    }
    std::vector<double> m(static_cast<size_t>(nout) * nin);
    int out_base = base;
    for (int c = 0; c < nin; c++) {
      Array<double> t(line);
      for (int i = 0; i < line; i++) t.set(i) = (i == c) ? 1.0 : 0.0;
      switch (op) {
        case 0: coef_1d(base, t); break;
        case 1: coef_i_1d(base, t); break;
        case 2: out_base = der_1d(base, t); break;
        case 3: out_base = mult_sin_1d(base, t); break;
        case 4: out_base = div_sin_1d(base, t); break;
        case 5: out_base = mult_cos_1d(base, t); break;
        case 6: out_base = div_cos_1d(base, t); break;
        case 7: out_base = mult_x_1d(base, t); break;
        case 8: out_base = div_x_1d(base, t); break;
        case 9: out_base = mult_xm1_1d(base, t); break;
        case 10: out_base = div_xm1_1d(base, t); break;
        case 11: out_base = div_xp1_1d(base, t); break;
        case 12: out_base = div_1mx2_1d(base, t); break;
      }
      for (int r = 0; r < nout; r++) m[static_cast<size_t>(r) * nin + c] = t(r);
    }
    std::printf("%d", out_base);
    for (double v : m) std::printf(" %.17g", v);
    std::printf("\n");
  }
  return 0;
}
