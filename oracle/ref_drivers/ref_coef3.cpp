// Golden-vector driver over Base_spectral::coef / coef_i with arbitrary basis
// tables (src/Coef/coef.cpp:28-104, src/Coef/coef_i.cpp:28-104), such as the
// bases of the bispheric domains (src/Domain/Bispheric/
// domain_bispheric_rect.cpp:466-479: COS or SIN in phi, CHEB_EVEN / CHEB_ODD
// in chi by the parity of the phi index, CHEB in eta).
//
// Test infrastructure only (built by oracle/Makefile.ref into oracle/_ref/).
// stdin: "N0 N1 N2 C0 C1 C2" (points, coefficients), the phi basis, the C2
// theta bases (per phi index k), the C1 x C2 radial bases (k outer, j inner:
// basis of the radial line (j, k)), then N0 N1 N2 values and C0 C1 C2
// coefficients in the reference's Array storage order.  stdout: the C0 C1 C2
// numbers of coef(values), then the N0 N1 N2 numbers of coef_i(coefficients),
// 17 significant digits.  The basis tables are handed to the reference
// through its own save format (Base_spectral::save: a definition flag, the
// number of dimensions, then each table by Array<int>::save), which its
// Base_spectral(FILE*) constructor reads.
#include <cstdio>
#include <iostream>
#include <vector>

#include "kadath.hpp"

using namespace Kadath;

int main() {
  int np[3], nc[3];
  if (!(std::cin >> np[0] >> np[1] >> np[2] >> nc[0] >> nc[1] >> nc[2])) return 2;
  int bp;
  std::cin >> bp;
  Array<int> b2(1);
  b2.set(0) = bp;
  Array<int> b1(nc[2]);
  for (int k = 0; k < nc[2]; k++) std::cin >> b1.set(k);
  Dim_array d0(2);
  d0.set(0) = nc[1];
  d0.set(1) = nc[2];
  Array<int> b0(d0);
  Index idx(d0);
  for (int k = 0; k < nc[2]; k++)
    for (int j = 0; j < nc[1]; j++) {
      idx.set(0) = j;
      idx.set(1) = k;
      std::cin >> b0.set(idx);
    }
  FILE* f = std::tmpfile();
  if (!f) return 3;
  int indic = 0, ndim = 3;
  fwrite_be(&indic, sizeof(int), 1, f);
  fwrite_be(&ndim, sizeof(int), 1, f);
  b0.save(f);
  b1.save(f);
  b2.save(f);
  std::rewind(f);
  Base_spectral base(f);
  std::fclose(f);

  Dim_array dp(3), dc(3);
  for (int i = 0; i < 3; i++) {
    dp.set(i) = np[i];
    dc.set(i) = nc[i];
  }
  Array<double> vals(dp), cfs(dc);
  const long npt = static_cast<long>(np[0]) * np[1] * np[2], ncf = static_cast<long>(nc[0]) * nc[1] * nc[2];
  for (long i = 0; i < npt; i++) std::cin >> vals.set_data()[i];
  for (long i = 0; i < ncf; i++) std::cin >> cfs.set_data()[i];
  if (!std::cin) return 4;
  Array<double> c = base.coef(dc, vals);
  Array<double> v = base.coef_i(dp, cfs);
  std::printf("%d\n", 0);
  for (long i = 0; i < ncf; i++) std::printf("%.17g\n", c.get_data()[i]);
  for (long i = 0; i < npt; i++) std::printf("%.17g\n", v.get_data()[i]);
  return 0;
}
