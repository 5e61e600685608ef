// facade_check.cpp -- exercises the C++ facade (include/fidibench_gb/Upwind.h)
// beyond the reference's members: advectHostStream against the serial
// setInitialCondition / advect / getField / checksum sequence (bit for bit),
// advectTransposed against the dL/df0-only adjoint (bit for bit) with the
// field untouched, and the dot-product identity <A x, y> = <x, A^T y>.
// Prints "facade ok" and exits 0 when every check holds.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "fidibench_gb/Upwind.h"

static int failures = 0;
#define CHECK(cond, what)                           \
  do {                                              \
    if (!(cond)) {                                  \
      std::printf("FAILED: %s\n", what);            \
      ++failures;                                   \
    }                                               \
  } while (0)

int main() {
  const std::vector<double> v = {0.8, -0.45, 0.3}, L = {1.0, 1.2, 0.9};
  const std::vector<size_t> n = {40, 33, 57};
  const double dt = 0.4 * std::fmin(std::fmin(1.0 / 40 / 0.8, 1.2 / 33 / 0.45), 0.9 / 57 / 0.3);
  const int steps = 13, count = 3;
  fdb::Upwind<3> up(v, L, n);
  const size_t N = up.size();
  std::mt19937_64 rng(7);
  std::normal_distribution<double> nd;
  std::vector<std::vector<double>> fields(count, std::vector<double>(N));
  for (auto& f : fields)
    for (auto& x : f) x = nd(rng);

  // serial reference
  std::vector<std::vector<double>> ref(count);
  std::vector<double> ref_sums(count);
  for (int k = 0; k < count; ++k) {
    up.setInitialCondition(fields[k]);
    up.advect(steps, dt);
    ref[k] = up.getField();
    ref_sums[k] = up.checksum();
  }
  // streamed, in place
  std::vector<std::vector<double>> work = fields;
  std::vector<double*> ptrs;
  for (auto& f : work) ptrs.push_back(f.data());
  const std::vector<double> sums = up.advectHostStream(ptrs, steps, dt);
  for (int k = 0; k < count; ++k) {
    CHECK(work[k] == ref[k], "advectHostStream result equals the serial cycle");
    CHECK(sums[k] == ref_sums[k], "advectHostStream checksum equals the serial checksum");
  }
  CHECK(up.getField() == ref[count - 1], "the handle holds the last result");

  // transposed advect: field untouched, equal to the dL/df0-only adjoint
  std::vector<double> y(N);
  for (auto& x : y) x = nd(rng);
  const std::vector<double> before = up.getField();
  const std::vector<double> aty = up.advectTransposed(steps, dt, y);
  CHECK(up.getField() == before, "advectTransposed leaves the field");
  up.setInitialCondition(fields[0]);
  const std::vector<double> g0 = up.adjoint(steps, dt, y);
  CHECK(g0 == aty, "advectTransposed equals the dL/df0-only adjoint");
  // <A x, y> = <x, A^T y> with x = fields[0]
  long double lhs = 0.0L, rhs = 0.0L;
  for (size_t i = 0; i < N; ++i) {
    lhs += (long double)ref[0][i] * y[i];
    rhs += (long double)fields[0][i] * aty[i];
  }
  CHECK(std::fabs((double)(lhs - rhs)) <= 1e-11 * std::fabs((double)lhs),
        "dot-product identity");
  // the OpenACC variants' constructor (std::vector<int>, product coefficient
  // form) and their one-step advect(double): under EXACT, S one-step calls
  // give the field of one advect(S, dt) call bit for bit
  {
    const std::vector<int> ni = {16, 12, 20};
    const double dt2 = 0.1 / 20;
    fdb::Upwind<3> a(v, L, ni), b(v, L, ni);
    a.setArith(FDB_ARITH_EXACT);
    b.setArith(FDB_ARITH_EXACT);
    for (int s = 0; s < 7; ++s) a.advect(dt2);
    b.advect(7, dt2);
    CHECK(a.getField() == b.getField(), "advect(double) x 7 equals advect(7, double)");
    CHECK(a.size() == (size_t)16 * 12 * 20, "std::vector<int> constructor sizes the field");
    std::vector<size_t> ns(ni.begin(), ni.end());
    fdb::Upwind<3> c(v, L, ns);
    c.setArith(FDB_ARITH_EXACT);
    c.advect(7, dt2);
    const std::vector<double> fa = a.getField(), fc = c.getField();
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < fa.size(); ++i) {
      num = std::fmax(num, std::fabs(fa[i] - fc[i]));
      den = std::fmax(den, std::fabs(fc[i]));
    }
    CHECK(num <= 1e-14 * den, "the two coefficient forms differ by rounding only");
  }
  if (failures) return 1;
  std::printf("facade ok\n");
  return 0;
}
