// Host copy of the f64 2 atanh of the sum-product rule (com-rs_gb300/csrc/atanh2.cuh),
// checked against 2 atanhl in long double: prints the worst error in ulps and the share of
// correctly rounded results over seeded inputs of four kinds (uniform on [-1, 1], small,
// near +-1, products of two tanh), then the bits of the results of special inputs.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "atanh2.cuh"

static double ulp_of(double x) {
  x = std::fabs(x);
  if (x == 0) return 4.9406564584124654e-324;
  int e;
  std::frexp(x, &e);
  return std::fmax(std::ldexp(1.0, e - 53), 4.9406564584124654e-324);
}

int main(int argc, char** argv) {
  const double B = 0.999999999999;
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::atol(argv[2]) : 1);
  std::uniform_real_distribution<double> U(0, 1);
  double worst = 0;
  long cr = 0;
  for (long i = 0; i < n; i++) {
    const int kind = (int)(i % 4);
    const double s = U(g) < 0.5 ? -1.0 : 1.0;
    double p;
    if (kind == 0) p = 2 * U(g) - 1;
    else if (kind == 1) p = s * std::pow(10.0, -16 * U(g));
    else if (kind == 2) p = s * (1 - std::pow(10.0, -12.5 * U(g)));
    else p = std::tanh(30 * U(g)) * std::tanh(30 * U(g)) * s;
    const double mine = at2::twice_atanh(p, B);
    const double pc = p < -B ? -B : (p > B ? B : p);
    const long double ref = 2.0L * atanhl((long double)pc);
    worst = std::fmax(worst, (double)(std::fabs((long double)mine - ref) / ulp_of((double)ref)));
    cr += mine == (double)ref;
  }
  std::printf("%.6f %.8f\n", worst, (double)cr / (double)n);
  const double special[] = {0.0, -0.0, 5e-324, -1e-300, 1e-20, 3.7e-9, 0.5, -0.25, B, -B, 1.0, -1.0, 2.0};
  for (double p : special) std::printf("%a %a\n", p, at2::twice_atanh(p, B));
  return 0;
}
