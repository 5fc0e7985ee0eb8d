// The fast correctly rounded log and sin/cos (com-rs_gb300/csrc/crmath_fast.cuh) against
// the double-double routines of crmath.cuh and against binary128 rounded once, on the
// host: prints the count of inputs, of results that differ from crmath.cuh's in any bit,
// and of results that differ from the binary128 ones, over the noise's arguments (1 - u
// and 2 pi u for seeded u) and hard cases (around 1, around multiples of pi/2 and
// pi/128, powers of two).
#if defined(__aarch64__)
typedef long double quad;  // IEEE binary128 on aarch64 Linux
static quad qlog(quad x) { return logl(x); }
static quad qsin(quad x) { return sinl(x); }
static quad qcos(quad x) { return cosl(x); }
#else
#include <quadmath.h>
typedef __float128 quad;
static quad qlog(quad x) { return logq(x); }
static quad qsin(quad x) { return sinq(x); }
static quad qcos(quad x) { return cosq(x); }
#endif
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "crmath_fast.cuh"

static double step(double a, long d) {
  int64_t b;
  std::memcpy(&b, &a, 8);
  b += d;
  std::memcpy(&a, &b, 8);
  return a;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::atol(argv[2]) : 1);
  long count = 0, diff = 0, diff_q = 0;
  auto log_chk = [&](double x) {
    const double a = crm::cr_log_fast(x), b = crm::cr_log(x), q = (double)qlog((quad)x);
    diff += std::memcmp(&a, &b, 8) != 0;
    diff_q += std::memcmp(&a, &q, 8) != 0;
    count++;
  };
  auto sc_chk = [&](double x) {
    double s1, c1, s2, c2;
    crm::cr_sincos_fast(x, &s1, &c1);
    crm::cr_sincos(x, &s2, &c2);
    const double sq = (double)qsin((quad)x), cq = (double)qcos((quad)x);
    diff += std::memcmp(&s1, &s2, 8) != 0 || std::memcmp(&c1, &c2, 8) != 0;
    diff_q += std::memcmp(&s1, &sq, 8) != 0 || std::memcmp(&c1, &cq, 8) != 0;
    count++;
  };
  for (long i = 0; i < n; i++) {
    const double u = (double)(g() >> 11) * (1.0 / 9007199254740992.0);
    log_chk(1.0 - u);
    sc_chk(6.283185307179586 * u);
  }
  for (long d = -3000; d <= 3000; d++) {
    log_chk(step(1.0, d));
    for (int k = 1; k <= 5; k++) sc_chk(step(k * 1.5707963267948966, d));
  }
  for (int j = 1; j < 330; j++)
    for (long d = -20; d <= 20; d++) sc_chk(step(j * 0.024543692606170259, d));
  for (int e = -1074; e <= 2; e++) {
    log_chk(std::ldexp(1.0, e));
    sc_chk(std::ldexp(1.0, e));
  }
  sc_chk(0.0);
  std::printf("%ld %ld %ld\n", count, diff, diff_q);
  return 0;
}
