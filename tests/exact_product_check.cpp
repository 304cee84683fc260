// Known-answer check of wg::exact_product (waves_gb300/csrc/exact_product.h) against the FP64
// multiply: random bit patterns (every class of float), uniform values and special values; exits
// non-zero on the first mismatching bit pattern.  Built and run by tests/test_cpu_exact_product.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "../waves_gb300/csrc/exact_product.h"

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(7);
  long bad = 0;
  auto check = [&](float a, float b) {
    const double x = wg::exact_product(a, b), y = (double)a * (double)b;
    uint64_t bx, by;
    std::memcpy(&bx, &x, 8);
    std::memcpy(&by, &y, 8);
    if (bx != by && !(std::isnan(x) && std::isnan(y))) {
      if (bad++ < 3) std::printf("mismatch %a * %a: %a vs %a\n", a, b, x, y);
    }
  };
  for (long k = 0; k < n; k++) {
    const uint32_t u = (uint32_t)g(), v = (uint32_t)g();
    float a, b;
    std::memcpy(&a, &u, 4);
    std::memcpy(&b, &v, 4);
    check(a, b);
  }
  std::uniform_real_distribution<float> d(-1e4f, 1e4f);
  for (long k = 0; k < n; k++) check(d(g), d(g));
  const float sp[] = {0.f, -0.f, 1.f, -1.f, 1.17549435e-38f, 1.4e-45f, 3.4028235e38f, INFINITY, -INFINITY, NAN,
                      1.9999999f, 1.5f, 0.75f, 1e-20f};
  for (float a : sp)
    for (float b : sp) check(a, b);
  std::printf("%ld mismatches\n", bad);
  return bad != 0;
}
