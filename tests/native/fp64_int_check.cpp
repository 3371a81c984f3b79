// CPU check of sdem_gb300/csrc/fp64_int.cuh: the integer-pipe binary64
// addition and multiplication against the host's IEEE arithmetic.
// Usage: fp64_int_check <seed> <pairs per family>; prints "ok <n>" or the
// first mismatches and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <random>

#include "../../sdem_gb300/csrc/fp64_int.cuh"

static uint64_t B(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static double D(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static bool same(double a, double b) {
  if (std::isnan(a) && std::isnan(b)) return true;
  return B(a) == B(b);
}

static long bad = 0, checked = 0;
static void check(double x, double y) {
  const double r[4] = {fpi::add(x, y), fpi::sub(x, y), fpi::mul(x, y), fpi::add(y, x)};
  const double e[4] = {x + y, x - y, x * y, y + x};
  const char* nm[4] = {"add", "sub", "mul", "add(y,x)"};
  for (int k = 0; k < 4; k++) {
    checked++;
    if (!same(r[k], e[k])) {
      if (bad < 20)
        printf("MISMATCH %s x=%a y=%a got=%a want=%a\n", nm[k], x, y, r[k], e[k]);
      bad++;
    }
  }
}

int main(int argc, char** argv) {
  const uint64_t seed = argc > 1 ? strtoull(argv[1], 0, 10) : 1;
  const long n = argc > 2 ? strtol(argv[2], 0, 10) : 1000000;
  std::mt19937_64 g(seed);
  auto u64 = [&]() { return g(); };
  auto mant = [&]() { return g() & fpi::kMant; };
  auto with_exp = [&](uint64_t e) { return D(((g() & 1) << 63) | (e << 52) | mant()); };
  // specials
  const double sp[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                       2.2250738585072009e-308, 1.7976931348623157e308, -1.7976931348623157e308, 0.5, 3.0, 1e-300};
  for (double a : sp)
    for (double b : sp) check(a, b);
  for (long i = 0; i < n; i++) {
    // 1) uniformly random bit patterns (every exponent, specials included)
    check(D(u64()), D(u64()));
    // 2) operands of the physics range (|x| in 1e-12..1e6), close exponents
    {
      uint64_t ea = 983 + g() % 60, eb = ea + (g() % 9) - 4;
      check(with_exp(ea), with_exp(eb));
    }
    // 3) exponent differences 0..70 (alignment, sticky), both signs
    {
      uint64_t ea = 600 + g() % 800, d = g() % 71;
      check(with_exp(ea), with_exp(ea - d));
    }
    // 4) cancellation: y = -x perturbed in the last bits
    {
      double x = with_exp(900 + g() % 200);
      uint64_t yb = (B(x) ^ fpi::kSign) + (g() % 7) - 3;
      check(x, D(yb));
    }
    // 5) products near ties: mantissas with few significant bits
    {
      // significands with many trailing zeros: their products and sums are
      // often exactly half-way between two doubles
      uint64_t ka = 20 + g() % 33, kb = 20 + g() % 33;
      uint64_t ma = (g() & fpi::kMant) >> ka << ka, mb = (g() & fpi::kMant) >> kb << kb;
      double x = D(((g() & 1) << 63) | ((uint64_t)(1000 + g() % 40) << 52) | ma);
      double y = D(((g() & 1) << 63) | ((uint64_t)(1000 + g() % 40) << 52) | mb);
      check(x, y);
    }
    // 6) results near overflow and underflow
    {
      check(with_exp(2040 + g() % 7), with_exp(1020 + g() % 8));
      check(with_exp(1 + g() % 8), with_exp(1010 + g() % 20));
      check(with_exp(1 + g() % 3), with_exp(1 + g() % 3));
    }
    // 7) small integers and halves (exact ties in additions)
    {
      double x = (double)((int64_t)(g() % 2000001) - 1000000) * std::ldexp(1.0, (int)(g() % 80) - 40);
      double y = (double)((int64_t)(g() % 2000001) - 1000000) * std::ldexp(1.0, (int)(g() % 80) - 40);
      check(x, y);
      check(x, 0.0);
      check(-0.0, y);
    }
  }
  if (bad) {
    printf("FAIL %ld of %ld\n", bad, checked);
    return 1;
  }
  printf("ok %ld\n", checked);
  return 0;
}
