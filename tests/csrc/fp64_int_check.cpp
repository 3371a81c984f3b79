// CPU check of sdem_gb300/csrc/fp64_int.cuh: the integer-pipe binary64
// sqrt, division, comparisons, -x/2, grid floor and floor of a quotient
// against the host's IEEE arithmetic.
// Usage: fp64_int_check <seed> <pairs per family>; prints "ok <n>" or the
// first mismatches and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <random>

// The device seeds (rsqrt.approx / rcp.approx) carry a few ulp of error that
// the host's 1/sqrtf and 1/x do not: with NOISE set, every host seed is moved
// by a pseudo-random amount of up to +-64 ulp (relative 2^-17), far beyond
// the device's error, so the refinement and the final rounding test are
// exercised with worse seeds than the GPU ever produces.
#include <cstdint>
#include <cstring>
static uint64_t g_noise = 0x9E3779B97F4A7C15ull;
static int g_noise_on = 0;
static float seed_noise(float r) {
  if (!g_noise_on) return r;
  g_noise ^= g_noise << 13; g_noise ^= g_noise >> 7; g_noise ^= g_noise << 17;
  uint32_t u;
  memcpy(&u, &r, 4);
  u += (uint32_t)((int32_t)(g_noise % 129) - 64);
  memcpy(&r, &u, 4);
  return r;
}
#define FPI_HOST_SEED_HOOK seed_noise
#include "../../sdem_gb300/csrc/fp64_int.cuh"

static uint64_t B(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static double D(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static bool same(double a, double b) {
  if (std::isnan(a) && std::isnan(b)) return true;
  return B(a) == B(b);
}

static long bad = 0, checked = 0;
// floor_div: the floor of the IEEE quotient for a few grid sizes, and the
// in-unit offset estimate within 2^-26 of q - floor (quotients below 2^26)
static void check_floor_div(double x, double y) {
  const fpi::Divisor v = fpi::divisor(y);
  const int ns[3] = {1, 37, 1000000};
  const double q = x / y, f = std::floor(q);
  for (int j = 0; j < 3; j++) {
    int32_t off = 0;
    const int k = fpi::floor_div(x, v, ns[j], off);
    const int want = (f >= 0.0 && f < (double)ns[j]) ? (int)f : -1;
    checked++;
    if (k != want) {
      if (bad < 20) printf("MISMATCH floor_div x=%a y=%a n=%d got=%d want=%d\n", x, y, ns[j], k, want);
      bad++;
    } else if (k >= 0 && std::fabs(q) < 0x1p26 && std::fabs(off * 0x1p-31 - (q - (double)k)) > 0x1p-26) {
      if (bad < 20) printf("MISMATCH floor_div offset x=%a y=%a off=%d q-k=%a\n", x, y, off, q - (double)k);
      bad++;
    }
  }
}

static void check(double x, double y) {
  check_floor_div(x, y);
  const double r[4] = {fpi::mul_neg_half(x), fpi::sqrt_rn(x), fpi::div_rn(x, y), fpi::div_rn(y, x)};
  const double e[4] = {x * -0.5, std::sqrt(x), x / y, y / x};
  const char* nm[4] = {"mul_neg_half", "sqrt", "div", "div(y,x)"};
  {
    // floor_in_range against floor() and a range test, for a few grid sizes
    const int ns[3] = {1, 37, 1000000};
    for (int j = 0; j < 3; j++) {
      for (double q : {x, y, x * 1e-300, y * 1e300, (double)(int64_t)(x) }) {
        const double f = std::floor(q);
        const int want = (f >= 0.0 && f < (double)ns[j]) ? (int)f : -1;
        checked++;
        if (fpi::floor_in_range(q, ns[j]) != want) {
          if (bad < 20) printf("MISMATCH floor_in_range q=%a n=%d got=%d want=%d\n", q, ns[j], fpi::floor_in_range(q, ns[j]), want);
          bad++;
        }
      }
    }
  }
  {
    const bool cg[4] = {fpi::gt(x, y), fpi::lt(x, y), fpi::ge(x, y), fpi::le(x, y)};
    const bool cw[4] = {x > y, x < y, x >= y, x <= y};
    for (int j = 0; j < 4; j++) {
      checked++;
      if (cg[j] != cw[j]) {
        if (bad < 20) printf("MISMATCH compare %d x=%a y=%a got=%d want=%d\n", j, x, y, (int)cg[j], (int)cw[j]);
        bad++;
      }
    }
    const fpi::Divisor v = fpi::divisor(y);
    checked++;
    if (!same(fpi::div_by(x, v), x / y)) {
      if (bad < 20) printf("MISMATCH div_by x=%a y=%a\n", x, y);
      bad++;
    }
  }
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
  if (argc > 3) g_noise_on = atoi(argv[3]);
  for (long i = 0; i < n; i++) {
    // 0) perfect squares and their neighbours (exact and near-exact roots),
    //    exact quotients and their neighbours
    {
      const uint64_t k = (g() >> 38) | 1u;            // up to 26 bits
      const double sq = (double)k * (double)k;          // exact
      uint64_t sb = B(sq) + (g() % 5) - 2;
      check(D(sb), (double)k);
      const uint64_t m1 = (g() >> 40) | 1u, m2 = (g() >> 40) | 1u;
      check((double)m1 * (double)m2, (double)m2);     // exact quotient m1
      check(D(B((double)m1 * (double)m2) + 1), (double)m2);
    }
    // grid coordinates: q = (x - x0) / cell around integers and cell edges
    {
      const double cell = 1.2e-3 * (1.0 + (g() % 1000) * 1e-4);
      const double xx = ((double)(int64_t)(g() % 4000) - 100.0) * cell + ((double)(g() % 2001) - 1000.0) * 1e-19;
      check(xx, cell);
      check(-0.0, cell);
      // the neighbours of an exact multiple of the cell: quotients within an
      // ulp of an integer, on both sides
      const double mk = (double)(int64_t)(g() % 4000) * cell;
      check_floor_div(D(B(mk) + (g() % 9) - 4), cell);
      check_floor_div(std::fabs(xx), cell);
    }
    // equal values, signed zeros and neighbours for the comparisons
    {
      const double x = D(u64());
      check(x, x);
      check(x, D(B(x) + 1));
      check(0.0, -0.0);
      check(-0.0, D(g() & 1 ? 0x8000000000000001ull : 1ull));
    }
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
