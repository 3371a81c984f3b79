/* Checks, on the CPU, that the division used by the kernels for several
 * quotients with one divisor -- y = RN(1/b), q = RN(a*y), r = fma(-q, b, a),
 * q' = fma(r, y, q) (Markstein's correction, IBM J. Res. Dev. 34(1), 1990) --
 * returns exactly the IEEE-rounded a/b.  Returns the number of mismatches. */
#include <math.h>
#include <stdint.h>

static uint64_t s;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double frand(double lo_exp, double hi_exp) {
  double m = 1.0 + (double)(rnd() >> 11) * (1.0 / 9007199254740992.0);
  double e = lo_exp + (hi_exp - lo_exp) * (double)(rnd() >> 11) * (1.0 / 9007199254740992.0);
  double v = ldexp(m, (int)e);
  return (rnd() & 1) ? -v : v;
}

long long markstein_mismatches(long long n, uint64_t seed, double lo_exp, double hi_exp,
                               const double* divisors, int nd) {
  s = seed | 1;
  long long bad = 0;
  for (long long i = 0; i < n; i++) {
    double b = nd > 0 ? divisors[rnd() % (uint64_t)nd] : frand(lo_exp, hi_exp);
    double a = frand(lo_exp, hi_exp);
    double y = 1.0 / b;
    double q = a * y;
    double r = fma(-q, b, a);
    double q2 = fma(r, y, q);
    double ref = a / b;
    if (q2 != ref && !(q2 != q2 && ref != ref)) bad++;
  }
  return bad;
}
