/* bedgen.c -- seeded random sequential placement of spheres (host code).
 *
 * The synthetic beds stand in for the reference's particle maker, whose
 * random placement is clock-seeded (Prtcl_Variables.f90:225-227,279-288) and
 * therefore not reproducible.  Sphere i (in index order) gets uniform random
 * centres in [lo + r_i, hi - r_i] until one overlaps no sphere placed before
 * it; that centre is kept.  The overlap test looks at the 27 cells around the
 * proposal in a grid of cells 2 * max radius wide (linked lists of the placed
 * spheres).  Deterministic for a seed on every host: the generator is
 * splitmix64 and the arithmetic is plain IEEE double without contraction.
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared (sdem_gb300/build.py). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

static uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double unit(uint64_t* s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Returns 0 on success; 1 on bad arguments; 2 when sphere *fail_at needed
 * more than max_tries proposals (the region is too full); 3 on allocation
 * failure.  pos receives 3 doubles per sphere; *proposals the total number of
 * proposals made. */
int bedgen_rsp(int n, const double* radius, const double* lo, const double* hi, unsigned long long seed,
               long long max_tries, double* pos, long long* proposals, int* fail_at) {
  if (n < 0 || (n > 0 && (!radius || !pos)) || !lo || !hi || !proposals || !fail_at) return 1;
  *proposals = 0;
  *fail_at = -1;
  if (n == 0) return 0;
  double rmax = 0.0;
  for (int i = 0; i < n; i++) {
    if (!(radius[i] > 0.0)) return 1;
    if (radius[i] > rmax) rmax = radius[i];
  }
  const double cell = 2.0 * rmax;
  long long dims[3];
  for (int a = 0; a < 3; a++) {
    if (!(hi[a] - lo[a] > 2.0 * rmax)) return 1;
    const double e = floor((hi[a] - lo[a]) / cell) + 1.0;
    if (!(e >= 1.0) || e > 1.0e8) return 1;
    dims[a] = (long long)e;
  }
  const long long ncell = dims[0] * dims[1] * dims[2];
  if (ncell > (1ll << 34)) return 1;
  int* head = (int*)malloc(sizeof(int) * (size_t)ncell);
  int* next = (int*)malloc(sizeof(int) * (size_t)n);
  if (!head || !next) {
    free(head);
    free(next);
    return 3;
  }
  for (long long c = 0; c < ncell; c++) head[c] = -1;
  uint64_t st = seed;
  long long total = 0;
  int rc = 0;
  for (int i = 0; i < n && rc == 0; i++) {
    const double r = radius[i];
    long long t = 0;
    for (;;) {
      if (t++ >= max_tries) {
        rc = 2;
        *fail_at = i;
        break;
      }
      double p[3];
      long long c3[3];
      for (int a = 0; a < 3; a++) {
        p[a] = (lo[a] + r) + unit(&st) * ((hi[a] - r) - (lo[a] + r));
        long long k = (long long)((p[a] - lo[a]) / cell);
        c3[a] = k < 0 ? 0 : (k >= dims[a] ? dims[a] - 1 : k);
      }
      int hit = 0;
      for (long long x = c3[0] - 1; x <= c3[0] + 1 && !hit; x++) {
        if (x < 0 || x >= dims[0]) continue;
        for (long long y = c3[1] - 1; y <= c3[1] + 1 && !hit; y++) {
          if (y < 0 || y >= dims[1]) continue;
          for (long long z = c3[2] - 1; z <= c3[2] + 1 && !hit; z++) {
            if (z < 0 || z >= dims[2]) continue;
            for (int j = head[(x * dims[1] + y) * dims[2] + z]; j >= 0; j = next[j]) {
              const double dx = pos[3 * j] - p[0], dy = pos[3 * j + 1] - p[1], dz = pos[3 * j + 2] - p[2];
              const double rs = radius[j] + r;
              if (dx * dx + dy * dy + dz * dz < rs * rs) {
                hit = 1;
                break;
              }
            }
          }
        }
      }
      if (hit) continue;
      pos[3 * i] = p[0];
      pos[3 * i + 1] = p[1];
      pos[3 * i + 2] = p[2];
      const long long key = (c3[0] * dims[1] + c3[1]) * dims[2] + c3[2];
      next[i] = head[key];
      head[key] = i;
      break;
    }
    total += t;
  }
  *proposals = total;
  free(head);
  free(next);
  return rc;
}
