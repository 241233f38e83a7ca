/*
 * Seeded random sphere packings (appended API, no counterpart in the
 * reference, which takes its spheres from files such as
 * examples/rcp_spheres.dat): random sequential addition in a periodic
 * n^3 box, with the solid-node mask of the accepted spheres.
 *
 * Draws: splitmix64 (Steele, Lea and Flood 2014), four outputs per try --
 * centre x, y, z uniform in [0, n) and radius uniform in [rmin, rmax] --
 * each as (z >> 11) * 2^-53.  A try is accepted when its periodic
 * minimum-image centre distance to every accepted sphere is at least the
 * sum of the radii (any distance with overlap set).  Every accepted sphere
 * is stamped into the mask with its periodic images (the nodes with
 * rsq < r^2, the membership test of reference src/lbobjs.c:214-215), and
 * addition stops once the stamped fraction reaches phi.  The arithmetic of
 * every decision (distances, node tests) is written so that the result is
 * the same sphere list and mask as the numpy formulation in
 * sunlightlb_gb300/workloads.py, bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "sunlightlb.h"

static uint64_t splitmix_next(uint64_t *state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static double unit(uint64_t z) { return (double)(z >> 11) * (1.0 / 9007199254740992.0); }

/* nodes of one sphere image inside the lattice, OR-ed into solid; returns
 * the nodes newly set */
static long stamp_image(unsigned char *solid, int n, double rad, const double c[3]) {
  int lo[3], hi[3], a, i, j, k;
  long added = 0;
  double rr = rad * rad;
  for (a = 0; a < 3; a++) {
    lo[a] = (int)floor(c[a] - rad) - 1;
    hi[a] = (int)ceil(c[a] + rad) + 1;
    if (lo[a] < 0) lo[a] = 0;
    if (hi[a] > n - 1) hi[a] = n - 1;
    if (lo[a] > hi[a]) return 0;
  }
  for (i = lo[0]; i <= hi[0]; i++) {
    double di = (double)i - c[0];
    for (j = lo[1]; j <= hi[1]; j++) {
      double dj = (double)j - c[1];
      double sij = di * di + dj * dj;
      unsigned char *row = solid + ((size_t)i * n + j) * (size_t)n;
      for (k = lo[2]; k <= hi[2]; k++) {
        double dk = (double)k - c[2];
        if (sij + dk * dk < rr && !row[k]) { row[k] = 1; added++; }
      }
    }
  }
  return added;
}

/* a sphere and each periodic image whose node set can meet the lattice */
static long stamp(unsigned char *solid, int n, double rad, const double c[3]) {
  int di, dj, dk, a;
  long added = 0;
  for (di = -1; di <= 1; di++) for (dj = -1; dj <= 1; dj++) for (dk = -1; dk <= 1; dk++) {
    double ci[3];
    int ok = 1;
    ci[0] = c[0] + di * n; ci[1] = c[1] + dj * n; ci[2] = c[2] + dk * n;
    for (a = 0; a < 3; a++) ok &= (-rad < ci[a]) && (ci[a] < n - 1 + rad);
    if (ok) added += stamp_image(solid, n, rad, ci);
  }
  return added;
}

/* periodic minimum-image overlap of an accepted sphere (a, ra) and a
 * candidate (b, rb); nearbyint rounds half to even, as numpy's round */
static int overlaps(const double *a, double ra, const double *b, double rb, double n) {
  double d[3], dist;
  int q;
  for (q = 0; q < 3; q++) {
    d[q] = a[q] - b[q];
    d[q] -= n * nearbyint(d[q] / n);
  }
  dist = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
  return dist < ra + rb;
}

/* Random sequential addition in a periodic n^3 box up to solid fraction
 * phi.  spheres receives (r, x, y, z) per accepted sphere (room for
 * max_spheres), solid (may be NULL) the n^3 node mask, k fastest.  Returns
 * the number of spheres, -1 when a sphere would be accepted only after more
 * than max_tries tries (the packing stalled short of phi), -2 when
 * max_spheres is too small, -3 on bad arguments or no memory. */
int rsapacking(int n, double phi, double rmin, double rmax, unsigned long long seed, int overlap,
               long max_tries, double *spheres, int max_spheres, unsigned char *solid) {
  uint64_t state = seed;
  size_t nn;
  unsigned char *mask = solid;
  int ncell, cap = 8, m = 0, rc = -1;
  double cw, target;
  long nset = 0, tries = 0;
  int *grid = NULL, *fill = NULL;
  if (n < 1 || !(rmax >= rmin) || rmin <= 0.0 || spheres == NULL || max_spheres < 1) return -3;
  nn = (size_t)n * n * n;
  if (mask == NULL && (mask = (unsigned char *)malloc(nn)) == NULL) return -3;
  memset(mask, 0, nn);
  ncell = (int)floor(n / (2.0 * rmax));
  if (ncell < 1) ncell = 1;
  cw = (double)n / ncell;
  if (!overlap && ncell >= 3) {
    grid = (int *)malloc((size_t)ncell * ncell * ncell * cap * sizeof(int));
    fill = (int *)calloc((size_t)ncell * ncell * ncell, sizeof(int));
    if (grid == NULL || fill == NULL) { rc = -3; goto done; }
  }
  target = phi * (double)nn;
  while ((double)nset < target) {
    double c[3], r;
    int hit = 0, q;
    if (tries >= 4 * max_tries) { rc = -1; goto done; }  /* no acceptance in sight */
    tries++;
    c[0] = 0.0 + (double)n * unit(splitmix_next(&state));
    c[1] = 0.0 + (double)n * unit(splitmix_next(&state));
    c[2] = 0.0 + (double)n * unit(splitmix_next(&state));
    r = rmin + (rmax - rmin) * unit(splitmix_next(&state));
    if (!overlap) {
      if (grid == NULL) {
        for (q = 0; q < m && !hit; q++) hit = overlaps(spheres + 4 * q + 1, spheres[4 * q], c, r, n);
      } else {
        int ci[3], a, b, d;
        for (q = 0; q < 3; q++) {
          ci[q] = (int)floor(c[q] / cw);
          if (ci[q] > ncell - 1) ci[q] = ncell - 1;
        }
        for (a = -1; a <= 1 && !hit; a++) for (b = -1; b <= 1 && !hit; b++) for (d = -1; d <= 1 && !hit; d++) {
          int x = (ci[0] + a + ncell) % ncell, y = (ci[1] + b + ncell) % ncell, z = (ci[2] + d + ncell) % ncell;
          size_t cell = ((size_t)x * ncell + y) * ncell + z;
          int e;
          for (e = 0; e < fill[cell] && !hit; e++) {
            int s = grid[cell * cap + e];
            hit = overlaps(spheres + 4 * s + 1, spheres[4 * s], c, r, n);
          }
        }
      }
      if (hit) continue;
    }
    if (tries > max_tries) { rc = -1; goto done; }
    if (m == max_spheres) { rc = -2; goto done; }
    spheres[4 * m] = r; spheres[4 * m + 1] = c[0]; spheres[4 * m + 2] = c[1]; spheres[4 * m + 3] = c[2];
    if (grid != NULL) {
      int ci[3];
      size_t cell;
      for (q = 0; q < 3; q++) {
        ci[q] = (int)floor(c[q] / cw);
        if (ci[q] > ncell - 1) ci[q] = ncell - 1;
      }
      cell = ((size_t)ci[0] * ncell + ci[1]) * ncell + ci[2];
      if (fill[cell] == cap) {  /* widen every cell's slot list */
        size_t nc = (size_t)ncell * ncell * ncell, s;
        int *g2 = (int *)malloc(nc * 2 * cap * sizeof(int)), e;
        if (g2 == NULL) { rc = -3; goto done; }
        for (s = 0; s < nc; s++) for (e = 0; e < fill[s]; e++) g2[s * 2 * cap + e] = grid[s * cap + e];
        free(grid);
        grid = g2;
        cap *= 2;
      }
      grid[cell * cap + fill[cell]++] = m;
    }
    m++;
    nset += stamp(mask, n, r, c);
  }
  rc = m;
done:
  free(grid);
  free(fill);
  if (mask != solid) free(mask);
  return rc;
}
