/*
 * Random-walk placement for the synthetic globule workload (see globule.py
 * for the rules and their interpretation).  Workload generation only; not
 * part of the GB hot path.  Uses a splitmix64 generator and only + - * / and
 * sqrt, so with -ffp-contract=off the walk is identical on x86 and Arm.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t sm_next(uint64_t* s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static double sm_unit(uint64_t* s) { return (double)(sm_next(s) >> 11) * (1.0 / 9007199254740992.0); }

/* uniform direction by rejection from the cube */
static void rand_dir(uint64_t* s, double d[3]) {
  for (;;) {
    double x = 2.0 * sm_unit(s) - 1.0, y = 2.0 * sm_unit(s) - 1.0, z = 2.0 * sm_unit(s) - 1.0;
    double r2 = x * x + y * y + z * z;
    if (r2 > 1e-6 && r2 <= 1.0) {
      double r = sqrt(r2);
      d[0] = x / r;
      d[1] = y / r;
      d[2] = z / r;
      return;
    }
  }
}

typedef struct {
  double cell, origin;
  int dim;
  int* head; /* dim^3 */
  int* next; /* n */
} hash3;

static int cell_of(const hash3* h, double v) {
  int c = (int)floor((v - h->origin) / h->cell);
  if (c < 0) c = 0;
  if (c >= h->dim) c = h->dim - 1;
  return c;
}

/* Returns 0 on success.  out_pos [3n] in Angstrom; out_meta: sphere radius,
 * final dmin. */
int gbx_globule_walk(int n, uint64_t seed, double density, double step, double dmin0, double dmin_floor,
                     int stall, int tries, double* out_pos, double* out_meta) {
  if (n < 1) return -1;
  const double pi = 3.14159265358979323846;
  double R = cbrt(3.0 * n / (4.0 * pi * density));
  double dmin = dmin0;
  uint64_t s = seed * 0x632be59bd9b4e019ULL + 0x1234567ULL;
  hash3 h;
  h.cell = step + dmin0;
  /* room for a sphere that may grow: 4x the initial radius */
  h.origin = -4.0 * R - h.cell;
  h.dim = (int)ceil((8.0 * R + 2.0 * h.cell) / h.cell) + 1;
  size_t ncell = (size_t)h.dim * h.dim * h.dim;
  h.head = (int*)malloc(sizeof(int) * ncell);
  h.next = (int*)malloc(sizeof(int) * (size_t)n);
  if (!h.head || !h.next) return -2;
  for (size_t c = 0; c < ncell; ++c) h.head[c] = -1;
  memset(out_pos, 0, sizeof(double) * 3 * (size_t)n);
#define HCELL(x, y, z) (((size_t)(x) * h.dim + (y)) * h.dim + (z))
  {
    size_t c = HCELL(cell_of(&h, 0), cell_of(&h, 0), cell_of(&h, 0));
    h.next[0] = h.head[c];
    h.head[c] = 0;
  }
  int placed = 1, cur = 0, fails = 0;
  while (placed < n) {
    const double* c = out_pos + 3 * cur;
    int cx = cell_of(&h, c[0]), cy = cell_of(&h, c[1]), cz = cell_of(&h, c[2]);
    int ok_any = 0;
    double cand[3];
    for (int t = 0; t < tries && !ok_any; ++t) {
      double d[3];
      rand_dir(&s, d);
      for (int k = 0; k < 3; ++k) cand[k] = c[k] + step * d[k];
      if (cand[0] * cand[0] + cand[1] * cand[1] + cand[2] * cand[2] > R * R) continue;
      int ok = 1;
      for (int dx = -1; dx <= 1 && ok; ++dx)
        for (int dy = -1; dy <= 1 && ok; ++dy)
          for (int dz = -1; dz <= 1 && ok; ++dz) {
            int X = cx + dx, Y = cy + dy, Z = cz + dz;
            if (X < 0 || Y < 0 || Z < 0 || X >= h.dim || Y >= h.dim || Z >= h.dim) continue;
            for (int j = h.head[HCELL(X, Y, Z)]; j >= 0; j = h.next[j]) {
              if (j == cur) continue;
              double ex = cand[0] - out_pos[3 * j], ey = cand[1] - out_pos[3 * j + 1], ez = cand[2] - out_pos[3 * j + 2];
              if (ex * ex + ey * ey + ez * ez < dmin * dmin) {
                ok = 0;
                break;
              }
            }
          }
      if (ok) ok_any = 1;
    }
    if (ok_any) {
      double* p = out_pos + 3 * placed;
      p[0] = cand[0];
      p[1] = cand[1];
      p[2] = cand[2];
      size_t cc = HCELL(cell_of(&h, p[0]), cell_of(&h, p[1]), cell_of(&h, p[2]));
      h.next[placed] = h.head[cc];
      h.head[cc] = placed;
      cur = placed;
      placed++;
      fails = 0;
      continue;
    }
    fails++;
    cur = (int)(sm_next(&s) % (uint64_t)placed);
    if (fails >= stall) {
      fails = 0;
      if (dmin - 0.1 >= dmin_floor - 1e-9)
        dmin = floor((dmin - 0.1) * 10.0 + 0.5) / 10.0;
      else if (R * 1.01 < 3.9 * cbrt(3.0 * n / (4.0 * pi * density)))
        R *= 1.01;
      else
        return -3;
    }
  }
#undef HCELL
  free(h.head);
  free(h.next);
  out_meta[0] = R;
  out_meta[1] = dmin;
  return 0;
}
