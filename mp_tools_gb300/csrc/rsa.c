/* Random sequential addition of hard spheres in a periodic cubic box (synthetic amorphous
 * alloy frames).  Cell list of side >= dmin (so only the 27 neighbouring cells can conflict),
 * up to 8 atoms per cell, own cell checked first; candidates come from a splitmix64 stream
 * seeded by the caller, so the output is identical on every machine.  Returns the number of
 * atoms placed (n unless max_attempts ran out). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define CAP 8

static uint64_t sm64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double unit(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

int64_t mpsq_rsa_hard_spheres(int64_t n, double box, double dmin, uint64_t seed,
                              int64_t max_attempts, double* pos /* n*3, in [0, box) */) {
  int64_t nc = (int64_t)floor(box / dmin);
  if (nc < 3) nc = 3;
  const double side = box / (double)nc;
  const int64_t ncell = nc * nc * nc;
  uint8_t* cnt = (uint8_t*)calloc((size_t)ncell, 1);
  int32_t* members = (int32_t*)malloc(sizeof(int32_t) * CAP * (size_t)ncell);
  if (!cnt || !members) {
    free(cnt);
    free(members);
    return -1;
  }
  const double d2 = dmin * dmin;
  static const int order[27][3] = {
      {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},  {0, 0, 1},   {0, 0, -1},
      {1, 1, 0},   {1, -1, 0},  {-1, 1, 0},  {-1, -1, 0}, {1, 0, 1},   {1, 0, -1},  {-1, 0, 1},
      {-1, 0, -1}, {0, 1, 1},   {0, 1, -1},  {0, -1, 1},  {0, -1, -1}, {1, 1, 1},   {1, 1, -1},
      {1, -1, 1},  {1, -1, -1}, {-1, 1, 1},  {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
  uint64_t st = seed;
  int64_t count = 0;
  for (int64_t att = 0; att < max_attempts && count < n; ++att) {
    const double x = unit(&st) * box, y = unit(&st) * box, z = unit(&st) * box;
    int64_t cx = (int64_t)(x / side), cy = (int64_t)(y / side), cz = (int64_t)(z / side);
    if (cx >= nc) cx = nc - 1;
    if (cy >= nc) cy = nc - 1;
    if (cz >= nc) cz = nc - 1;
    int bad = 0;
    for (int o = 0; o < 27 && !bad; ++o) {
      int64_t xx = cx + order[o][0], yy = cy + order[o][1], zz = cz + order[o][2];
      xx = xx < 0 ? xx + nc : (xx >= nc ? xx - nc : xx);
      yy = yy < 0 ? yy + nc : (yy >= nc ? yy - nc : yy);
      zz = zz < 0 ? zz + nc : (zz >= nc ? zz - nc : zz);
      const int64_t c = (zz * nc + yy) * nc + xx;
      const int k = cnt[c];
      const int32_t* m = members + (size_t)CAP * c;
      for (int i = 0; i < k; ++i) {
        const int32_t j = m[i];
        double ux = x - pos[3 * j], uy = y - pos[3 * j + 1], uz = z - pos[3 * j + 2];
        if (ux > 0.5 * box) ux -= box; else if (ux < -0.5 * box) ux += box;
        if (uy > 0.5 * box) uy -= box; else if (uy < -0.5 * box) uy += box;
        if (uz > 0.5 * box) uz -= box; else if (uz < -0.5 * box) uz += box;
        if (ux * ux + uy * uy + uz * uz < d2) {
          bad = 1;
          break;
        }
      }
    }
    if (bad) continue;
    const int64_t c = (cz * nc + cy) * nc + cx;
    if (cnt[c] >= CAP) continue; /* cannot happen for side < 2 dmin; keeps the store bounded */
    members[(size_t)CAP * c + cnt[c]] = (int32_t)count;
    cnt[c]++;
    pos[3 * count] = x;
    pos[3 * count + 1] = y;
    pos[3 * count + 2] = z;
    ++count;
  }
  free(cnt);
  free(members);
  return count;
}
