// CPU restatement of the reference's configuration makers (test
// infrastructure: the checker of the device makers and the CPU baseline of
// their timing; never shipped).  Same C++ library generator and distribution
// as the reference (std::mt19937, std::uniform_real_distribution<double>), the
// same site loops, the same linear search for distinct deletion sites.
//   orc_make_fcc      ConfigurationMaker::Execute (confmaker.cc:9-44)
//   orc_make_extract  ExtractConfigurationMaker::Execute (confmaker.cc:174-252),
//                     one unit spanning the box
//   orc_make_droplet  DropletMaker::Execute / AddSub (burst.cc:10-61)
//   orc_make_collision  the two BallAdder balls of Collision::Run
//                     (collision.cc:8-63), each site kept by MDRect::IsInside
//                     of the one unit [0, L) (mdunit.cc:44-49, mdrect.h:35-38)
//   orc_initial_velocity  Variables::SetInitialVelocity (variables.cc:82-108)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace {

void put(double *q3, long &n, long cap, double x, double y, double z) {
  if (n < cap) {
    q3[3 * n + 0] = x;
    q3[3 * n + 1] = y;
    q3[3 * n + 2] = z;
  }
  n++;
}

}  // namespace

extern "C" {

long orc_make_fcc(const double L[3], double density, double *q3, long cap) {
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const double hs = s * 0.5;
  const int sx = static_cast<int>(L[0] / s), sy = static_cast<int>(L[1] / s), sz = static_cast<int>(L[2] / s);
  const double e = 0.0000001;
  long n = 0;
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const double x = static_cast<double>(ix) * s, y = static_cast<double>(iy) * s, z = static_cast<double>(iz) * s;
        put(q3, n, cap, x + e, y + e, z + e);
        put(q3, n, cap, x + e, y + hs + e, z + hs + e);
        put(q3, n, cap, x + hs + e, y + e, z + hs + e);
        put(q3, n, cap, x + hs + e, y + hs + e, z + e);
      }
  return n;
}

long orc_make_extract(const double L[3], double density, int unit_id, double *q3, long cap) {
  const double *w = L;
  double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const int sx = static_cast<unsigned long>(w[0] / s) + 1;
  const int sy = static_cast<unsigned long>(w[1] / s) + 1;
  const int sz = static_cast<unsigned long>(w[2] / s) + 1;
  const int n_full = sx * sy * sz * 4;
  const int n_exact = static_cast<int>(w[0] * w[1] * w[2] * density);
  const int n_delete = n_full - n_exact;
  std::vector<int> del;
  std::mt19937 mt(unit_id);
  std::uniform_real_distribution<double> ud(0.0, 1.0);
  while (static_cast<int>(del.size()) < n_delete) {
    const int v = static_cast<unsigned long>(n_full * ud(mt));
    if (std::find(del.begin(), del.end(), v) == del.end()) del.push_back(v);
  }
  std::sort(del.begin(), del.end());
  del.push_back(n_full);  // sentinel
  s = w[0] / sx;
  const double hs = s * 0.5;
  long n = 0;
  int site = 0;
  size_t pos = 0;
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const double x = 0.0 + static_cast<double>(ix) * s, y = 0.0 + static_cast<double>(iy) * s,
                     z = 0.0 + static_cast<double>(iz) * s;
        const double sub[4][3] = {{x, y, z}, {x, y + hs, z + hs}, {x + hs, y, z + hs}, {x + hs, y + hs, z}};
        for (int k = 0; k < 4; k++, site++) {
          if (del[pos] == site) {
            pos++;
            continue;
          }
          put(q3, n, cap, sub[k][0], sub[k][1], sub[k][2]);
        }
      }
  return n;
}

long orc_make_droplet(const double L[3], double density, double radius, double *q3, long cap) {
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const double hs = s * 0.5;
  const double c = L[0] * 0.5;
  const int sx = static_cast<int>(L[0] / s), sy = static_cast<int>(L[1] / s), sz = static_cast<int>(L[2] / s);
  const double e = 0.0000001;
  long n = 0;
  auto add = [&](double x, double y, double z) {
    const double dx = x - c, dy = y - c, dz = z - c;
    if (dx * dx + dy * dy + dz * dz < radius * radius) put(q3, n, cap, x, y, z);
  };
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const double x = static_cast<double>(ix) * s, y = static_cast<double>(iy) * s, z = static_cast<double>(iz) * s;
        add(x + e, y + e, z + e);
        add(x + e, y + hs + e, z + hs + e);
        add(x + hs + e, y + e, z + hs + e);
        add(x + hs + e, y + hs + e, z + e);
      }
  return n;
}

long orc_make_collision(const double L[3], double density, double radius, double speed, double *q3, double *p3,
                        long cap) {
  const double centre[2][3] = {{L[0] * 0.25, L[1] * 0.5, L[2] * 0.5}, {L[0] * 0.75, L[1] * 0.5, L[2] * 0.5}};
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const int is = static_cast<int>(2 * radius / s);
  const double hs = s * 0.5;
  long n = 0;
  for (int b = 0; b < 2; b++) {
    const double *c = centre[b];
    const double v = b == 0 ? speed : -speed;
    auto add = [&](double x, double y, double z) {
      const double dx = x - c[0], dy = y - c[1], dz = z - c[2];
      if (dx * dx + dy * dy + dz * dz > radius * radius) return;
      if (!(0.0 <= x && x < L[0] && 0.0 <= y && y < L[1] && 0.0 <= z && z < L[2])) return;
      if (p3 && n < cap) {
        p3[3 * n + 0] = v;
        p3[3 * n + 1] = 0.0;
        p3[3 * n + 2] = 0.0;
      }
      put(q3, n, cap, x, y, z);
    };
    for (int iz = 0; iz < is; iz++)
      for (int iy = 0; iy < is; iy++)
        for (int ix = 0; ix < is; ix++) {
          const double x = ix * s - radius + c[0], y = iy * s - radius + c[1], z = iz * s - radius + c[2];
          add(x, y, z);
          add(x + hs, y, z);
          add(x, y + hs, z);
          add(x, y, z + hs);
        }
  }
  return n;
}

void orc_initial_velocity(double *p3, long n, double v0, int seed) {
  std::mt19937 mt(seed);
  std::uniform_real_distribution<double> ud(0.0, 1.0);
  for (long i = 0; i < n; i++) {
    const double z = ud(mt) * 2.0 - 1.0;
    const double phi = ud(mt) * 2.0 * M_PI;
    p3[3 * i + 0] = v0 * sqrt(1 - z * z) * cos(phi);
    p3[3 * i + 1] = v0 * sqrt(1 - z * z) * sin(phi);
    p3[3 * i + 2] = v0 * z;
  }
  double av[3] = {0.0, 0.0, 0.0};
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) av[d] += p3[3 * i + d];
  for (int d = 0; d < 3; d++) av[d] /= static_cast<double>(n);
  for (long i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) p3[3 * i + d] -= av[d];
}

}  // extern "C"
