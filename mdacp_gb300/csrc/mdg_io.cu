// The reference's output and restart formats, written from [n][4] state
// arrays (host code; the handle forms read the state back from the device
// first).  The bytes are those of the reference's own writers for the same
// particles in the same order:
//   dump          MDManager::SaveAsDumpFile (mdmanager.cc:475-505): per particle
//                 qx qy qz px py pz as native doubles;
//   CDView        MDUnit::SaveAsCdview (mdunit.cc:52-67): "0 type qx qy qz px py pz"
//                 lines through an ostream with default formatting;
//   configuration Variables::SaveConfiguration (variables.cc:45-56): "qx qy qz
//                 px py pz" lines (the reference also writes its ghost copies,
//                 which the engine does not keep: real particles only);
//   stream        Variables::SaveToStream (variables.cc:111-118): per particle,
//                 for d = 0..3, q[d] then p[d]; Variables::LoadFromStream
//                 (variables.cc:121-131) reads an int particle count, the
//                 simulation time and zeta before that body, a header the
//                 writer does not produce.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <vector>

#include "../../include/mdg.h"

namespace {

std::ios::openmode mode(bool append, bool binary) {
  std::ios::openmode m = std::ios::out | (append ? std::ios::app : std::ios::trunc);
  return binary ? (m | std::ios::binary) : m;
}

int state_of(mdg_handle *h, std::vector<double> &q4, std::vector<double> &p4) {
  mdg_stats st;
  int rc = mdg_get_stats(h, &st);
  if (rc) return rc;
  q4.assign((size_t)st.particles * 4, 0.0);
  p4.assign((size_t)st.particles * 4, 0.0);
  if (st.particles == 0) return MDG_OK;
  return mdg_get_state(h, q4.data(), p4.data());
}

}  // namespace

extern "C" {

int mdg_write_dump(const char *path, const double *q4, const double *p4, int32_t n, int32_t append) {
  if (!path || n < 0 || (n > 0 && (!q4 || !p4))) return MDG_ERR_INVALID;
  std::ofstream ofs(path, mode(append != 0, true));
  if (!ofs) return MDG_ERR_INVALID;
  std::vector<double> buf((size_t)n * 6);
  for (int32_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      buf[6 * (size_t)i + d] = q4[4 * i + d];
      buf[6 * (size_t)i + 3 + d] = p4[4 * i + d];
    }
  ofs.write(reinterpret_cast<const char *>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
  return ofs ? MDG_OK : MDG_ERR_INVALID;
}

int mdg_write_cdview(const char *path, const double *q4, const double *p4, const int32_t *type, int32_t n,
                     int32_t append) {
  if (!path || n < 0 || (n > 0 && (!q4 || !p4))) return MDG_ERR_INVALID;
  std::ofstream ofs(path, mode(append != 0, false));
  if (!ofs) return MDG_ERR_INVALID;
  for (int32_t i = 0; i < n; i++) {
    ofs << "0 " << (type ? type[i] : 0) << " " << q4[4 * i + 0] << " " << q4[4 * i + 1] << " " << q4[4 * i + 2]
        << " " << p4[4 * i + 0] << " " << p4[4 * i + 1] << " " << p4[4 * i + 2] << "\n";
  }
  return ofs ? MDG_OK : MDG_ERR_INVALID;
}

int mdg_write_configuration(const char *path, const double *q4, const double *p4, int32_t n) {
  if (!path || n < 0 || (n > 0 && (!q4 || !p4))) return MDG_ERR_INVALID;
  std::ofstream ofs(path, mode(false, false));
  if (!ofs) return MDG_ERR_INVALID;
  for (int32_t i = 0; i < n; i++) {
    ofs << q4[4 * i + 0] << " " << q4[4 * i + 1] << " " << q4[4 * i + 2] << " " << p4[4 * i + 0] << " "
        << p4[4 * i + 1] << " " << p4[4 * i + 2] << "\n";
  }
  return ofs ? MDG_OK : MDG_ERR_INVALID;
}

int mdg_write_stream(const char *path, const double *q4, const double *p4, int32_t n, int32_t append) {
  if (!path || n < 0 || (n > 0 && (!q4 || !p4))) return MDG_ERR_INVALID;
  std::ofstream ofs(path, mode(append != 0, true));
  if (!ofs) return MDG_ERR_INVALID;
  std::vector<double> buf((size_t)n * 8);
  for (int32_t i = 0; i < n; i++)
    for (int d = 0; d < 4; d++) {
      buf[8 * (size_t)i + 2 * d] = q4[4 * i + d];
      buf[8 * (size_t)i + 2 * d + 1] = p4[4 * i + d];
    }
  ofs.write(reinterpret_cast<const char *>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
  return ofs ? MDG_OK : MDG_ERR_INVALID;
}

int mdg_read_stream(const char *path, double *q4, double *p4, int32_t capacity, int32_t *n, double *time,
                    double *zeta) {
  if (!path || !n || capacity < 0) return MDG_ERR_INVALID;
  std::ifstream ifs(path, std::ios::in | std::ios::binary);
  if (!ifs) return MDG_ERR_INVALID;
  int32_t count = 0;
  double t = 0.0, z = 0.0;
  ifs.read(reinterpret_cast<char *>(&count), sizeof count);
  ifs.read(reinterpret_cast<char *>(&t), sizeof t);
  ifs.read(reinterpret_cast<char *>(&z), sizeof z);
  if (!ifs || count < 0) return MDG_ERR_INVALID;
  *n = count;
  if (time) *time = t;
  if (zeta) *zeta = z;
  if (count > capacity) return MDG_ERR_CAPACITY;
  if (count > 0 && (!q4 || !p4)) return MDG_ERR_INVALID;
  for (int32_t i = 0; i < count; i++)
    for (int d = 0; d < 4; d++) {
      ifs.read(reinterpret_cast<char *>(&q4[4 * i + d]), sizeof(double));
      ifs.read(reinterpret_cast<char *>(&p4[4 * i + d]), sizeof(double));
    }
  return ifs ? MDG_OK : MDG_ERR_INVALID;
}

int mdg_save_dump(mdg_handle *h, const char *path) {
  std::vector<double> q4, p4;
  int rc = state_of(h, q4, p4);
  if (rc) return rc;
  return mdg_write_dump(path, q4.data(), p4.data(), (int32_t)(q4.size() / 4), 0);
}

int mdg_save_cdview(mdg_handle *h, const char *path) {
  std::vector<double> q4, p4;
  int rc = state_of(h, q4, p4);
  if (rc) return rc;
  return mdg_write_cdview(path, q4.data(), p4.data(), nullptr, (int32_t)(q4.size() / 4), 0);
}

}  // extern "C"
