#include "mdg_host.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mdghost {

bool Parameter::LoadFromFile(const std::string &path) {
  std::ifstream is(path);
  if (is.fail()) {
    valid_ = false;
    return false;
  }
  std::stringstream ss;
  ss << is.rdbuf();
  ReadFromString(ss.str());
  return true;
}

void Parameter::ReadFromString(const std::string &text) {
  std::istringstream is(text);
  std::string line;
  while (std::getline(is, line)) {
    const size_t k = line.find('=');
    if (k != std::string::npos) params_.insert(std::make_pair(line.substr(0, k), line.substr(k + 1)));
  }
}

std::string Parameter::GetStringDef(const std::string &key, const std::string &def) const {
  auto it = params_.find(key);
  return it == params_.end() ? def : it->second;
}

double Parameter::GetDoubleDef(const std::string &key, double def) const {
  auto it = params_.find(key);
  return it == params_.end() ? def : atof(it->second.c_str());
}

int Parameter::GetIntegerDef(const std::string &key, int def) const {
  auto it = params_.find(key);
  return it == params_.end() ? def : atoi(it->second.c_str());
}

bool Parameter::GetBooleanDef(const std::string &key, bool def) const {
  auto it = params_.find(key);
  if (it == params_.end()) return def;
  return it->second == "yes" || it->second == "Yes";
}

SimulationInfo::SimulationInfo(const Parameter &p) {
  TimeStep = p.GetDoubleDef("TimeStep", 0.001);
  AimedTemperature = p.GetDoubleDef("AimedTemperature", 1.0);
  ControlTemperature = p.GetBooleanDef("ControlTemperature", false);
  HeatbathTau = p.GetDoubleDef("HeatbathTau", 0.1);
  HeatbathGamma = p.GetDoubleDef("HeatbathGamma", 0.1);
  const std::string hb = p.GetStringDef("HeatbathType", "NoseHoover");
  if (hb == "NoseHoover") HeatbathType = 0;
  else if (hb == "Langevin") HeatbathType = 1;
  else throw std::runtime_error("Unknown Heatbath type " + hb);
  if (p.Contains("SystemSize")) {
    L[0] = L[1] = L[2] = p.GetDoubleDef("SystemSize", 0.0);
  } else if (p.Contains("UnitLength")) {
    L[0] = L[1] = L[2] = p.GetDoubleDef("UnitLength", 0.0);  // one unit spans the box
  }
  if (p.Contains("SystemSizeX")) L[0] = p.GetDoubleDef("SystemSizeX", 0.0);
  if (p.Contains("SystemSizeY")) L[1] = p.GetDoubleDef("SystemSizeY", 0.0);
  if (p.Contains("SystemSizeZ")) L[2] = p.GetDoubleDef("SystemSizeZ", 0.0);
  CutoffLength = p.GetDoubleDef("CutoffLength", 3.0);
  BufferLength = p.GetDoubleDef("BufferLength", 0.3);
  const std::string prec = p.GetStringDef("Precision", "fp64");
  if (prec == "fp64") Precision = MDG_FP64;
  else if (prec == "mixed") Precision = MDG_MIXED;
  else if (prec == "mixed_plain") Precision = MDG_MIXED_PLAIN;
  else throw std::runtime_error("Precision must be fp64, mixed or mixed_plain");
  LangevinHalfDriftCompat = p.GetBooleanDef("LangevinHalfDriftCompat", true);
  // keys of this engine: the GPU only (Device=cpu is the reference's own
  // path), and the rebuild rule (the reference's PairList policy or half the
  // margin)
  const std::string dev = p.GetStringDef("Device", "gpu");
  if (dev == "gpu") Device = 0;
  else if (dev.rfind("gpu:", 0) == 0 && dev.size() > 4 && dev.find_first_not_of("0123456789", 4) == std::string::npos)
    Device = atoi(dev.c_str() + 4);
  else throw std::runtime_error("Device=" + dev + ": this engine runs on the GPU (Device=gpu or gpu:<ordinal>)");
  const std::string policy = p.GetStringDef("RebuildPolicy", "halfmargin");
  if (policy == "halfmargin") RebuildPolicy = MDG_REBUILD_HALFMARGIN;
  else if (policy == "reference") RebuildPolicy = MDG_REBUILD_REFERENCE;
  else
    throw std::runtime_error("RebuildPolicy=" + policy +
                             ": halfmargin (rebuild once a particle moved half the margin) or reference (the "
                             "buffer budget and displacement check of PairList)");
  CheckListLength = p.GetIntegerDef("CheckListLength", 500);
}

MDManager::MDManager(const Parameter &param, int capacity) : sinfo_(param) {
  mdg_params p;
  mdg_params_default(&p);
  p.capacity = capacity;
  for (int k = 0; k < 3; k++) p.box[k] = sinfo_.L[k];
  p.cutoff = sinfo_.CutoffLength;
  p.margin = sinfo_.BufferLength;
  p.dt = sinfo_.TimeStep;
  p.precision = sinfo_.Precision;
  p.thermostat = !sinfo_.ControlTemperature ? MDG_NVE : (sinfo_.HeatbathType == 1 ? MDG_LANGEVIN : MDG_NOSEHOOVER);
  p.langevin_half_drift_compat = sinfo_.LangevinHalfDriftCompat ? 1 : 0;
  p.temperature = sinfo_.AimedTemperature;
  p.gamma = sinfo_.HeatbathGamma;
  p.tau = sinfo_.HeatbathTau;
  p.seed = (uint64_t)param.GetIntegerDef("Seed", 1);
  p.device = sinfo_.Device;
  p.rebuild_policy = sinfo_.RebuildPolicy;
  p.check_list_length = sinfo_.CheckListLength;
  const int rc = mdg_create(&p, &h_);
  if (rc != MDG_OK)
    throw std::runtime_error("mdg_create failed (" + std::to_string(rc) + "): " + mdg_last_error(nullptr));
}

MDManager::~MDManager() { mdg_destroy(h_); }

void MDManager::Check(int rc, const char *what) {
  if (rc != MDG_OK) throw std::runtime_error(std::string(what) + ": " + mdg_last_error(h_));
}

void MDManager::AddParticle(const double x[3], const double v[3]) {
  // MDRect::IsInside (mdrect.h:36-39) for the single unit [0, L)
  for (int k = 0; k < 3; k++)
    if (!(0.0 <= x[k] && x[k] < sinfo_.L[k])) return;
  q_.insert(q_.end(), {x[0], x[1], x[2], 0.0});
  p_.insert(p_.end(), {v[0], v[1], v[2], 0.0});
  uploaded_ = false;
}

void MDManager::SetInitialVelocity(double V0, int seed) {
  std::mt19937 mt(seed);
  std::uniform_real_distribution<double> ud(0.0, 1.0);
  const int n = GetParticleNumber();
  for (int i = 0; i < n; i++) {
    const double z = ud(mt) * 2.0 - 1.0;
    const double phi = ud(mt) * 2.0 * M_PI;
    p_[4 * i + 0] = V0 * sqrt(1 - z * z) * cos(phi);
    p_[4 * i + 1] = V0 * sqrt(1 - z * z) * sin(phi);
    p_[4 * i + 2] = V0 * z;
  }
  for (int d = 0; d < 3; d++) {
    double av = 0;
    for (int i = 0; i < n; i++) av += p_[4 * i + d];
    av /= (double)n;
    for (int i = 0; i < n; i++) p_[4 * i + d] -= av;
  }
  uploaded_ = false;
}

void MDManager::Sync() {
  if (!uploaded_) {
    Check(mdg_set_state(h_, q_.data(), p_.data(), GetParticleNumber()), "mdg_set_state");
    uploaded_ = true;
  }
}

void MDManager::MakePairList() {
  Sync();
  Check(mdg_make_pairlist(h_), "mdg_make_pairlist");
}

void MDManager::Calculate() { Calculate(1); }

void MDManager::Calculate(int nsteps) {
  Sync();
  Check(mdg_calculate(h_, nsteps), "mdg_calculate");
  s_time_ += sinfo_.TimeStep * nsteps;
}

void MDManager::Observe(double out[3]) {
  Sync();
  Check(mdg_observe(h_, out), "mdg_observe");
}

// MDManager::KineticEnergy / PotentialEnergy / Temperature / Pressure /
// TotalEnergy (mdmanager.cc:389-429).
double MDManager::KineticEnergy() {
  double o[3];
  Observe(o);
  return o[0] / (double)GetTotalParticleNumber();
}

double MDManager::PotentialEnergy() {
  double o[3];
  Observe(o);
  return o[1] / (double)GetTotalParticleNumber();
}

double MDManager::Temperature() { return KineticEnergy() / 1.5; }

double MDManager::Pressure() {
  double o[3];
  Observe(o);
  const double pn = (double)GetTotalParticleNumber();
  const double phi = o[2] / pn;
  const double T = o[0] / pn / 1.5;
  const double V = sinfo_.L[0] * sinfo_.L[1] * sinfo_.L[2];
  return (T - phi) * pn / V;
}

double MDManager::TotalEnergy() {
  double o[3];
  Observe(o);
  const double pn = (double)GetTotalParticleNumber();
  return o[0] / pn + o[1] / pn;
}

void MDManager::SetSeed(int seed) { Check(mdg_set_seed(h_, (uint64_t)seed), "mdg_set_seed"); }

void MDManager::SetControlTemperature(bool b) {
  sinfo_.ControlTemperature = b;
  const int t = !b ? MDG_NVE : (sinfo_.HeatbathType == 1 ? MDG_LANGEVIN : MDG_NOSEHOOVER);
  Check(mdg_set_thermostat(h_, t, sinfo_.AimedTemperature), "mdg_set_thermostat");
}

void MDManager::SetAimedTemperature(double t) {
  sinfo_.AimedTemperature = t;
  SetControlTemperature(sinfo_.ControlTemperature);
}

void MDManager::GetState(std::vector<double> &q4, std::vector<double> &p4) {
  Sync();
  q4.resize(q_.size());
  p4.resize(p_.size());
  Check(mdg_get_state(h_, q4.data(), p4.data()), "mdg_get_state");
}

void MDManager::SaveStateRaw(const std::string &path) {
  std::vector<double> q4, p4;
  GetState(q4, p4);
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const int64_t n = GetParticleNumber();
  fwrite(&n, sizeof n, 1, f);
  for (int64_t i = 0; i < n; i++) {
    const double rec[6] = {q4[4 * i], q4[4 * i + 1], q4[4 * i + 2], p4[4 * i], p4[4 * i + 1], p4[4 * i + 2]};
    fwrite(rec, sizeof(double), 6, f);
  }
  fclose(f);
}

void MDManager::MakeStateOnDevice(int maker, double density, double radius, double v0) {
  Check(mdg_make_state(h_, maker, density, radius, v0), "mdg_make_state");
  mdg_stats st;
  Check(mdg_get_stats(h_, &st), "mdg_get_stats");
  q_.assign((size_t)st.particles * 4, 0.0);  // the state lives on the device
  p_.assign((size_t)st.particles * 4, 0.0);
  uploaded_ = true;
}

void MDManager::SaveAsDumpFile(const char *filename) {
  Sync();
  Check(mdg_save_dump(h_, filename), "mdg_save_dump");
}

void MDManager::SaveAsDumpFileSequential() {
  char filename[256];
  snprintf(filename, sizeof filename, "conf%04d.dump", dump_index_++);
  SaveAsDumpFile(filename);
}

void MDManager::SaveAsCdview(const char *filename) {
  Sync();
  Check(mdg_save_cdview(h_, filename), "mdg_save_cdview");
}

void MDManager::SaveAsCdviewSequential() {
  char filename[256];
  snprintf(filename, sizeof filename, "conf%04d.cd", cdview_index_++);
  SaveAsCdview(filename);
}

void MakeFCC(const Parameter &param, MDManager &m) {
  const double *L = m.GetSystemSize();
  const double density = param.GetDoubleDef("Density", 0.5);
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const double hs = s * 0.5;
  const int sx = (int)(L[0] / s), sy = (int)(L[1] / s), sz = (int)(L[2] / s);
  const double e = 0.0000001;
  const double zero[3] = {0.0, 0.0, 0.0};
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const double x0[3] = {ix * s + e, iy * s + e, iz * s + e};
        const double x1[3] = {ix * s + e, iy * s + hs + e, iz * s + hs + e};
        const double x2[3] = {ix * s + hs + e, iy * s + e, iz * s + hs + e};
        const double x3[3] = {ix * s + hs + e, iy * s + hs + e, iz * s + e};
        m.AddParticle(x0, zero);
        m.AddParticle(x1, zero);
        m.AddParticle(x2, zero);
        m.AddParticle(x3, zero);
      }
}

}  // namespace mdghost
