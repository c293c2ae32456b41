// Host side of the GB300 engine in the reference's own language: the .cfg
// parser, SimulationInfo, an MDManager stand-in for one box on one GPU, and
// the initial-condition makers the reference's projects use.  Everything
// physical goes through the C ABI of include/mdg.h.
#pragma once
#include <map>
#include <random>
#include <string>
#include <vector>

#include "mdg.h"

namespace mdghost {

// Parameter (parameter.h:12-31, parameter.cc:35-110): key=value lines split
// at the first '=', no trimming, first occurrence kept, atof/atoi, booleans
// true only for "yes"/"Yes".
class Parameter {
 public:
  bool LoadFromFile(const std::string &path);
  void ReadFromString(const std::string &text);
  bool Contains(const std::string &key) const { return params_.count(key) != 0; }
  std::string GetStringDef(const std::string &key, const std::string &def) const;
  double GetDoubleDef(const std::string &key, double def) const;
  int GetIntegerDef(const std::string &key, int def) const;
  bool GetBooleanDef(const std::string &key, bool def) const;
  bool IsValid() const { return valid_; }

 private:
  std::map<std::string, std::string> params_;
  bool valid_ = true;
};

// SimulationInfo (simulationinfo.cc:5-51) plus the engine's keys:
// CutoffLength (3.0), BufferLength (0.3), Precision (fp64|mixed),
// LangevinHalfDriftCompat (yes).
struct SimulationInfo {
  explicit SimulationInfo(const Parameter &p);
  double L[3] = {0, 0, 0};
  double TimeStep, AimedTemperature, HeatbathTau, HeatbathGamma;
  bool ControlTemperature;
  int HeatbathType;  // 0 NoseHoover, 1 Langevin
  double CutoffLength, BufferLength;
  int Precision;     // MDG_FP64 / MDG_MIXED / MDG_MIXED_PLAIN
  bool LangevinHalfDriftCompat;
  int Device;        // CUDA ordinal from Device=gpu (0) or gpu:<ordinal>
  int RebuildPolicy; // mdg_rebuild_policy from RebuildPolicy=halfmargin|reference
  int CheckListLength;  // simulationinfo.cc:27, the reference policy's candidate limit
};

// MDManager for one box (mdmanager.h:32-83).  Particles are staged on the
// host by AddParticle (MDUnit::AddParticle, mdunit.cc:44-49) and handed to
// the device at MakePairList.
class MDManager {
 public:
  MDManager(const Parameter &param, int capacity);
  ~MDManager();
  MDManager(const MDManager &) = delete;
  MDManager &operator=(const MDManager &) = delete;

  void AddParticle(const double x[3], const double v[3]);
  int GetParticleNumber() const { return (int)q_.size() / 4; }
  unsigned long GetTotalParticleNumber() const { return (unsigned long)GetParticleNumber(); }
  // Variables::SetInitialVelocity (variables.cc:82-108): isotropic, fixed speed V0.
  void SetInitialVelocity(double v0, int seed);

  void MakePairList();
  void Calculate();
  void Calculate(int nsteps);

  double KineticEnergy();
  double PotentialEnergy();
  double Temperature();
  double Pressure();
  double TotalEnergy();
  double GetSimulationTime() const { return s_time_; }
  const double *GetSystemSize() const { return sinfo_.L; }

  void SetSeed(int seed);
  void SetControlTemperature(bool b);
  void SetAimedTemperature(double t);

  // state exchange in the reference's [n][4] layout
  void GetState(std::vector<double> &q4, std::vector<double> &p4);
  void SaveStateRaw(const std::string &path);  // int64 n, n x {q,p}
  // the reference's makers + SetInitialVelocity(v0) on the device (mdg_make_state)
  void MakeStateOnDevice(int maker, double density, double radius, double v0);
  // the reference's writers (mdmanager.h:54-57): conf%04d.dump / conf%04d.cd
  // in the working directory for the Sequential forms
  void SaveAsDumpFile(const char *filename);
  void SaveAsDumpFileSequential();
  void SaveAsCdview(const char *filename);
  void SaveAsCdviewSequential();
  mdg_handle *Handle() { return h_; }

 private:
  void Check(int rc, const char *what);
  void Observe(double out[3]);
  void Sync();
  SimulationInfo sinfo_;
  mdg_handle *h_ = nullptr;
  std::vector<double> q_, p_;
  bool uploaded_ = false;
  double s_time_ = 0.0;
  int dump_index_ = 0, cdview_index_ = 0;
};

// ConfigurationMaker (confmaker.cc:9-44): FCC sites with a 1e-7 offset.
void MakeFCC(const Parameter &param, MDManager &m);

}  // namespace mdghost
