// Oracle harness for the MDACP reference (test infrastructure, never shipped).
//
// An extra MDACP Project, registered under Mode=Oracle exactly the way the
// reference's own projects register themselves (benchmark.h:11-13,
// projectmanager.cc:7-13).  It runs the UNMODIFIED reference call points
// (MDManager::MakePairList / Calculate / SendBorderParticles, MDUnit::
// CalculateForce, the observers) on an injected state and dumps what the
// parity tests need.  Everything is reached through the reference's public
// API; the pair list is read through the DoubleObserver hook
// (observer.h:13-16, mdunit.h:73), which hands an observer the unit's MeshList.
//
// .cfg keys read here (all other keys are the reference's own):
//   OracleTask=pairs|force|trace|bench|write|make   what to run
//   OracleMaker=fcc|extract|collision|droplet (task make: ConfigurationMaker or
//     ExtractConfigurationMaker on the empty system, then
//     MDManager::SetInitialVelocity(InitialVelocity); Density as the reference
//     reads it.  collision and droplet run the reference's own Collision::Run
//     (collision.cc:55-81) and Burst::Run (burst.cc:103-140), whose makers are
//     local to those files, with TotalLoop=0 (and ThermalizeLoop=0) in the
//     .cfg so that only their set-up runs)
//   OracleInput=<file>                    int64 n, then n x {qx qy qz px py pz} doubles
//   OracleOutput=<prefix>                 output file prefix
//   OracleBufferLength=<margin>           overrides BufferLength (simulationinfo.cc:6)
//   OracleSteps, ObserveLoop, ThermalizeLoop, Seed
//
// Particle identity: the input index is stored in Variables::type, which the
// reference carries through migration (mdunit.cc:87,118) and uses for nothing
// else on this path.
#include <cstddef>
#include <cstdint>
#include <fstream>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include <tuple>
#include <omp.h>
#include "projectmanager.h"
#include "confmaker.h"
#include "collision.h"
#include "burst.h"

extern Collision coll;  // collision.cc:6
extern Burst burst;     // burst.cc:8
#include "communicator.h"
#include "mpistream.h"

namespace {

struct InputState {
  std::vector<double> qp;  // n x 6
  int64_t n = 0;
};

bool read_input(const std::string &fn, InputState &s) {
  FILE *f = fopen(fn.c_str(), "rb");
  if (!f) return false;
  if (fread(&s.n, sizeof(int64_t), 1, f) != 1) { fclose(f); return false; }
  s.qp.resize((size_t)s.n * 6);
  size_t got = fread(s.qp.data(), sizeof(double), s.qp.size(), f);
  fclose(f);
  return got == s.qp.size();
}

class Loader : public Executor {
  const InputState &s;
  bool zero_p;
 public:
  Loader(const InputState &s_, bool zp) : s(s_), zero_p(zp) {}
  void Execute(MDUnit *mdu) {
    for (int64_t i = 0; i < s.n; i++) {
      double x[D] = {s.qp[6 * i + 0], s.qp[6 * i + 1], s.qp[6 * i + 2], 0.0};
      double v[D] = {0.0, 0.0, 0.0, 0.0};
      if (!zero_p) { v[X] = s.qp[6 * i + 3]; v[Y] = s.qp[6 * i + 4]; v[Z] = s.qp[6 * i + 5]; }
      mdu->AddParticle(x, v, (int)i);
    }
  }
};

// SimulationInfo is owned privately by MDManager; GetSystemSize() returns its
// first member L, from which the object itself is recovered.
SimulationInfo *sim_info(MDManager *mdm) {
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Winvalid-offsetof"
  return reinterpret_cast<SimulationInfo *>(reinterpret_cast<char *>(mdm->GetSystemSize()) -
                                            offsetof(SimulationInfo, L));
#pragma GCC diagnostic pop
}

// Resolves every ghost of one unit to (input id, image shift) and writes the
// directed pair records (key id, partner id, sx, sy, sz) of the half list.
class PairDumper : public DoubleObserver {
  FILE *out;
  const double *L;
 public:
  int64_t written = 0;
  PairDumper(FILE *f, const double *L_) : out(f), L(L_) {}
  double Observe(Variables *vars, MeshList *mesh) {
    const int pn = vars->GetParticleNumber();
    typedef std::tuple<uint64_t, uint64_t, uint64_t> Key;
    std::map<Key, std::pair<int, int>> images;  // bit pattern -> (real index, shift code)
    for (int j = 0; j < pn; j++) {
      for (int sz = -1; sz <= 1; sz++)
        for (int sy = -1; sy <= 1; sy++)
          for (int sx = -1; sx <= 1; sx++) {
            if (!sx && !sy && !sz) continue;
            double x = vars->q[j][X] + (sx ? sx * L[X] : 0.0);
            double y = vars->q[j][Y] + (sy ? sy * L[Y] : 0.0);
            double z = vars->q[j][Z] + (sz ? sz * L[Z] : 0.0);
            uint64_t bx, by, bz;
            memcpy(&bx, &x, 8); memcpy(&by, &y, 8); memcpy(&bz, &z, 8);
            images[Key(bx, by, bz)] = std::make_pair(j, (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1));
          }
    }
    const int tn = vars->GetTotalParticleNumber();
    std::vector<std::pair<int, int>> ghost(tn, std::make_pair(-1, 13));
    for (int g = pn; g < tn; g++) {
      uint64_t bx, by, bz;
      memcpy(&bx, &vars->q[g][X], 8); memcpy(&by, &vars->q[g][Y], 8); memcpy(&bz, &vars->q[g][Z], 8);
      auto it = images.find(Key(bx, by, bz));
      if (it != images.end()) ghost[g] = it->second;
    }
    const int np = mesh->GetPairNumber();
    const int *key = mesh->GetKeyParticles();
    const int *partner = mesh->GetPartnerParticles();
    for (int k = 0; k < np; k++) {
      int a = key[k], b = partner[k];
      int32_t rec[3];
      rec[0] = vars->type[a];
      if (b < pn) { rec[1] = vars->type[b]; rec[2] = 13; }
      else { rec[1] = ghost[b].first >= 0 ? vars->type[ghost[b].first] : -1; rec[2] = ghost[b].second; }
      fwrite(rec, sizeof(int32_t), 3, out);
      written++;
    }
    return 0.0;
  }
};

// Unit particles in order: q, p (6 doubles each).
class OrderDumper : public Executor {
  FILE *out;
 public:
  OrderDumper(FILE *f) : out(f) {}
  void Execute(MDUnit *mdu) {
    Variables *v = mdu->GetVariables();
    for (int i = 0; i < v->GetParticleNumber(); i++) {
      double rec[6] = {v->q[i][X], v->q[i][Y], v->q[i][Z], v->p[i][X], v->p[i][Y], v->p[i][Z]};
      fwrite(rec, sizeof(double), 6, out);
    }
  }
};

class StateDumper : public Executor {
  FILE *out;
 public:
  StateDumper(FILE *f) : out(f) {}
  void Execute(MDUnit *mdu) {
    Variables *v = mdu->GetVariables();
    for (int i = 0; i < v->GetParticleNumber(); i++) {
      double rec[7] = {(double)v->type[i], v->q[i][X], v->q[i][Y], v->q[i][Z], v->p[i][X], v->p[i][Y], v->p[i][Z]};
      fwrite(rec, sizeof(double), 7, out);
    }
  }
};

void observe_row(MDManager *mdm, SimulationInfo *sinfo, int step, FILE *f) {
  mdm->SendBorderParticles();  // fresh ghost images before observing
  double row[7];
  row[0] = step;
  row[1] = mdm->Temperature();
  row[2] = mdm->Pressure();
  row[3] = mdm->TotalEnergy();
  row[4] = mdm->KineticEnergy();
  row[5] = mdm->PotentialEnergy();
  VirialObserver vobs;
  row[6] = mdm->ObserveDouble(&vobs) / (double)mdm->GetTotalParticleNumber();
  (void)sinfo;
  fwrite(row, sizeof(double), 7, f);
}

class OracleProject : public Project {
 public:
  OracleProject() { ProjectManager::GetInstance().AddProject("Oracle", this); }
  void Run(MDManager *mdm) {
    Parameter *param = mdm->GetParameter();
    SimulationInfo *sinfo = sim_info(mdm);
    const std::string task = param->GetStringDef("OracleTask", "force");
    const std::string out = param->GetStringDef("OracleOutput", "oracle_out");
    if (param->Contains("OracleBufferLength")) {
      sinfo->BufferLength = param->GetDouble("OracleBufferLength");
      sinfo->SearchLength = CUTOFF_LENGTH + sinfo->BufferLength;
      for (int i = 0; i < mdm->GetTotalThreads(); i++) mdm->GetMDUnit(i)->ChangeScale(1.0);
    }
    if (task == "make") {
      const std::string maker = param->GetStringDef("OracleMaker", "fcc");
      if (maker == "collision") {
        coll.Run(mdm);
      } else if (maker == "droplet") {
        burst.Run(mdm);
      } else {
        if (maker == "extract") {
          ExtractConfigurationMaker c(param);
          mdm->ExecuteAll(&c);
        } else {
          ConfigurationMaker c(param);
          mdm->ExecuteAll(&c);
        }
        if (param->Contains("InitialVelocity")) mdm->SetInitialVelocity(param->GetDouble("InitialVelocity"));
      }
      FILE *f = fopen((out + "_made.bin").c_str(), "wb");
      OrderDumper od(f);
      mdm->ExecuteAllSerial(&od);
      fclose(f);
      return;
    }
    InputState s;
    if (!read_input(param->GetStringDef("OracleInput", "oracle_in.bin"), s)) {
      mout << "# Oracle: cannot read input" << std::endl;
      return;
    }
    Loader loader(s, task == "force");
    mdm->ExecuteAll(&loader);
    if ((int64_t)mdm->GetTotalParticleNumber() != s.n) {
      mout << "# Oracle: loaded " << mdm->GetTotalParticleNumber() << " of " << s.n << std::endl;
    }
    if (task == "pairs") {
      mdm->MakePairList();
      FILE *f = fopen((out + "_pairs.bin").c_str(), "wb");
      PairDumper pd(f, sinfo->L);
      mdm->ObserveDouble(&pd);
      fclose(f);
    } else if (task == "force") {
      sinfo->TimeStep = 1.0;  // ForceCalculator folds dt into the kick; dt=1 makes p the force
      mdm->MakePairList();
      for (int i = 0; i < mdm->GetTotalThreads(); i++) mdm->GetMDUnit(i)->CalculateForce();
      FILE *f = fopen((out + "_force.bin").c_str(), "wb");
      StateDumper sd(f);
      mdm->ExecuteAllSerial(&sd);
      fclose(f);
      FILE *g = fopen((out + "_obs.bin").c_str(), "wb");
      PotentialEnergyObserver pobs(sinfo);
      VirialObserver vobs;
      double obs[2] = {mdm->ObserveDouble(&pobs), mdm->ObserveDouble(&vobs)};
      fwrite(obs, sizeof(double), 2, g);
      fclose(g);
    } else if (task == "trace") {
      const int steps = param->GetIntegerDef("OracleSteps", 100);
      const int every = param->GetIntegerDef("ObserveLoop", 10);
      if (sinfo->ControlTemperature) mdm->SetSeed(param->GetIntegerDef("Seed", 1));
      FILE *f = fopen((out + "_trace.bin").c_str(), "wb");
      mdm->MakePairList();
      observe_row(mdm, sinfo, 0, f);
      for (int i = 1; i <= steps; i++) {
        mdm->Calculate();
        if (i % every == 0) observe_row(mdm, sinfo, i, f);
      }
      fclose(f);
      FILE *g = fopen((out + "_state.bin").c_str(), "wb");
      StateDumper sd(g);
      mdm->ExecuteAllSerial(&sd);
      fclose(g);
    } else if (task == "write") {
      // the reference's writers on the loaded state (no step, no ghosts yet):
      // MDManager::SaveAsDumpFile, MDManager::SaveAsCdview,
      // MDUnit::SaveConfiguration (writes conf000.cnf), Variables::SaveToStream
      mdm->SaveAsDumpFile((out + "_dump.bin").c_str());
      mdm->SaveAsCdview((out + "_cdview.cd").c_str());
      mdm->GetMDUnit(0)->SaveConfiguration();
      std::ofstream fs((out + "_stream.bin").c_str(), std::ios::binary);
      mdm->GetMDUnit(0)->GetVariables()->SaveToStream(fs);
    } else if (task == "bench") {
      // Timed like Benchmark::Run (benchmark.cc:24-51): list build and warm-up
      // outside, the stepping loop with its periodic observation inside.
      const int warm = param->GetIntegerDef("ThermalizeLoop", 0);
      const int steps = param->GetIntegerDef("OracleSteps", 100);
      const int every = param->GetIntegerDef("ObserveLoop", 100);
      mdm->MakePairList();
      for (int i = 0; i < warm; i++) mdm->Calculate();
      double t0 = Communicator::GetTime();
      double acc = 0.0;
      for (int i = 0; i < steps; i++) {
        mdm->Calculate();
        if (i % every == 0) acc += mdm->Temperature() + mdm->Pressure() + mdm->TotalEnergy();
      }
      double sec = Communicator::GetTime() - t0;
      const unsigned long pn = mdm->GetTotalParticleNumber();
      printf("# N = %lu %.6f [SEC] %.6f [MUPS] threads=%d check=%.10g\n", pn, sec,
             (double)steps * (double)pn / sec / 1e6, mdm->GetTotalThreads(), acc);
    }
  }
};

OracleProject oracle_project;

}  // namespace
