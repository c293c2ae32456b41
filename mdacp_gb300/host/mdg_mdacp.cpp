// mdg_mdacp: runs MDACP's Benchmark, Langevin, Collision and Burst projects
// (benchmark.cc:12-52, langevin.cc:9-32, collision.cc:55-81, burst.cc:103-140)
// on one GB300 through the C ABI.  Usage: mdg_mdacp [input.cfg]
// (the reference reads input.cfg when no file is given, mdmanager.cc:18-23).
//
// Output lines keep the reference's layout: "time T P E #observe" every
// ObserveLoop steps and "# N = n sec [SEC] mups [MUPS]" at the end.  The
// initial state is the reference project's: Benchmark uses
// ExtractConfigurationMaker (benchmark.cc:15-19, Density default 0.7), made on
// the device; Langevin uses ConfigurationMaker's sites with the 1e-7 offset
// (langevin.cc:12-15, Density default 0.5), made on the host; both give the
// fixed-speed isotropic velocity of Variables::SetInitialVelocity seeded with
// the unit id 0.  Extra keys: InitialConfiguration=extract|fcc overrides the
// project's maker; InitialStateFile=<path> writes the initial state (int64 n,
// n x {q, p}); FinalDumpFile / FinalCdviewFile write the final state.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "mdg_host.hpp"

namespace {

double now() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int lattice_count(const mdghost::Parameter &param) {
  const mdghost::SimulationInfo si(param);
  const double s = 1.0 / pow(param.GetDoubleDef("Density", 0.5) * 0.25, 1.0 / 3.0);
  return 4 * (int)(si.L[0] / s) * (int)(si.L[1] / s) * (int)(si.L[2] / s);
}

void observe_line(mdghost::MDManager &m, bool tag) {
  const double T = m.Temperature(), P = m.Pressure(), E = m.TotalEnergy();
  printf("%.15g %.15g %.15g %.15g%s\n", m.GetSimulationTime(), T, P, E, tag ? " #observe" : "");
}

std::string maker_of(const mdghost::Parameter &param, const char *project_default) {
  return param.GetStringDef("InitialConfiguration", project_default);
}

// Particles the project's maker places (the handle's capacity).
int maker_count(const mdghost::Parameter &param, const std::string &maker) {
  if (maker == "extract") {
    const mdghost::SimulationInfo si(param);
    return (int)(si.L[0] * si.L[1] * si.L[2] * param.GetDoubleDef("Density", 0.7));
  }
  return lattice_count(param);
}

void setup(const mdghost::Parameter &param, mdghost::MDManager &m, const std::string &maker) {
  const double v0 = param.GetDoubleDef("InitialVelocity", 1.0);
  if (maker == "extract") {
    m.MakeStateOnDevice(MDG_MAKER_EXTRACT, param.GetDoubleDef("Density", 0.7), 0.0, v0);
  } else {
    mdghost::MakeFCC(param, m);
    m.SetInitialVelocity(v0, 0);
  }
  if (param.Contains("InitialStateFile")) m.SaveStateRaw(param.GetStringDef("InitialStateFile", ""));
}

// Added keys FinalDumpFile / FinalCdviewFile: the final state in the
// reference's dump (SaveAsDumpFile) and CDView (SaveAsCdview) formats.
void final_files(const mdghost::Parameter &param, mdghost::MDManager &m) {
  if (param.Contains("FinalDumpFile")) m.SaveAsDumpFile(param.GetStringDef("FinalDumpFile", "").c_str());
  if (param.Contains("FinalCdviewFile")) m.SaveAsCdview(param.GetStringDef("FinalCdviewFile", "").c_str());
}

void run_benchmark(const mdghost::Parameter &param) {
  const std::string maker = maker_of(param, "extract");
  const int n = maker_count(param, maker);
  mdghost::MDManager m(param, n > 0 ? n : 1);
  setup(param, m, maker);
  const int T_LOOP = param.GetIntegerDef("ThermalizeLoop", 150);
  const int LOOP = param.GetIntegerDef("TotalLoop", 1000);
  const int OBSERVE_LOOP = param.GetIntegerDef("ObserveLoop", 100);
  printf("# Number of Particles = %lu\n", m.GetTotalParticleNumber());
  m.MakePairList();
  if (T_LOOP > 0) m.Calculate(T_LOOP);
  const double start = now();
  for (int i = 0; i < LOOP;) {
    // steps up to and including the next observation point run as one call
    int next = i + 1;
    if (i % OBSERVE_LOOP != 0) next = ((i / OBSERVE_LOOP) + 1) * OBSERVE_LOOP + 1;
    if (next > LOOP) next = LOOP;
    m.Calculate(next - i);
    if ((next - 1) % OBSERVE_LOOP == 0) observe_line(m, true);
    i = next;
  }
  const double sec = now() - start;
  const unsigned long pn = m.GetTotalParticleNumber();
  printf("# N = %lu %g [SEC] %g [MUPS]\n", pn, sec, (double)LOOP * (double)pn / sec / 1.0e6);
  final_files(param, m);
}

void run_langevin(const mdghost::Parameter &param) {
  const std::string maker = maker_of(param, "fcc");
  const int n = maker_count(param, maker);
  mdghost::MDManager m(param, n > 0 ? n : 1);
  setup(param, m, maker);
  const int LOOP = param.GetIntegerDef("TotalLoop", 1000);
  const int OBSERVE_LOOP = param.GetIntegerDef("ObserveLoop", 100);
  m.SetSeed(param.GetIntegerDef("Seed", 1));
  m.SetControlTemperature(true);
  printf("# Number of Particles = %lu\n", m.GetTotalParticleNumber());
  m.MakePairList();
  for (int i = 0; i < LOOP; i++) {
    m.Calculate();
    if (i % OBSERVE_LOOP == 0) observe_line(m, false);
  }
}

// Collision::Run (collision.cc:55-81): two balls of radius L_y / 4 at density
// 0.374 moving at +1 and -1 along x, made on the device; no SetInitialVelocity.
void run_collision(const mdghost::Parameter &param) {
  const mdghost::SimulationInfo si(param);
  const double radius = si.L[1] * 0.25, density = 0.374;
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const long is = (long)(2 * radius / s);
  const long sites = 8 * is * is * is;  // both balls' candidate sites bound the count
  if (sites > 2000000000L) throw std::runtime_error("collision balls too large");
  mdghost::MDManager m(param, sites > 0 ? (int)sites : 1);
  m.MakeStateOnDevice(MDG_MAKER_COLLISION, density, radius, 1.0);
  m.SaveAsCdviewSequential();
  const int OBSERVE_LOOP = param.GetIntegerDef("ObserveLoop", 100);
  const int TOTAL_LOOP = param.GetIntegerDef("TotalLoop", 1000);
  const bool save_cdview_file = param.GetBooleanDef("SaveCdviewFile", false);
  printf("# Number of Particles = %lu\n", m.GetTotalParticleNumber());
  for (int i = 0; i < TOTAL_LOOP; i++) {
    m.Calculate();
    if (i % OBSERVE_LOOP == 0) {
      printf("%.15g %.15g# observe\n", m.GetSimulationTime(), m.Temperature());
      if (save_cdview_file) m.SaveAsCdviewSequential();
    }
  }
  final_files(param, m);
}

// Burst::Run (burst.cc:103-140): a droplet of radius Radius (default 10) at
// Density (default 0.5) with SetInitialVelocity(InitialVelocity), thermalised
// ThermalizeLoop steps under the heat bath, then TotalLoop free steps.
void run_burst(const mdghost::Parameter &param) {
  const int n = lattice_count(param);
  mdghost::MDManager m(param, n > 0 ? n : 1);
  m.MakeStateOnDevice(MDG_MAKER_DROPLET, param.GetDoubleDef("Density", 0.5), param.GetDoubleDef("Radius", 10),
                      param.GetDoubleDef("InitialVelocity", 1.0));
  const int T_LOOP = param.GetIntegerDef("ThermalizeLoop", 150);
  const int LOOP = param.GetIntegerDef("TotalLoop", 1000);
  const int OBSERVE_LOOP = param.GetIntegerDef("ObserveLoop", 100);
  printf("# Number of Particles = %lu\n", m.GetTotalParticleNumber());
  m.MakePairList();
  m.SetControlTemperature(true);
  for (int i = 0; i < T_LOOP; i++) {
    m.Calculate();
    if (i % OBSERVE_LOOP == 0) m.SaveAsCdviewSequential();
  }
  m.SetControlTemperature(false);
  const double start = now();
  for (int i = 0; i < LOOP; i++) {
    m.Calculate();
    if (i % OBSERVE_LOOP == 0) {
      observe_line(m, true);
      m.SaveAsCdviewSequential();
    }
  }
  const double sec = now() - start;
  const unsigned long pn = m.GetTotalParticleNumber();
  printf("# N = %lu %g [SEC] %g [MUPS]\n", pn, sec, (double)LOOP * (double)pn / sec / 1.0e6);
  final_files(param, m);
}

}  // namespace

// mdg_mdacp --print-config file.cfg: the parsed simulation settings, no GPU use.
int print_config(const std::string &path) {
  mdghost::Parameter param;
  if (!param.LoadFromFile(path)) return 1;
  try {
    const mdghost::SimulationInfo si(param);
    printf("L %.17g %.17g %.17g\n", si.L[0], si.L[1], si.L[2]);
    printf("TimeStep %.17g\nAimedTemperature %.17g\nHeatbathTau %.17g\nHeatbathGamma %.17g\n", si.TimeStep,
           si.AimedTemperature, si.HeatbathTau, si.HeatbathGamma);
    printf("ControlTemperature %d\nHeatbathType %d\nCutoffLength %.17g\nBufferLength %.17g\n",
           si.ControlTemperature ? 1 : 0, si.HeatbathType, si.CutoffLength, si.BufferLength);
    printf("Precision %d\nLangevinHalfDriftCompat %d\nMode %s\nlattice %d\n", si.Precision,
           si.LangevinHalfDriftCompat ? 1 : 0, param.GetStringDef("Mode", "").c_str(), lattice_count(param));
    printf("RebuildPolicy %d\nCheckListLength %d\n", si.RebuildPolicy, si.CheckListLength);
  } catch (const std::exception &e) {
    printf("error %s\n", e.what());
    return 2;
  }
  return 0;
}

int main(int argc, char **argv) {
  setvbuf(stdout, nullptr, _IOLBF, 0);
  if (argc > 2 && std::string(argv[1]) == "--print-config") return print_config(argv[2]);
  printf("# %s\n", mdg_version());
  const std::string input = argc > 1 ? argv[1] : "input.cfg";
  mdghost::Parameter param;
  if (!param.LoadFromFile(input)) {
    printf("Could not open input file %s\n", input.c_str());
    printf("Program is aborted.\n");
    return 1;
  }
  if (!param.Contains("Mode")) {
    printf("Mode is not defined in inputfile.\n");
    return 1;
  }
  const std::string mode = param.GetStringDef("Mode", "");
  printf("# Mode = %s\n", mode.c_str());
  try {
    if (mode == "Benchmark") run_benchmark(param);
    else if (mode == "Langevin") run_langevin(param);
    else if (mode == "Collision") run_collision(param);
    else if (mode == "Burst") run_burst(param);
    else {
      printf("Mode %s is not found.\n", mode.c_str());
      return 1;
    }
  } catch (const std::exception &e) {
    printf("# Error: %s\n", e.what());
    return 2;
  }
  return 0;
}
