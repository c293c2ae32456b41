""".cfg handling with the reference's semantics.

Parameter follows parameter.cc:35-110: one `key=value` per line split at the
first '=', no trimming, no comments (a `#key=v` line is stored under `#key`),
first occurrence wins (std::map::insert), atof/atoi conversions (leading
numeric prefix, 0 when none), booleans true only for `yes` / `Yes`.

SimulationInfo follows simulationinfo.cc:5-51 for the reference keys and adds
the keys of this engine, whose defaults keep the reference behaviour:
  CutoffLength (3.0, CUTOFF_LENGTH of mdconfig.h:15), BufferLength (0.3,
  simulationinfo.cc:6), Precision (fp64|mixed|mixed_plain), Device (gpu or
  gpu:<ordinal>), RebuildPolicy (halfmargin: rebuild once a particle moved
  half the margin; reference: the buffer budget and displacement check of
  pairlist.cc:26-121, with CheckListLength), LangevinHalfDriftCompat (yes).
"""
import re

_NUM = re.compile(r"^[ \t\n\v\f\r]*([+-]?(\d+(\.\d*)?|\.\d+)([eE][+-]?\d+)?)")
_INT = re.compile(r"^[ \t\n\v\f\r]*([+-]?\d+)")


def parse_device(value):
    """Device=gpu or gpu:<ordinal> -> the CUDA device ordinal.  The engine runs
    only on the GPU; Device=cpu is the reference's own path."""
    if value == "gpu":
        return 0
    if value.startswith("gpu:") and value[4:].isdigit():
        return int(value[4:])
    raise ValueError("Device=%s: this engine runs on the GPU (Device=gpu or gpu:<ordinal>)" % value)


def atof(s):
    m = _NUM.match(s)
    return float(m.group(1)) if m else 0.0


def atoi(s):
    m = _INT.match(s)
    return int(m.group(1)) if m else 0


class Parameter:
    def __init__(self, text=""):
        self.params = {}
        self.valid = True
        self.read(text)

    @classmethod
    def from_file(cls, path):
        p = cls()
        try:
            with open(path) as f:
                p.read(f.read())
        except OSError:
            p.valid = False
        return p

    def read(self, text):
        for line in text.split("\n"):
            if "=" in line:
                k, v = line.split("=", 1)
                self.params.setdefault(k, v)

    def contains(self, key):
        return key in self.params

    def get_string(self, key, default=""):
        return self.params.get(key, default)

    def get_double(self, key, default=0.0):
        return atof(self.params[key]) if key in self.params else default

    def get_int(self, key, default=0):
        return atoi(self.params[key]) if key in self.params else default

    def get_bool(self, key, default=False):
        if key not in self.params:
            return default
        return self.params[key] in ("yes", "Yes")


class SimulationInfo:
    def __init__(self, param, grid_size=(1, 1, 1)):
        self.cutoff = param.get_double("CutoffLength", 3.0)
        self.buffer_length = param.get_double("BufferLength", 0.3)
        self.search_length = self.cutoff + self.buffer_length
        self.time_step = param.get_double("TimeStep", 0.001)
        self.is_periodic = param.get_bool("IsPeriodic", True)
        self.aimed_temperature = param.get_double("AimedTemperature", 1.0)
        self.control_temperature = param.get_bool("ControlTemperature", False)
        self.heatbath_tau = param.get_double("HeatbathTau", 0.1)
        self.heatbath_gamma = param.get_double("HeatbathGamma", 0.1)
        self.sort_particle = param.get_bool("SortParticle", False)
        hb = param.get_string("HeatbathType", "NoseHoover")
        if hb not in ("NoseHoover", "Langevin"):
            raise ValueError("Unknown Heatbath type " + hb)
        self.heatbath_type = hb
        self.check_list_length = param.get_int("CheckListLength", 500)
        L = [0.0, 0.0, 0.0]
        if param.contains("SystemSize"):
            L = [param.get_double("SystemSize")] * 3
        elif param.contains("UnitLength"):
            ul = param.get_double("UnitLength")
            L = [ul * grid_size[0], ul * grid_size[1], ul * grid_size[2]]
        for k, key in enumerate(("SystemSizeX", "SystemSizeY", "SystemSizeZ")):
            if param.contains(key):
                L[k] = param.get_double(key)
        self.L = L
        self.precision = param.get_string("Precision", "fp64")
        if self.precision not in ("fp64", "mixed", "mixed_plain"):
            raise ValueError("Precision must be fp64, mixed or mixed_plain")
        self.device = parse_device(param.get_string("Device", "gpu"))
        self.rebuild_policy = param.get_string("RebuildPolicy", "halfmargin")
        if self.rebuild_policy not in ("halfmargin", "reference"):
            raise ValueError("RebuildPolicy=%s: halfmargin (rebuild once a particle moved half the margin) or "
                             "reference (the buffer budget and displacement check of PairList)" % self.rebuild_policy)
        self.langevin_half_drift_compat = param.get_bool("LangevinHalfDriftCompat", True)

    @property
    def thermostat(self):
        if not self.control_temperature:
            return "nve"
        return "langevin" if self.heatbath_type == "Langevin" else "nosehoover"
