"""The .cfg semantics of parameter.cc / simulationinfo.cc and the added keys."""
import pytest

from mdacp_gb300.config import Parameter, SimulationInfo, atof, atoi


def test_parameter_semantics():
    p = Parameter("Mode=Benchmark\nTimeStep=0.005\nTimeStep=0.1\n#Density=0.9\nflag=Yes\nflag2=true\n x=1\nnoeq\n")
    assert p.get_string("Mode") == "Benchmark"
    assert p.get_double("TimeStep") == 0.005          # first occurrence wins (std::map::insert)
    assert p.contains("#Density") and not p.contains("Density")  # no comment syntax
    assert p.get_bool("flag") and not p.get_bool("flag2")         # only yes / Yes
    assert p.contains(" x") and not p.contains("x")    # no trimming
    assert p.get_int("missing", 7) == 7


def test_atof_atoi_prefix():
    assert atof("1.5e2abc") == 150.0 and atof("abc") == 0.0 and atof(" -2.") == -2.0
    assert atoi("42x") == 42 and atoi("x") == 0 and atoi("3.9") == 3


def test_simulationinfo_defaults_are_reference():
    si = SimulationInfo(Parameter("SystemSize=50\n"))
    assert si.cutoff == 3.0 and si.buffer_length == 0.3 and si.search_length == 3.3
    assert si.time_step == 0.001 and si.heatbath_tau == 0.1 and si.heatbath_gamma == 0.1
    assert si.L == [50.0, 50.0, 50.0] and si.thermostat == "nve"
    assert si.precision == "fp64" and si.langevin_half_drift_compat


def test_simulationinfo_keys():
    si = SimulationInfo(Parameter("UnitLength=20\nSystemSizeZ=7\nControlTemperature=yes\nHeatbathType=Langevin\n"
                                  "CutoffLength=2.5\nBufferLength=0.5\nPrecision=mixed\n"), grid_size=(2, 1, 1))
    assert si.L == [40.0, 20.0, 7.0] and si.thermostat == "langevin"
    assert si.search_length == 3.0 and si.precision == "mixed"
    assert SimulationInfo(Parameter("ControlTemperature=yes\n")).thermostat == "nosehoover"
    with pytest.raises(ValueError):
        SimulationInfo(Parameter("HeatbathType=Berendsen\n"))


def test_engine_keys_device_and_rebuild_policy():
    # Device selects the GPU ordinal (the engine has no CPU path); two rebuild
    # rules (half the margin, the reference's budget and check with its
    # CheckListLength); Precision takes the plain-sum mixed form too
    assert SimulationInfo(Parameter("")).device == 0
    assert SimulationInfo(Parameter("Device=gpu:3\n")).device == 3
    assert SimulationInfo(Parameter("Precision=mixed_plain\n")).precision == "mixed_plain"
    assert SimulationInfo(Parameter("")).rebuild_policy == "halfmargin"
    si = SimulationInfo(Parameter("RebuildPolicy=reference\nCheckListLength=64\n"))
    assert si.rebuild_policy == "reference" and si.check_list_length == 64
    for bad in ("Device=cpu\n", "Device=gpu:x\n", "RebuildPolicy=budget\n", "Precision=f16\n"):
        with pytest.raises(ValueError):
            SimulationInfo(Parameter(bad))
