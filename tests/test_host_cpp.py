"""The C++ host front-end (mdacp_gb300/host): builds, parses .cfg like the reference,
and (GPU) runs MDACP's Benchmark project with results matching the oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

from mdacp_gb300 import build
from mdacp_gb300.config import Parameter, SimulationInfo


@pytest.fixture(scope="module")
def host_bin():
    try:
        build.build()
        return build.build_host()
    except RuntimeError as e:
        pytest.skip("toolchain unavailable: %s" % e)


def _cfg(tmp_path, text):
    p = tmp_path / "in.cfg"
    p.write_text(text)
    return str(p)


def test_print_config_matches_python_semantics(host_bin, tmp_path):
    text = ("Mode=Benchmark\nSystemSize=16\nSystemSizeZ=18.5\nTimeStep=0.002\nTimeStep=9\nDensity=0.5\n"
            "ControlTemperature=Yes\nHeatbathType=Langevin\nCutoffLength=2.5\nBufferLength=0.5\nPrecision=mixed\n"
            "#AimedTemperature=3\nHeatbathGamma=0.7x\n")
    out = subprocess.run([host_bin, "--print-config", _cfg(tmp_path, text)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    kv = dict(line.split(" ", 1) for line in out.stdout.strip().splitlines())
    si = SimulationInfo(Parameter(text))
    assert [float(x) for x in kv["L"].split()] == si.L
    assert float(kv["TimeStep"]) == si.time_step == 0.002
    assert float(kv["AimedTemperature"]) == si.aimed_temperature == 1.0
    assert float(kv["HeatbathGamma"]) == si.heatbath_gamma == 0.7
    assert kv["ControlTemperature"] == "1" and kv["HeatbathType"] == "1" and kv["Precision"] == "1"
    assert float(kv["CutoffLength"]) == 2.5 and float(kv["BufferLength"]) == 0.5
    assert int(kv["lattice"]) == 4 * 8 * 8 * 9


def test_rebuild_policy_keys(host_bin, tmp_path):
    # RebuildPolicy (halfmargin by default, or the reference's PairList
    # policy) and its CheckListLength, read as the Python mirror reads them
    for text, policy, cl in (("", 0, 500), ("RebuildPolicy=reference\nCheckListLength=64\n", 1, 64)):
        out = subprocess.run([host_bin, "--print-config", _cfg(tmp_path, text)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        kv = dict(line.split(" ", 1) for line in out.stdout.strip().splitlines())
        si = SimulationInfo(Parameter(text))
        assert int(kv["RebuildPolicy"]) == policy == {"halfmargin": 0, "reference": 1}[si.rebuild_policy]
        assert int(kv["CheckListLength"]) == cl == si.check_list_length
    out = subprocess.run([host_bin, "--print-config", _cfg(tmp_path, "RebuildPolicy=budget\n")], capture_output=True,
                         text=True)
    assert out.returncode == 2 and "RebuildPolicy=budget" in out.stdout


def test_bad_heatbath_rejected(host_bin, tmp_path):
    out = subprocess.run([host_bin, "--print-config", _cfg(tmp_path, "HeatbathType=Foo\n")], capture_output=True,
                         text=True)
    assert out.returncode == 2 and "Unknown Heatbath" in out.stdout


@pytest.mark.gpu
def test_benchmark_project_matches_oracle(host_bin, tmp_path):
    from oracle import port
    init = str(tmp_path / "init.bin")
    # ConfigurationMaker sites: the extract lattice puts sites on the box faces,
    # where the reference's ghost search misses images until the first rebuild
    text = ("Mode=Benchmark\nSystemSize=16\nDensity=0.5\nInitialVelocity=1.7320508\nThermalizeLoop=0\n"
            "TotalLoop=200\nObserveLoop=50\nTimeStep=0.001\nCutoffLength=2.5\nBufferLength=0.5\n"
            "InitialConfiguration=fcc\n"
            "InitialStateFile=%s\nFinalDumpFile=%s\n" % (init, tmp_path / "final.dump"))
    out = subprocess.run([host_bin, _cfg(tmp_path, text)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = np.array([[float(x) for x in l.split()[:4]] for l in out.stdout.splitlines() if l.endswith("#observe")])
    assert re.search(r"# N = 2048 .* \[MUPS\]", out.stdout)
    raw = np.fromfile(init, dtype="<f8", offset=8).reshape(-1, 6)
    s = port.System(raw[:, :3], raw[:, 3:], 16.0, rc=2.5, margin=0.5, dt=0.001)
    s.make_pairlist()
    ref, done = [], 0
    for c in (1, 51, 101, 151):
        s.calculate(c - done)
        done = c
        T, P, E = s.observe()[:3]
        ref.append([c * 0.001, T, P, E])
    np.testing.assert_allclose(rows, np.array(ref), rtol=1e-10, atol=1e-12)
    # the final state in the reference's dump format (qx qy qz px py pz doubles)
    s.calculate(200 - done)
    qf, pf = s.state()
    dump = np.fromfile(tmp_path / "final.dump", dtype="<f8").reshape(-1, 6)
    assert dump.shape == (2048, 6)
    dq = (dump[:, :3] - qf + 8.0) % 16.0 - 8.0
    assert np.abs(dq).max() < 1e-9 and np.abs(dump[:, 3:] - pf).max() < 1e-9


@pytest.mark.gpu
def test_langevin_project_runs(host_bin, tmp_path):
    text = ("Mode=Langevin\nSystemSize=16\nDensity=0.5\nInitialVelocity=1.8\nTimeStep=0.005\nTotalLoop=2000\n"
            "ObserveLoop=100\nAimedTemperature=0.9\nHeatbathType=Langevin\nHeatbathGamma=1.0\nSeed=12345\n"
            "CutoffLength=2.5\nBufferLength=0.5\n")
    out = subprocess.run([host_bin, _cfg(tmp_path, text)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    T = np.array([float(l.split()[1]) for l in out.stdout.splitlines() if l and l[0].isdigit()])
    assert len(T) == 20 and abs(T[10:].mean() - 0.9) < 0.08


@pytest.mark.gpu
def test_benchmark_project_starts_from_the_reference_extract_state(host_bin, tmp_path):
    # Benchmark::Run makes ExtractConfigurationMaker's state (benchmark.cc:15-19)
    from oracle import port
    init = str(tmp_path / "init.bin")
    text = ("Mode=Benchmark\nSystemSize=20\nDensity=0.6\nInitialVelocity=1.2\nThermalizeLoop=0\nTotalLoop=20\n"
            "ObserveLoop=10\nTimeStep=0.001\nCutoffLength=2.5\nBufferLength=0.5\nInitialStateFile=%s\n" % init)
    out = subprocess.run([host_bin, _cfg(tmp_path, text)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    raw = np.fromfile(init, dtype="<f8", offset=8).reshape(-1, 6)
    q = port.make_configuration("extract", 20.0, 0.6)
    assert raw.shape[0] == len(q) == int(20.0 ** 3 * 0.6)
    assert np.array_equal(raw[:, :3], q)
    np.testing.assert_allclose(raw[:, 3:], port.initial_velocity(len(q), 1.2, 0), rtol=0, atol=1e-13)


@pytest.mark.gpu
def test_collision_project_matches_oracle(host_bin, tmp_path):
    # Collision::Run: the two balls made on the device, then NVE steps with a
    # temperature line every ObserveLoop steps and the initial CDView file
    from oracle import port
    text = ("Mode=Collision\nSystemSizeX=60\nSystemSizeY=30\nSystemSizeZ=30\nTimeStep=0.002\nTotalLoop=100\n"
            "ObserveLoop=20\nCutoffLength=2.5\nBufferLength=0.5\nFinalDumpFile=%s\n" % (tmp_path / "final.dump"))
    out = subprocess.run([host_bin, _cfg(tmp_path, text)], capture_output=True, text=True, timeout=300,
                         cwd=str(tmp_path))
    assert out.returncode == 0, out.stdout + out.stderr
    rows = np.array([[float(x) for x in l.replace("# observe", "").split()] for l in out.stdout.splitlines()
                     if l.endswith("# observe")])
    L = np.array([60.0, 30.0, 30.0])
    q, p = port.make_state("collision", L, 0.374, 7.5, 1.0)
    first = np.loadtxt(tmp_path / "conf0000.cd")
    assert first.shape == (len(q), 8) and np.allclose(first[:, 2:5], q, rtol=1e-5)
    s = port.System(q, p, L, rc=2.5, margin=0.5, dt=0.002)
    s.make_pairlist()
    ref, done = [], 0
    for c in (1, 21, 41, 61, 81):
        s.calculate(c - done)
        done = c
        ref.append([c * 0.002, s.observe()[0]])
    np.testing.assert_allclose(rows, np.array(ref), rtol=1e-10, atol=1e-12)
    s.calculate(100 - done)
    qf, pf = s.state()
    dump = np.fromfile(tmp_path / "final.dump", dtype="<f8").reshape(-1, 6)
    dq = (dump[:, :3] - qf + L / 2) % L - L / 2
    assert np.abs(dq).max() < 1e-9 and np.abs(dump[:, 3:] - pf).max() < 1e-9


@pytest.mark.gpu
def test_burst_project_runs(host_bin, tmp_path):
    # Burst::Run: droplet + SetInitialVelocity, heat-bath thermalisation, then free steps
    text = ("Mode=Burst\nSystemSize=30\nDensity=0.8\nRadius=8\nInitialVelocity=0.9\nAimedTemperature=1.5\n"
            "HeatbathType=Langevin\nHeatbathGamma=1.0\nThermalizeLoop=200\nTotalLoop=200\nObserveLoop=100\n"
            "TimeStep=0.005\nCutoffLength=2.5\nBufferLength=0.5\n")
    out = subprocess.run([host_bin, _cfg(tmp_path, text)], capture_output=True, text=True, timeout=300,
                         cwd=str(tmp_path))
    assert out.returncode == 0, out.stdout + out.stderr
    from oracle import port
    q, _ = port.make_state("droplet", 30.0, 0.8, 8.0, 0.9)
    assert re.search(r"# N = %d .* \[MUPS\]" % len(q), out.stdout)
    assert len([l for l in out.stdout.splitlines() if l.endswith("#observe")]) == 2
    assert sorted(f for f in os.listdir(tmp_path) if f.endswith(".cd")) == ["conf%04d.cd" % i for i in range(4)]
