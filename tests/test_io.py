"""The reference's output and restart formats, byte for byte.

Golden bytes come from the reference's own writers (tests/golden/io_small.npz,
made by tests/golden/make_golden.py): MDManager::SaveAsDumpFile
(mdmanager.cc:475-505), MDUnit::SaveAsCdview (mdunit.cc:52-67, the harness
stores the input index as the particle type), Variables::SaveConfiguration
(variables.cc:45-56) and Variables::SaveToStream (variables.cc:111-118).  The
writers are host code of libmdg.so, so these tests run without a GPU; the
handle forms (state read back from the device) are marked gpu.
"""
import os
import struct

import numpy as np
import pytest

from mdacp_gb300 import io as mio

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "io_small.npz"))


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


def test_dump_matches_reference(tmp_path):
    fn = tmp_path / "conf.dump"
    mio.write_dump(fn, GOLD["q"], GOLD["p"])
    assert _bytes(fn) == GOLD["dump"].tobytes()


def test_cdview_matches_reference(tmp_path):
    fn = tmp_path / "conf.cd"
    mio.write_cdview(fn, GOLD["q"], GOLD["p"], types=np.arange(len(GOLD["q"])))
    assert _bytes(fn) == GOLD["cdview"].tobytes()


def test_configuration_matches_reference(tmp_path):
    fn = tmp_path / "conf000.cnf"
    mio.write_configuration(fn, GOLD["q"], GOLD["p"])
    assert _bytes(fn) == GOLD["configuration"].tobytes()


def test_stream_matches_reference(tmp_path):
    fn = tmp_path / "state.bin"
    mio.write_stream(fn, GOLD["q"], GOLD["p"])
    assert _bytes(fn) == GOLD["stream"].tobytes()


def test_append_concatenates(tmp_path):
    fn = tmp_path / "two.dump"
    q, p = GOLD["q"], GOLD["p"]
    mio.write_dump(fn, q[:50], p[:50])
    mio.write_dump(fn, q[50:], p[50:], append=True)
    assert _bytes(fn) == GOLD["dump"].tobytes()


def test_read_stream_header_then_body(tmp_path):
    # LoadFromStream reads int particle_number, double SimulationTime, double
    # Zeta, then the SaveToStream body (variables.cc:121-131)
    n = len(GOLD["q"])
    fn = tmp_path / "restart.bin"
    with open(fn, "wb") as f:
        f.write(struct.pack("<i", n) + struct.pack("<d", 12.5) + struct.pack("<d", -0.25))
        f.write(GOLD["stream"].tobytes())
    q4, p4, t, z = mio.read_stream(fn, capacity=n)
    assert (t, z) == (12.5, -0.25)
    np.testing.assert_array_equal(q4[:, :3], GOLD["q"])
    np.testing.assert_array_equal(p4[:, :3], GOLD["p"])
    assert not q4[:, 3].any() and not p4[:, 3].any()
    with pytest.raises(Exception):
        mio.read_stream(fn, capacity=n - 1)


@pytest.mark.gpu
def test_handle_writers_read_the_device_state(tmp_path):
    from mdacp_gb300.manager import MDManager
    from tests.helpers import liquid_like
    q, p, L = liquid_like(0.5, 8, seed=9)
    m = MDManager(L, capacity=len(q), cutoff=2.5, margin=0.5, dt=0.001)
    m.set_state(q, p)
    m.calculate(20)
    qs, ps = m.state()
    m.save_dump(tmp_path / "a.dump")
    mio.write_dump(tmp_path / "b.dump", qs, ps)
    assert _bytes(tmp_path / "a.dump") == _bytes(tmp_path / "b.dump")
    m.save_cdview(tmp_path / "a.cd")
    mio.write_cdview(tmp_path / "b.cd", qs, ps)
    assert _bytes(tmp_path / "a.cd") == _bytes(tmp_path / "b.cd")
    m.close()
