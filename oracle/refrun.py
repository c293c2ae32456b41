"""Runs the MDACP reference itself (built by build_ref.sh) on an injected state.

Test infrastructure only.  Drives the Mode=Oracle project of ref_harness.cc
through a generated .cfg and reads back the binary dumps.
"""
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


SRC_DIR = os.path.join(REF_DIR, "src")


def binary(rc=2.5, bench=False):
    """The parity binary for cut-off rc (no fused multiply-adds), or with
    bench=True the timed-baseline build (the compiler's default contraction)."""
    return os.path.join(REF_DIR, ("mdacp_bench_rc%.1f" if bench else "mdacp_rc%.1f") % rc)


def available(rc=2.5, bench=False):
    return os.path.exists(binary(rc, bench))


def sources_available():
    """The reference sources: MDG_REFERENCE_DIR, or the copy build_ref.sh
    staged under oracle/_ref/src (which travels with a copy of this tree)."""
    ref = os.environ.get("MDG_REFERENCE_DIR")
    if ref and os.path.exists(os.path.join(ref, "mdconfig.h")):
        return True
    return os.path.exists(os.path.join(SRC_DIR, "mdconfig.h"))


def build():
    """Builds the reference binaries when the reference sources are present."""
    if not sources_available():
        return False
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])
    return True


def write_input(path, q, p):
    q = np.asarray(q, dtype=np.float64)[:, :3]
    p = np.asarray(p, dtype=np.float64)[:, :3]
    with open(path, "wb") as f:
        f.write(struct.pack("<q", len(q)))
        f.write(np.ascontiguousarray(np.hstack([q, p]), dtype="<f8").tobytes())


def run(task, q, p, L, rc=2.5, margin=0.5, dt=0.001, steps=100, observe_every=10, threads=1,
        extra=None, timeout=3600, bench=False):
    """Runs one Oracle task; returns a dict of numpy arrays (and 'stdout').
    threads = OpenMP threads = MDUnits (the reference runs one unit per
    thread, its local grid from MPI_Dims_create, parainfo.cc:29-35)."""
    L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
    with tempfile.TemporaryDirectory(prefix="mdacp_ref_") as d:
        write_input(os.path.join(d, "in.bin"), q, p)
        cfg = ["Mode=Oracle", "OracleTask=%s" % task, "OracleInput=in.bin", "OracleOutput=o",
               "OracleBufferLength=%r" % float(margin), "TimeStep=%r" % float(dt),
               "SystemSizeX=%r" % float(L[0]), "SystemSizeY=%r" % float(L[1]),
               "SystemSizeZ=%r" % float(L[2]),
               "OracleSteps=%d" % steps, "ObserveLoop=%d" % observe_every]
        for k, v in (extra or {}).items():
            cfg.append("%s=%s" % (k, v))
        with open(os.path.join(d, "o.cfg"), "w") as f:
            f.write("\n".join(cfg) + "\n")
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        r = subprocess.run([binary(rc, bench), "o.cfg"], cwd=d, env=env, capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference failed: %s\n%s" % (r.stdout[-2000:], r.stderr[-2000:]))
        out = {"stdout": r.stdout}
        fn = os.path.join(d, "o_pairs.bin")
        if os.path.exists(fn):
            out["pairs"] = np.fromfile(fn, dtype="<i4").reshape(-1, 3)
        fn = os.path.join(d, "o_force.bin")
        if os.path.exists(fn):
            rec = np.fromfile(fn, dtype="<f8").reshape(-1, 7)
            f = np.zeros((len(rec), 3))
            f[rec[:, 0].astype(np.int64)] = rec[:, 4:7]
            out["force"] = f
        fn = os.path.join(d, "o_obs.bin")
        if os.path.exists(fn):
            out["obs"] = np.fromfile(fn, dtype="<f8")
        fn = os.path.join(d, "o_trace.bin")
        if os.path.exists(fn):
            out["trace"] = np.fromfile(fn, dtype="<f8").reshape(-1, 7)
        for key, fn in (("dump", "o_dump.bin"), ("cdview", "o_cdview.cd"), ("configuration", "conf000.cnf"),
                        ("stream", "o_stream.bin")):
            if os.path.exists(os.path.join(d, fn)):
                with open(os.path.join(d, fn), "rb") as f:
                    out[key] = f.read()
        fn = os.path.join(d, "o_made.bin")
        if os.path.exists(fn):
            rec = np.fromfile(fn, dtype="<f8").reshape(-1, 6)
            out["q"], out["p"] = rec[:, :3].copy(), rec[:, 3:].copy()
        fn = os.path.join(d, "o_state.bin")
        if os.path.exists(fn):
            rec = np.fromfile(fn, dtype="<f8").reshape(-1, 7)
            ids = rec[:, 0].astype(np.int64)
            qs = np.zeros((len(rec), 3)); ps = np.zeros((len(rec), 3))
            qs[ids] = rec[:, 1:4]; ps[ids] = rec[:, 4:7]
            out["q"], out["p"] = qs, ps
        return out
