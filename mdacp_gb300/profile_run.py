"""Runs one LJ workload through the C ABI for profiling (e.g. under ncu).

    python -m mdacp_gb300.profile_run --cells 63 --precision mixed --steps 8 [--no-graphs | --profiled]
    python -m mdacp_gb300.profile_run --boxes 256 --precision mixed --steps 20 [--shape 512,1,4[,inner]]
    python -m mdacp_gb300.profile_run --adjoint

cells^3 FCC unit cells at density 0.5 (cells=100 -> 4,000,000 atoms, cells=63 ->
1,000,188 atoms), Maxwell velocities at T=1, rc 2.5, margin 0.5, dt 0.001:
one list build, then `steps` NVE steps.  --profiled runs the steps as plain
launches of both step-kernel variants (ordinary, re-selecting; each returns at
once when the step is not its kind) with CUDA events around them, the form a
kernel profiler sees one launch at a time; the mean step-kernel time is printed.
--adjoint runs one gradient of the 200-step mean potential energy (4,000
atoms, density 0.8, dt 0.002, checkpoint every 20), forward and backward.
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=63)
    ap.add_argument("--density", type=float, default=0.5)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_plain", "fp64"])
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--no-graphs", action="store_true")
    ap.add_argument("--profiled", action="store_true")
    ap.add_argument("--boxes", type=int, default=0,
                    help="run the batched-replica workload instead: this many boxes (N ~ U[500, 8000], "
                         "density ~ U[0.3, 0.9], T ~ U[0.7, 1.5], margin 0.4, dt 0.002), autotuned shape")
    ap.add_argument("--shape", default="",
                    help="threads,lanes,ctas_per_sm[,inner 0|1[,flat 0|1]] for --boxes instead of the autotuner")
    ap.add_argument("--adjoint", action="store_true", help="one adjoint gradient instead (4,000 atoms)")
    ap.add_argument("--rebuild-policy", default="halfmargin", choices=["halfmargin", "reference"],
                    help="single box: the list rebuild rule")
    a = ap.parse_args()
    if a.adjoint:
        import time
        from mdacp_gb300 import lattice
        from mdacp_gb300.adjoint import Adjoint
        q, L = lattice.fcc_cube(10, 0.8)
        p = lattice.maxwell(len(q), 1.0, 1)
        ad = Adjoint(L, len(q), steps=200, checkpoint_every=20, dt=0.002, margin=0.5, objective="pe")
        t0 = time.perf_counter()
        ad.forward(q, p)
        t1 = time.perf_counter()
        ad.backward()
        t2 = time.perf_counter()
        print("adjoint atoms %d forward %.2f ms backward %.2f ms" % (len(q), 1e3 * (t1 - t0), 1e3 * (t2 - t1)))
        return
    if a.boxes:
        from mdacp_gb300.batch import Batch, make_replicas
        boxes = make_replicas(a.boxes, seed=1)
        b = Batch(boxes, cutoff=2.5, margin=0.4, dt=0.002, precision=a.precision)
        if a.shape:
            shape = tuple(int(x) for x in a.shape.split(","))
            b.set_shape(*shape[:3])
            if len(shape) > 3:
                b.set_inner(shape[3] != 0)
            if len(shape) > 4:
                b.set_flat(shape[4] != 0)
        else:
            shape = b.tune(trial_steps=10)
        b.calculate(a.steps)
        st = b.stats()
        print("boxes %d atoms %d steps %d ms/step %.4f shape %s rebuilds %d" % (
            a.boxes, sum(len(x[0]) for x in boxes), a.steps, st["elapsed_ms"] / max(a.steps, 1), shape,
            st["rebuilds"]))
        return
    from mdacp_gb300 import lattice
    from mdacp_gb300.manager import MDManager
    q, L = lattice.fcc_cube(a.cells, a.density)
    p = lattice.maxwell(len(q), 1.0, 1)
    m = MDManager(L, capacity=len(q), cutoff=2.5, margin=0.5, dt=0.001, precision=a.precision,
                  use_graphs=not a.no_graphs, rebuild_policy=a.rebuild_policy)
    m.set_state(q, p)
    m.make_pairlist()
    if a.profiled:
        kms = m.calculate_profiled(a.steps) / max(a.steps, 1)
        st = m.stats()
        print("atoms %d steps %d step-kernel ms %.4f pairs/atom %.2f inner %.2f rebuilds %d prunes %d" % (
            len(q), a.steps, kms, st["listed_pairs"] / len(q), st["inner_pairs"] / len(q), st["rebuilds"],
            st["prunes"]))
        return
    m.calculate(a.steps)
    st = m.stats()
    print("atoms %d steps %d ms/step %.4f pairs/atom %.2f rebuilds %d" % (
        len(q), a.steps, st["elapsed_ms"] / max(a.steps, 1), st["listed_pairs"] / len(q), st["rebuilds"]))


if __name__ == "__main__":
    main()
