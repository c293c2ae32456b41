#!/usr/bin/env python3
"""Benchmark of the MDACP LJ hot path on GB300: atom-steps/s at 4M atoms, mixed vs FP64.

Workload (the large NVE configuration): 100^3 FCC unit cells = 4,000,000 atoms,
density 0.5 (L = 200), Maxwell velocities at T = 1 (seeded), rc = 2.5,
margin 0.5, dt = 0.001, NVE drift-kick-drift.  One benchmark step is one MD
step of the whole box: list rebuild when due, fused force/kick/drift kernel.
Inputs are synthetic (seeded lattice + velocities); they are larger than L2
(positions, momenta and the neighbour list total > 2 GB), so no flush is needed.

value     mixed-form atom-steps/s over K steps (pair force in f32, per-atom
          force sums in compensated f32, state and energy sums in f64), device
          time: the K steps replay the library's step graph with CUDA event
          nodes around every step kernel (mdg_calculate_profiled), max over
          ranks, summed over ranks.  `mixed_plain` (plain f32 force sums) and
          `fp64` blocks are measured the same way; each reports the list
          rebuilds inside its window, and when there were none, a
          rebuild-amortised figure (rebuild time x rebuild rate measured over
          the next 400 steps, added to the window's time per step).
e2e       the same through the public C ABI from host memory: pinned host state
          uploaded with mdg_set_state, K calls of mdg_calculate(1), mdg_observe
          every 100 steps (as Benchmark::Run observes), state read back with
          mdg_get_state; wall clock, the median of seven such windows.
roofline  the fused step kernel (mixed) over the same K steps: its mean launch
          time from the window's event nodes; achieved = DRAM bytes per launch
          (an ncu capture of the same kernel, per atom, scaled by the atoms and
          weighted by the window's ordinary / re-selecting launches) over that
          time; frac = achieved / the measured HBM copy bandwidth.  The pair
          model's algorithmic bytes (20 B per walked pair + 72 B per atom) are
          reported beside it as algorithmic_gbs / algorithmic_frac: the
          partner gathers they count are mostly served by L1/L2.
--impl reference  the reference's CPU implementation on the host cores: the
          reference binary built from its sources when present (oracle/_ref),
          else the oracle's C restatement, with all host threads.
--workload drift10k  the same box for 10,000 steps in each form with the
          energy drift per atom per tau.

Multi-GPU: independent replica boxes, one per rank (no collective on the data
path); scaling is weak.  `--gpus N` without torchrun's environment starts N
ranks itself under torch.distributed.run.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LJ atom-steps/s, 4M atoms: mixed vs FP64 on 1 GB300 @ rel force err<=1e-5"
UNIT = "atom-steps/s"
E2E_WINDOWS = 7
RC, MARGIN, DT, TEMP, DENSITY = 2.5, 0.5, 0.001, 1.0, 0.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="mdg", choices=["mdg", "reference"])
    ap.add_argument("--cells", type=int, default=100, help="FCC unit cells per side (100 -> 4M atoms)")
    ap.add_argument("--density", type=float, default=DENSITY,
                    help="number density of the NVE workload (the large configuration runs 0.5 and 0.8)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the CPU baseline sample")
    ap.add_argument("--cpu-threads", type=int, default=0, help="host threads of the CPU baseline (0: all cores)")
    ap.add_argument("--workload", default="nve4m",
                    choices=["nve4m", "drift10k", "langevin16m", "batch1024", "adjoint4k", "io4m", "init16m"],
                    help="nve4m: the headline (4M atoms NVE); drift10k: the same box 10,000 steps per form with "
                         "its energy drift; langevin16m: 160^3 FCC Langevin NVT; "
                         "batch1024: 1024 replica boxes; adjoint4k: 4000-atom trajectory gradient; "
                         "io4m: the reference's dump and stream files of the 4M-atom state; "
                         "init16m: the reference's exact-density initial state of the 16.4M-atom box, on the device")
    return ap.parse_args()


class Dist:
    """The ranks of the job (torchrun's environment; one process when unset).
    `n` is the rank count asked for with --gpus and must match."""

    def __init__(self, n):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        if n != self.world:
            raise SystemExit("bench.py: --gpus %d but WORLD_SIZE is %d" % (n, self.world))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        return self._reduce(v, "MAX")

    def sum(self, v):
        return self._reduce(v, "SUM")

    def _reduce(self, v, op):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=getattr(self.pg.ReduceOp, op))
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during a timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload(cells, seed, density=DENSITY):
    from mdacp_gb300 import lattice
    q, L = lattice.fcc_cube(cells, density)
    p = lattice.maxwell(len(q), TEMP, seed)
    return q, p, L


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_atom(form):
    """DRAM bytes per atom of one step-kernel launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)[form]["dram_bytes_per_atom"])
    except (OSError, KeyError, ValueError):
        return None


def cpu_sample(q, p, L, budget_s, threads, prefer_reference=True):
    """Times the reference CPU path on the same workload; returns
    (atom-steps/s, kind, description, threads used)."""
    n = len(q)
    from oracle import refrun
    if prefer_reference and refrun.available(RC, bench=True):
        # the reference itself (built from its sources on this host, -O3
        # -fopenmp), one MDUnit per OpenMP thread on the grid the reference
        # derives from the thread count, timed like Benchmark::Run (list build
        # outside, observation every ObserveLoop=100 steps inside); a 2-step
        # probe sizes the run
        def mups(steps):
            out = refrun.run("bench", q, p, L, rc=RC, margin=MARGIN, dt=DT, steps=steps, observe_every=100,
                             threads=threads, timeout=max(600, int(budget_s * 20)), bench=True)
            line = [x for x in out["stdout"].splitlines() if "[MUPS]" in x][-1]
            return float(line.split("[SEC]")[1].split("[MUPS]")[0])
        probe = mups(2)
        steps = max(2, min(200, int(budget_s * probe * 1e6 / n)))
        v = mups(steps) * 1e6
        return v, "reference", ("MDACP reference binary built here from its sources (g++ -O3 -fopenmp), %d steps "
                                "of the full %d-atom box, %d OpenMP threads = %d MDUnits" % (
                                    steps, n, threads, threads)), threads
    from oracle import port
    s = port.System(q, p, L, rc=RC, margin=MARGIN, dt=DT, threads=threads)
    s.make_pairlist()
    t0 = time.perf_counter()
    s.calculate(1)
    one = time.perf_counter() - t0
    steps = max(2, min(50, int(budget_s / max(one, 1e-6)) - 1))
    t0 = time.perf_counter()
    s.calculate(steps)
    dt = time.perf_counter() - t0
    s.close()
    return n * steps / dt, "port", "oracle C restatement (half list, Newton-3), %d steps of the full %d-atom box, %d threads" % (
        steps, n, threads), threads


def run_reference(args):
    d = Dist(args.gpus)
    ranks = d.sum(1)  # every rank joined the job
    if d.rank != 0:
        d.close()
        return
    q, p, L = workload(args.cells, 1, args.density)
    threads = args.cpu_threads or os.cpu_count() or 1
    value, kind, descr, cores = cpu_sample(q, p, L, args.cpu_seconds, threads)
    n = len(q)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": d.world,
            "ranks_joined": int(ranks), "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_block(args, n, d.world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": descr},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    d.close()


def config_block(args, n, world):
    return {"workload": "LJ NVE %d atoms (%d^3 FCC), rho %.1f, rc %.1f, margin %.1f, dt %g, T %.1f" % (
        n, args.cells, args.density, RC, MARGIN, DT, TEMP), "atoms": n, "density": args.density, "cutoff": RC,
        "margin": MARGIN, "dt": DT,
        "precision": "mixed: compensated f32 force sums (value); mixed_plain and fp64 blocks beside it",
        "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas x%d" % world}


DTYPE = {"mixed": "f32 pair distance/force, compensated (Kahan) f32 per-atom force sums, f64 state/integration/"
                  "energy-virial sums",
         "mixed_plain": "f32 pair distance/force, plain f32 per-atom force sums, f64 state/integration/energy-virial "
                        "sums",
         "fp64": "f64"}


def timed_window(m, d, K):
    """K steps of handle m replayed from the step graph with event nodes around
    every step kernel (mdg_calculate_profiled's path); returns the window's
    device ms (max over ranks), the step kernels' summed ms and the counters
    that moved inside the window."""
    s0 = m.stats()
    d.barrier()
    ph = m.calculate_phases(K)
    d.barrier()
    s1 = m.stats()
    return {"ms": d.max(ph["all"]), "kernel_ms": ph["force"], "rebuild_ms": ph["pair"],
            "rebuilds": s1["rebuilds"] - s0["rebuilds"], "prunes": s1["prunes"] - s0["prunes"],
            "launches": s1["kernel_launches"] - s0["kernel_launches"], "stats": s1}


def run_mine(args):
    import numpy as np
    from mdacp_gb300.manager import MDManager
    d = Dist(args.gpus)
    q, p, L = workload(args.cells, 1 + d.rank, args.density)
    n = len(q)
    K, W = args.steps, max(3, args.warmup)
    res = {}
    clk = Clocks(d.local)
    clocks = None
    for prec in ("mixed", "mixed_plain", "fp64"):
        m = MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, dt=DT, precision=prec, device=d.local)
        m.set_state(q, p)
        m.make_pairlist()
        m.calculate(W)
        e0 = m.observe()[2]
        if prec == "mixed":
            clk.start()
        w = timed_window(m, d, K)
        if prec == "mixed":
            clocks = clk.stop()
        e1 = m.observe()[2]
        w.update({"drift": (e1 - e0) / (K * DT), "handle": m})
        if w["rebuilds"] == 0:
            # no list rebuild fell inside the window: the rebuild cost per step
            # is measured over a longer continuation of the same run (rebuild
            # time x rebuild rate) and added to the window's time per step
            R = 400
            a = timed_window(m, d, R)
            w["amortised"] = {"steps": R, "rebuilds": a["rebuilds"], "rebuild_ms_per_step": a["rebuild_ms"] / R,
                              "ms_per_step": w["ms"] / K + a["rebuild_ms"] / R}
        res[prec] = w
    # force error of both mixed forms against FP64 at the same (warmed-up) state
    md = res["fp64"]["handle"]
    qs, ps = md.state()
    f_fp64 = md.forces()
    for prec in ("mixed", "mixed_plain"):
        mf = res[prec]["handle"]
        mf.set_state(qs, ps)
        f = mf.forces()
        rel = np.linalg.norm(f - f_fp64, axis=1) / np.maximum(np.linalg.norm(f_fp64, axis=1), 1e-300)
        res[prec]["rms_err"] = float(np.sqrt(np.mean(rel ** 2)))
    for prec in res:
        res[prec]["handle"].close()
    mixed = res["mixed"]
    # roofline of the fused step kernel (mixed form), from the window itself:
    # the mean step-kernel time of its K steps against (a) the DRAM bytes an
    # ncu capture of the same kernel measured per atom and (b) the algorithmic
    # bytes of the pair model (20 B per walked pair + 72 B per atom), most of
    # whose partner gathers are served by L1/L2
    st = mixed["stats"]
    kernel_ms = mixed["kernel_ms"] / K
    ppa, opa = st["inner_pairs"] / n, st["listed_pairs"] / n
    n_sel = min(max(mixed["prunes"], 0), K)
    alg_bytes = n * ((K - n_sel) * (ppa * 20.0 + 72.0) + n_sel * (opa * 20.0 + ppa * 4.0 + 72.0)) / K
    peak, peak_kind = peaks()
    t_ord, t_sel = ncu_traffic_per_atom("mixed"), ncu_traffic_per_atom("mixed_reselect")
    tpa = None
    if t_ord and t_sel and abs(args.density - DENSITY) < 1e-12:  # the captures are of density 0.5
        tpa = ((K - n_sel) * t_ord + n_sel * t_sel) / K
    dram_gbs = tpa * n / (kernel_ms * 1e-3) / 1e9 if tpa else None
    alg_gbs = alg_bytes / (kernel_ms * 1e-3) / 1e9
    roof = {"kernel": "k_step<NVE,mixed>", "bound": "hbm", "achieved": dram_gbs, "peak": peak, "unit": "GB/s",
            "frac": dram_gbs / peak if dram_gbs else None,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": tpa * n if tpa else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per atom of one launch "
                              "(profiles/step_kernel_traffic.json), x atoms, weighted by the window's "
                              "ordinary/re-selecting launches",
            "launch_ms": kernel_ms, "launches_timed": K, "window_ms_per_step": mixed["ms"] / K,
            "algorithmic_bytes": alg_bytes, "algorithmic_gbs": alg_gbs, "algorithmic_frac": alg_gbs / peak,
            "algorithmic_note": "pair model (20 B per walked pair + 72 B per atom); counts partner gathers "
                                "served by L1/L2, so it can exceed the DRAM figure",
            "pairs_per_atom": ppa, "listed_pairs_per_atom": opa, "reselecting_launches": n_sel}
    # end to end through the C ABI with host buffers
    import torch
    qh = torch.zeros((n, 4), dtype=torch.float64).pin_memory().numpy()
    ph = torch.zeros((n, 4), dtype=torch.float64).pin_memory().numpy()
    qh[:, :3] = q
    ph[:, :3] = p
    qo = torch.zeros((n, 4), dtype=torch.float64).pin_memory().numpy()
    po = torch.zeros((n, 4), dtype=torch.float64).pin_memory().numpy()
    me = MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, dt=DT, precision="mixed", device=d.local)
    me.set_state(qh, ph)
    me.calculate(W)
    me.synchronize()  # the warm-up steps finish before the clock starts
    # E2E_WINDOWS windows, each from the upload to the read-back; the median
    # is reported (one window of the short default run lasts ~20 ms, so a
    # single host-side stall would otherwise decide the figure)
    windows, window_rebuilds = [], []
    for _ in range(E2E_WINDOWS):
        d.barrier()
        t0 = time.perf_counter()
        me.set_state(qh, ph)
        nobs = 0
        for k in range(K):
            me.calculate(1)
            if k % 100 == 0:
                me.observe_raw()
                nobs += 1
        me.state(qo, po)
        windows.append(d.max(time.perf_counter() - t0))
        window_rebuilds.append(me.stats()["rebuilds"])  # counted from the upload (mdg_set_state resets it)
    t_e2e = float(np.median(windows))
    e2e_rebuilds = window_rebuilds
    me.close()
    e2e_value = d.world * n * K / t_e2e
    cpu = None
    if d.rank == 0 and d.world == 1:
        v, kind, descr, cores = cpu_sample(q, p, L, args.cpu_seconds, args.cpu_threads or os.cpu_count() or 1)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": descr}
    value = d.world * n * K / (mixed["ms"] * 1e-3)

    def form(r):
        out = {"value": d.world * n * K / (r["ms"] * 1e-3), "unit": UNIT, "ms_per_step": r["ms"] / K,
               "step_kernel_ms": r["kernel_ms"] / K, "rebuilds_in_window": r["rebuilds"],
               "reselections_in_window": r["prunes"],
               "energy_drift_per_atom_per_tau_window": r["drift"]}
        if "amortised" in r:
            a = r["amortised"]
            out["rebuild_amortised"] = dict(a, value=d.world * n / (a["ms_per_step"] * 1e-3))
        if "rms_err" in r:
            out["rms_rel_force_err_vs_fp64"] = r["rms_err"]
        return out

    if d.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": d.world, "steps": K, "warmup": W,
                "ms_per_step": mixed["ms"] / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": DTYPE["mixed"], "data": "synthetic",
                "config": config_block(args, n, d.world),
                "rebuilds_in_window": mixed["rebuilds"],
                "mixed": form(mixed), "mixed_plain": form(res["mixed_plain"]), "fp64": form(res["fp64"]),
                "mixed_over_fp64": res["fp64"]["ms"] / mixed["ms"],
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * n * 32 / K,
                        "d2h_bytes_per_step": (2 * n * 32 + 24 * nobs) / K, "rebuilds_per_window": e2e_rebuilds,
                        "windows_ms": [round(1e3 * t, 3) for t in windows], "reported": "median window"},
                "gpu_launches": mixed["launches"],
                "roofline": roof, "cpu_baseline": cpu, "clocks": clocks}
        if "amortised" in mixed:
            line["value_rebuild_amortised"] = line["mixed"]["rebuild_amortised"]["value"]
            line["mixed_over_fp64_rebuild_amortised"] = (res["fp64"]["amortised"]["ms_per_step"] /
                                                         mixed["amortised"]["ms_per_step"]
                                                         if "amortised" in res["fp64"] else None)
        print(json.dumps(line), flush=True)
    d.close()


def base_line(metric, value, n_gpus, K, W, ms, config, dtype):
    return {"metric": metric, "value": value, "unit": UNIT, "n_gpus": n_gpus, "steps": K, "warmup": W,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic", "config": config}


def run_drift10k(args):
    """The large NVE configuration run for 10,000 steps in each form (FP64,
    compensated mixed, plain mixed) from the same state: total energy per atom
    observed every 100 steps; drift = least-squares slope of E/N against time
    (per atom per tau) and the end-to-start difference over the run time."""
    import numpy as np
    from mdacp_gb300.manager import MDManager
    q, p, L = workload(args.cells, 1, args.density)
    n = len(q)
    K = args.steps if args.steps != 1000 else 10000
    every = 100
    out = {}
    for prec in ("fp64", "mixed", "mixed_plain"):
        m = MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, dt=DT, precision=prec)
        m.set_state(q, p)
        m.make_pairlist()
        t, E = [0.0], [m.observe()[2]]
        dev_ms = 0.0
        for k in range(K // every):
            m.calculate(every)
            dev_ms += m.stats()["elapsed_ms"]
            t.append((k + 1) * every * DT)
            E.append(m.observe()[2])
        st = m.stats()
        m.close()
        t, E = np.array(t), np.array(E)
        slope = float(np.polyfit(t, E, 1)[0])
        out[prec] = {"energy_drift_per_atom_per_tau": slope,
                     "energy_change_per_atom_per_tau": float((E[-1] - E[0]) / (t[-1] - t[0])),
                     "E_start": float(E[0]), "E_end": float(E[-1]), "E_rms_fluct": float(np.std(E - np.polyval(np.polyfit(t, E, 1), t))),
                     "value": n * K / (dev_ms * 1e-3), "ms_per_step": dev_ms / K, "rebuilds": st["rebuilds"],
                     "reselections": st["prunes"]}
    cfg = {"workload": "LJ NVE %d atoms (%d^3 FCC), rho %.1f, rc %.1f, margin %.1f, dt %g, T %.1f, %d steps, "
                       "E observed every %d" % (n, args.cells, args.density, RC, MARGIN, DT, TEMP, K, every),
           "atoms": n, "density": args.density, "l2": "inputs larger than L2 (no flush)"}
    line = base_line("LJ atom-steps/s over a 10,000-step NVE run with energy drift, 4M atoms", out["mixed"]["value"],
                     1, K, 0, out["mixed"]["ms_per_step"], cfg, DTYPE["mixed"])
    line.update(out)
    line["mixed_over_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    print(json.dumps(line), flush=True)


def run_langevin16m(args):
    """Langevin NVT, 160^3 FCC = 16,384,000 atoms, density 0.5, T 0.9, gamma 1, dt 0.005."""
    from mdacp_gb300.manager import MDManager
    cells = 160 if args.cells == 100 else args.cells
    from mdacp_gb300 import lattice
    q, L = lattice.fcc_cube(cells, DENSITY)
    p = lattice.maxwell(len(q), 1.0, 1)
    n = len(q)
    K, W = args.steps if args.steps != 1000 else 200, max(3, args.warmup)
    res = {}
    clk = Clocks(0)
    clocks = None
    for prec in ("mixed", "fp64"):
        m = MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, dt=0.005, precision=prec, thermostat="langevin",
                      temperature=0.9, gamma=1.0, seed=12345)
        m.set_state(q, p)
        m.make_pairlist()
        m.calculate(W)
        if prec == "mixed":
            clk.start()
        m.calculate(K)
        st = m.stats()
        if prec == "mixed":
            clocks = clk.stop()
        res[prec] = {"ms": st["elapsed_ms"], "rebuilds": st["rebuilds"], "prunes": st["prunes"],
                     "T_end": float(m.observe()[0]), "pairs_per_atom": st["listed_pairs"] / n}
        m.close()
    cfg = {"workload": "Langevin NVT %d atoms (%d^3 FCC), rho 0.5, T 0.9, gamma 1.0, dt 0.005, rc 2.5, margin 0.5"
           % (n, cells), "atoms": n, "l2": "inputs larger than L2 (no flush)"}
    v = n * K / (res["mixed"]["ms"] * 1e-3)
    line = base_line("LJ atom-steps/s, 16.4M atoms Langevin NVT: mixed vs FP64 on 1 GB300", v, 1, K, W,
                     res["mixed"]["ms"] / K, cfg, DTYPE["mixed"])
    line.update({"fp64": {"value": n * K / (res["fp64"]["ms"] * 1e-3), "ms_per_step": res["fp64"]["ms"] / K,
                          "rebuilds": res["fp64"]["rebuilds"], "T_end": res["fp64"]["T_end"]},
                 "mixed": res["mixed"], "clocks": clocks})
    print(json.dumps(line), flush=True)


def run_batch1024(args):
    """1024 replica boxes: N ~ U[500, 8000], density ~ U[0.3, 0.9], T ~ U[0.7, 1.5], rc 2.5, margin 0.4, dt 0.002."""
    from mdacp_gb300.batch import Batch, make_replicas
    boxes = make_replicas(1024, seed=1)
    n = sum(len(b[0]) for b in boxes)
    K, W = args.steps if args.steps != 1000 else 500, max(3, args.warmup)
    res = {}
    for prec in ("mixed", "fp64"):
        b = Batch(boxes, cutoff=2.5, margin=0.4, dt=0.002, precision=prec)
        shape = b.tune(trial_steps=10)
        b.calculate(W)
        b.calculate(K)
        st = b.stats()
        res[prec] = {"ms": st["elapsed_ms"], "shape": {"threads": shape[0], "lanes_per_particle": shape[1],
                                                        "ctas_per_sm": st["ctas_per_sm"], "inner_list": st["inner_list"],
                                                        "flat": st["flat"], "prune_buffer": st["prune_buffer"]},
                     "rebuilds": st["rebuilds"], "kernels_per_step": 7 if st["flat"] else 6}
        b.close()
    cfg = {"workload": "1024 replica boxes, %d atoms total, N~U[500,8000], rho~U[0.3,0.9], T~U[0.7,1.5], "
                       "rc 2.5, margin 0.4, dt 0.002" % n, "atoms": n, "boxes": 1024}
    v = n * K / (res["mixed"]["ms"] * 1e-3)
    line = base_line("LJ atom-steps/s, 1024 batched replicas: mixed vs FP64 on 1 GB300", v, 1, K, W,
                     res["mixed"]["ms"] / K, cfg, DTYPE["mixed"])
    line.update({"fp64": {"value": n * K / (res["fp64"]["ms"] * 1e-3), "ms_per_step": res["fp64"]["ms"] / K,
                          "shape": res["fp64"]["shape"]}, "mixed": res["mixed"]})
    print(json.dumps(line), flush=True)


def run_adjoint4k(args):
    """Gradient of mean PE and of mean pressure, 4000 atoms at density 0.8, 200 steps, checkpoint every 20."""
    from mdacp_gb300 import lattice
    from mdacp_gb300.adjoint import Adjoint
    q, L = lattice.fcc_cube(10, 0.8)
    p = lattice.maxwell(len(q), 1.0, 1)
    n = len(q)
    out = {}
    for obj in ("pe", "pressure"):
        a = Adjoint(L, n, steps=200, checkpoint_every=20, dt=0.002, margin=0.5, objective=obj)
        a.forward(q, p)
        a.backward()
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            a.forward(q, p)
            a.backward()
        dt = (time.perf_counter() - t0) / reps
        out[obj] = {"ms_per_gradient": dt * 1e3}
        a.close()
    # one gradient = 200 forward steps + 200 recomputed steps + 200 reverse steps
    v = n * 200 / (out["pe"]["ms_per_gradient"] * 1e-3)
    cfg = {"workload": "adjoint, 4000 atoms (10^3 FCC), rho 0.8, T 1, dt 0.002, 200 steps, checkpoint every 20",
           "atoms": n}
    line = base_line("LJ adjoint: trajectory atom-steps/s per gradient (forward+backward), 4000 atoms", v, 1, 200,
                     1, out["pe"]["ms_per_gradient"] / 200, cfg, "f64")
    line.update({"gradients": out})
    print(json.dumps(line), flush=True)


def run_io4m(args):
    """Writes the 4M-atom state in the reference's dump (SaveAsDumpFile) and
    stream (SaveToStream) formats: from the device handle (state read back,
    then written) and from host arrays; wall clock, file in a temporary
    directory, median of a few repetitions."""
    from mdacp_gb300 import io as mio
    from mdacp_gb300.manager import MDManager
    q, p, L = workload(args.cells, 1, args.density)
    n = len(q)
    m = MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, dt=DT, precision="mixed")
    m.set_state(q, p)
    m.calculate(10)
    qs, ps = m.state()
    res = {}
    with tempfile.TemporaryDirectory(prefix="mdg_io_") as d:
        fn = os.path.join(d, "conf.dump")
        for name, fun, nbytes in (("save_dump (device state)", lambda: m.save_dump(fn), 48 * n),
                                  ("write_dump (host arrays)", lambda: mio.write_dump(fn, qs, ps), 48 * n),
                                  ("write_stream (host arrays)", lambda: mio.write_stream(fn, qs, ps), 64 * n)):
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                fun()
                ts.append(time.perf_counter() - t0)
            ts.sort()
            res[name] = {"ms": ts[2] * 1e3, "GB_per_s": nbytes / ts[2] / 1e9, "bytes": nbytes}
    m.close()
    v = n / (res["save_dump (device state)"]["ms"] * 1e-3)
    cfg = {"workload": "dump and stream files of the %d-atom NVE state" % n, "atoms": n}
    line = base_line("atoms/s written in the reference's dump format from the device state", v, 1, 5, 0,
                     res["save_dump (device state)"]["ms"], cfg, "f64")
    line["unit"] = "atoms/s"
    line.update({"files": res})
    print(json.dumps(line), flush=True)


def run_init16m(args):
    """ExtractConfigurationMaker + SetInitialVelocity (the reference Benchmark
    project's initial state) for the 160^3-cell box at density 0.5 (L = 320,
    16,384,000 atoms) on the device, against the reference's algorithm on the
    host cores (oracle/makers.cc: the same generator and linear search for
    distinct deletions) for the 4M-atom box (L = 200)."""
    from mdacp_gb300.manager import MDManager
    L = 320.0
    n_expect = int(L ** 3 * DENSITY)
    m = MDManager(L, capacity=n_expect, cutoff=RC, margin=MARGIN, dt=DT, precision="mixed")
    m.make_state("extract", DENSITY, v0=1.0)  # warm-up (allocations, module load)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        m.make_state("extract", DENSITY, v0=1.0)
        n = m.stats()["particles"]
        ts.append(time.perf_counter() - t0)
    m.close()
    t = sorted(ts)[1]
    from oracle import port  # the reference's algorithm, timed as the CPU baseline
    Lc = 200.0
    t0 = time.perf_counter()
    qc = port.make_configuration("extract", Lc, DENSITY)
    port.initial_velocity(len(qc), 1.0, 0)
    tc = time.perf_counter() - t0
    cfg = {"workload": "ExtractConfigurationMaker + SetInitialVelocity, L %.0f, density %.1f, %d atoms" % (
        L, DENSITY, n), "atoms": n}
    line = base_line("atoms/s of the reference's initial state made on the device", n / t, 1, 3, 1, t * 1e3, cfg,
                     "f64")
    line["unit"] = "atoms/s"
    line["cpu_baseline"] = {"value": len(qc) / tc, "unit": "atoms/s", "cores": 1, "kind": "port",
                            "sample": "oracle/makers.cc (the reference's algorithm: std::mt19937, linear search for "
                                      "distinct deletions) for L %.0f, %d atoms, %.2f s" % (Lc, len(qc), tc)}
    print(json.dumps(line), flush=True)


def launch_ranks(n):
    """Runs this command as n ranks under torch.distributed.run (one process
    per GPU, rendezvous on 127.0.0.1) and returns its exit status; rank 0
    prints the JSON line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus))
    if args.impl == "mdg" and args.workload != "nve4m":
        if int(os.environ.get("RANK", "0")) != 0:  # single-GPU workloads: rank 0 runs them
            return
        {"langevin16m": run_langevin16m, "batch1024": run_batch1024, "adjoint4k": run_adjoint4k,
         "io4m": run_io4m, "init16m": run_init16m, "drift10k": run_drift10k}[args.workload](args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_mine(args)


if __name__ == "__main__":
    main()
