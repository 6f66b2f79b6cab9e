"""ATM evaluation throughput on GB300: 22 replicas of a 23,558-atom PME box per
launch (difference path) next to the plain single-replica drop-in (two full
inner evaluations, as the reference does).

One "step" = one evaluation of every replica of the batch (forces, energies,
perturbation energies and the replicas x states energy matrix).
value = replica evaluations per second summed over the batch (22 x launches/s),
with positions already in HBM; e2e = the same through the C ABI with host
buffers (positions H2D and forces/results D2H inside the timed region).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "openmm-atmmetaforce-plugin_gb300"))

METRIC = "ATM evals/sec/replica at 23.5k-atom PME: batched vs plain on one GB300 at fixed error"
F_PAIR = 55.0  # FP32 flops per pair (accounting constant)
L2_BYTES = 129 * 1024 * 1024
# DRAM bytes (read + write) of one k_tiles launch on this workload, from a
# one-launch ncu --set full capture of the pair-tile kernel at commit 55d5dbd
# (92.50 MB read + 6.94 MB write; profiles/k_tiles_abfe-pme-23558x22.md)
TILES_TRAFFIC_BYTES = 99.43e6
TILES_CAPTURE = "55d5dbd"
# warp instructions of one k_tiles launch on this workload (same capture): the
# kernel is bound by instruction issue, so its issue rate is the second roofline
# reported
TILES_WARP_INSTR = 346.5e6


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--replicas", type=int, default=22)
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-md", action="store_true", help="skip the MD step-rate measurements")
    p.add_argument("--md-steps", type=int, default=10000,
                   help="MD steps of the single 23,558-atom replica (22-replica runs take 1/50, RBFE 1/100)")
    p.add_argument("--tune-cache", action="store_true",
                   help="reuse a stored autotuning choice for this GPU and workload (profiling runs)")
    p.add_argument("--ncu-case", type=int, default=0, metavar="N",
                   help="profiling case: build the batch, run N evaluations (no tuning, no timing) and exit")
    return p.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("ATM_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def max_over_ranks(x, pg, device=None):
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:  # sampling has started before the timed region
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def count_pairs(case):
    """Non-excluded pairs within the cutoff at state 1, and the ligand pairs
    (moving x non-moving) within the cutoff at both geometries."""
    from scipy.spatial import cKDTree

    L = case.spec.box
    pos = np.mod(case.pos, L)
    tree = cKDTree(pos, boxsize=L)
    rc = case.spec.cutoff
    n_all = (tree.count_neighbors(tree, rc) - len(pos)) // 2
    ei, ej = case.spec.exc_i, case.spec.exc_j
    d = case.pos[ej] - case.pos[ei]
    d -= L * np.round(d / L)
    n_exc = int((np.sqrt((d * d).sum(1)) < rc).sum())
    moving = np.any(case.displ != 0, axis=1)
    lig = np.where(moving)[0]
    env = np.where(~moving)[0]
    te = cKDTree(pos[env], boxsize=L)
    n_lig = 0
    for g in (0, 1):
        p = np.mod(case.pos[lig] + (case.displ[lig] if g else 0.0), L)
        n_lig += int(sum(len(x) for x in te.query_ball_point(p, rc)))
    return n_all - n_exc, n_lig


def cpu_baseline(cases, threads, warm=True):
    """The FP64 oracle timed on the host cores: one full ATM evaluation (two inner
    evaluations + merge) of each case.  Returns (evals/s, the oracle's results)."""
    import oracle as O

    O.set_threads(threads)
    if warm:
        O.atm_eval(cases[0].spec, cases[0].pos, cases[0].displ, cases[0].params)
    t0 = time.perf_counter()
    refs = [O.atm_eval(c.spec, c.pos, c.displ, c.params) for c in cases]
    dt = (time.perf_counter() - t0) / len(cases)
    O.set_threads(1)
    return 1.0 / dt, refs


def force_rms_rel(F, G):
    return float(np.sqrt(((F - G) ** 2).sum() / (G ** 2).sum()))


def reference_arm(args, rank, world, pg):
    """The reference's CPU path for this workload: its Reference-platform math,
    restated in the FP64 oracle (the reference itself needs OpenMM, absent here),
    on all host cores; each step evaluates one 23,558-atom replica (two full
    inner evaluations + merge)."""
    from atmmetaforce import synthetic as S

    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    case = S.abfe_pme_23558(seed=100)
    for _ in range(args.warmup):
        O.atm_eval(case.spec, case.pos, case.displ, case.params)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.atm_eval(case.spec, case.pos, case.displ, case.params)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "abfe-pme-23558 (one replica per step; 23,558 atoms, PME rc 0.9 nm, grid 56^3)",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} evaluations of one 23,558-atom replica"},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MD_SETTINGS = {"temperature_K": 300.0, "friction_per_ps": 1.0, "step_size_ps": 0.002,
               "thermalise_steps": 300, "thermalise_friction_per_ps": 50.0,
               "constraints": "rigid water (SETTLE)",
               "group0": "ligand bonds and angles; flat-bottom restraint of every ligand atom to its ligand's "
                         "centroid, k 25 kJ/mol/nm^2, tolerance 0.15 nm"}


def md_bench(cases_fn, R, steps, warmup, device, record_interval=0):
    """Langevin MD step rate of R replicas stepped together: 300 K, 1/ps friction,
    2 fs steps, rigid water, the ligands' bonds and angles and the flat-bottom
    centroid restraint of every ligand atom.  Host wall clock around
    ``step(steps)``, which ends with a device synchronisation; every step is one
    batched ATM evaluation plus the group-0 terms, the Langevin update, SETTLE and
    the velocity update.  With record_interval, the replicas' result records
    (u, W, dW/dlambda1, dW/dlambda2, ...) and the R x R reduced-energy matrix are
    kept on the device every record_interval steps and drained once at the end
    (inside the timed region)."""
    import atmmetaforce as atm
    from atmmetaforce import synthetic as S

    cases, terms = [], []
    for r in range(R):
        c = cases_fn(r)
        t, p = S.md_terms_ligand_centroid(c)
        c.pos = p
        cases.append(c)
        terms.append(t)
    systems = [atm.md_system_from_case(c, t)[0] for c, t in zip(cases, terms)]
    dt = MD_SETTINGS["step_size_ps"]
    integ = atm.LangevinIntegrator(MD_SETTINGS["temperature_K"], MD_SETTINGS["friction_per_ps"], dt)
    integ.setRandomNumberSeed(2024)
    sim = atm.ReplicaSimulation(systems, integ, device)
    sim.setPositions(np.concatenate([c.pos for c in cases]))
    sim.setVelocitiesToTemperature(MD_SETTINGS["temperature_K"], 7)
    # the seeded boxes start from a lattice far from equilibrium: the energy it
    # releases is taken out at high friction first, then the stated friction applies
    integ.setFriction(MD_SETTINGS["thermalise_friction_per_ps"])
    sim.step(MD_SETTINGS["thermalise_steps"])
    integ.setFriction(MD_SETTINGS["friction_per_ps"])
    # launch configuration and pair-list skin chosen by the autotuner (state restored after)
    tune = sim.autotune(trials=60).strip().splitlines()  # 60 timed steps per skin: steadier choice
    sim.step(warmup)
    if record_interval:
        sim.setRecording(record_interval, capacity=steps // record_interval + 1)
    t0 = time.perf_counter()
    sim.step(steps)
    rec = sim.getRecords() if record_interval else None
    el = time.perf_counter() - t0
    sps = steps / el
    n_atoms = int(sum(c.n for c in cases))
    st = sim.getState(getEnergy=True)
    temps = sim.temperatures(st.getKineticEnergy())
    out = {"replicas": R, "atoms": n_atoms, "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 * el / steps,
           "steps_per_s": sps, "ns_per_day_per_replica": sps * dt * 86400.0 / 1000.0,
           "ns_per_day_aggregate": R * sps * dt * 86400.0 / 1000.0, "reorders": sim.info()["reorders"],
           "lambdas": [[float(c.params[0]), float(c.params[1])] for c in cases[:1]] if R == 1 else "22-state schedule",
           "final_temperature_K": float(np.mean(temps)), "settings": MD_SETTINGS,
           "autotune": [l for l in tune if l.startswith("list skin") or l.startswith("chosen")],
           "lists": sim.listInfo()}
    if rec is not None:
        out["records"] = {"interval_steps": record_interval, "kept": int(len(rec["steps"])),
                          "per_record": "R result records (u, W, dW/dlambda1, dW/dlambda2, ...) + R x R matrix",
                          "last_dW_dlambda1": rec["results"][-1, :, 10].tolist()[:3],
                          "last_dW_dlambda2": rec["results"][-1, :, 11].tolist()[:3]}
    del sim
    return out


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        reference_arm(args, rank, world, pg)
        return
    import torch

    import atmmetaforce as atm
    from atmmetaforce import synthetic as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    R = args.replicas
    if R == 22:
        cases = S.abfe_pme_23558_x22(seed0=100 + 1000 * rank)
    else:
        cases = []
        for r in range(R):
            l1, l2 = S.SCHEDULE_22[r % 22]
            cases.append(S.abfe_pme_23558(seed=100 + 1000 * rank + r, lambdas=(l1, l2), alpha=0.1, u0=110.0))
    systems = [atm.system_from_case(c)[0] for c in cases]
    pos_host = np.ascontiguousarray(np.concatenate([c.pos for c in cases]))
    batch = atm.ReplicaBatch(systems, local, {"DifferencePath": 1})
    batch.evaluate(pos_host)  # layout + capacity
    if args.ncu_case:
        # a few evaluations of the benchmarked batch, for a profiler to capture
        # (with --tune-cache: at the tuning a plain run stored for this GPU)
        if args.tune_cache:
            batch.autotune(trials=5, use_cache=True)
        for _ in range(args.ncu_case):
            batch.evaluate(pos_host)
        print(json.dumps({"ncu_case": args.ncu_case, "launches_per_evaluation": batch.launchCount()}), flush=True)
        return
    tune_report = batch.autotune(trials=5, use_cache=args.tune_cache)  # set-up, outside the timed region

    stream = torch.cuda.current_stream(dev)
    d_pos = torch.from_numpy(pos_host).to(dev)
    d_f = torch.empty_like(d_pos)
    d_res = torch.empty((R, atm.NUM_RES), dtype=torch.float64, device=dev)
    flush = torch.empty(int(2 * L2_BYTES) // 4, dtype=torch.float32, device=dev)

    def timed_steps(b, dp, df, dr, steps, warmup):
        for _ in range(warmup):
            b.evaluateDevice(dp.data_ptr(), df.data_ptr(), dr.data_ptr(), stream.cuda_stream)
        total = 0.0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        barrier(pg)
        for k in range(steps):
            flush.zero_()  # L2 flush between timed iterations (outside the events)
            ev[k][0].record(stream)
            b.evaluateDevice(dp.data_ptr(), df.data_ptr(), dr.data_ptr(), stream.cuda_stream)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        barrier(pg)
        for s, e in ev:
            total += s.elapsed_time(e)
        return total / steps

    with ClockSampler(local) as clk:
        ms_batched = timed_steps(batch, d_pos, d_f, d_res, args.steps, args.warmup)
    ms_batched = max_over_ranks(ms_batched, pg, dev)
    value = world * R * 1000.0 / ms_batched

    # end to end through the C ABI with page-locked host buffers: every step copies
    # the positions in and the forces, energies and results out
    pos_pin = torch.from_numpy(pos_host).pin_memory().numpy()
    F_pin = torch.empty(pos_host.shape, dtype=torch.float64).pin_memory().numpy()
    for _ in range(args.warmup):
        batch.evaluate(pos_pin, out=F_pin, as_array=True)
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        E, F, res = batch.evaluate(pos_pin, out=F_pin, as_array=True)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, pg, dev)
    e2e_value = world * R / e2e_s
    h2d = pos_host.nbytes
    d2h = F.nbytes + R * atm.NUM_RES * 8 + R * R * 8  # forces, result records, R x R matrix
    F_gpu, res_gpu = F.copy(), res.copy()  # the last evaluation of the batch (positions pos_host)

    # plain single-replica drop-in (two full inner evaluations)
    plain = None
    if not args.no_plain:
        p_sys = [atm.system_from_case(cases[0])[0]]
        pb = atm.ReplicaBatch(p_sys, local, {"DifferencePath": 0})
        pb.evaluate(cases[0].pos)
        pb.autotune(trials=5, use_cache=args.tune_cache)
        dp1 = torch.from_numpy(np.ascontiguousarray(cases[0].pos)).to(dev)
        df1 = torch.empty_like(dp1)
        dr1 = torch.empty((1, atm.NUM_RES), dtype=torch.float64, device=dev)
        ms_plain = timed_steps(pb, dp1, df1, dr1, args.steps, args.warmup)
        plain = {"value": 1000.0 / ms_plain, "unit": "evals/s", "ms_per_eval": ms_plain,
                 "config": "1 replica, two full inner evaluations (reference's path)"}
        _, F_plain, res_plain = pb.evaluate(cases[0].pos, as_array=True)
        pbd = atm.ReplicaBatch([atm.system_from_case(cases[0])[0]], local, {"DifferencePath": 1})
        pbd.evaluate(cases[0].pos)
        pbd.autotune(trials=5, use_cache=args.tune_cache)
        ms_pd = timed_steps(pbd, dp1, df1, dr1, args.steps, args.warmup)
        plain["difference_path_single"] = {"value": 1000.0 / ms_pd, "ms_per_eval": ms_pd}

    # roofline of the dominant kernel (pair tiles), timed live with CUDA events
    batch.setProfiling(True)
    kt = {}
    for _ in range(3):
        batch.evaluate(pos_host)
        for k, v in batch.kernelTimes().items():
            kt.setdefault(k, []).append(v)
    batch.setProfiling(False)
    kt = {k: float(np.median(v)) for k, v in kt.items()}
    pairs_state1 = 0
    pairs_lig = 0
    for c in cases:
        a, b = count_pairs(c)
        pairs_state1 += a
        pairs_lig += b
    # the pair-tile kernel, or the fused lists + pair-tile kernel when the autotuner chose it
    fused = "find_tiles" in kt
    t_tiles = kt.get("find_tiles" if fused else "tiles", float("nan")) * 1e-3
    flops = (pairs_state1 + pairs_lig) * F_PAIR
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(dev)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = flops / t_tiles / 1e12
    roofline = {"bound": "fp32",
                "kernel": "k_find_tiles (lists + pair tiles, fused)" if fused else "k_tiles (pair tiles)",
                "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "traffic": None if fused else TILES_TRAFFIC_BYTES,
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one k_tiles launch, ncu --set full "
                                  f"capture of this workload at commit {TILES_CAPTURE} (bytes per launch)"
                                  + ("; not captured for the fused kernel" if fused else ""),
                "peak_source": f"nominal FP32: {props.multi_processor_count} SMs x 128 lanes x 2 x {sm_mhz:.0f} MHz "
                               "(MEASURED_PEAKS holds no FP32 figure)",
                "algorithmic": f"{pairs_state1 + pairs_lig} pairs within cutoff x {F_PAIR:.0f} flops",
                "kernel_ms": t_tiles * 1e3, "kernel_times_ms": kt, "tile_stats": batch.stats(),
                "pair_slot_efficiency": (pairs_state1 + pairs_lig) / max(1, 256 * batch.stats()["tiles"]),
                "issue": None if fused else {"achieved": TILES_WARP_INSTR / t_tiles / 1e12,
                          "peak": props.multi_processor_count * 4 * sm_mhz * 1e6 / 1e12,
                          "unit": "T warp instructions/s",
                          "frac": TILES_WARP_INSTR / t_tiles / (props.multi_processor_count * 4 * sm_mhz * 1e6),
                          "source": f"instructions per launch from the ncu capture at commit {TILES_CAPTURE}, "
                                    "kernel time live"}}

    md = None
    if not args.no_md:
        from atmmetaforce import synthetic as S

        def abfe(r):
            l1, l2 = S.SCHEDULE_22[r % 22]
            return S.abfe_pme_23558(seed=100 + 1000 * rank + r, lambdas=(l1, l2), alpha=0.1, u0=110.0)

        def rbfe(r):
            l1, l2 = S.SCHEDULE_22[r % 22]
            c = S.rbfe_pme_60000(seed=400 + 1000 * rank + r)
            c.params = S.default_params(l1, l2, 0.1, 110.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
            return c

        def plain_md(r):  # lambda1 = lambda2 = 0.25, alpha 0
            return S.abfe_pme_23558(seed=100 + 1000 * rank + r)

        md = {"abfe-pme-23558 x1": md_bench(plain_md, 1, args.md_steps, 20, local),
              "abfe-pme-23558 x22": md_bench(abfe, 22, max(20, args.md_steps // 50), 20, local),
              "rbfe-pme-60000 x22": md_bench(rbfe, 22, max(20, args.md_steps // 100), 10, local,
                                             record_interval=1)}

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        threads = os.cpu_count() or 1
        checked = sorted({0, R - 1})
        v, refs = cpu_baseline([cases[k] for k in checked], threads)
        v1, _ = cpu_baseline([cases[0]], 1, warm=False)
        cpu = {"value": v, "unit": "evals/s", "cores": threads, "kind": "port",
               "sample": f"{len(checked)} evaluations (replicas {checked}) of the 23,558-atom batch, two full "
                         "FP64 inner evaluations + merge each",
               "single_thread": {"value": v1, "unit": "evals/s", "cores": 1,
                                 "sample": "1 evaluation, one thread (the serial Reference-platform shape)"}}
        # the oracle's evaluations double as the checker of the batch's results for those replicas
        pert = atm.RES_KEYS.index("pert")
        du, fr = [], []
        for k, ref in zip(checked, refs):
            du.append(abs(float(res_gpu[k, pert]) - ref["usc"]))
            fr.append(force_rms_rel(F_gpu[batch.offsets[k]:batch.offsets[k + 1]], ref["forces"]))
        parity = {"replicas_checked": checked, "max_du_kj_mol": max(du), "max_force_rms_rel": max(fr),
                  "targets": {"du_kj_mol": 0.01, "force_rms_rel": 1e-4}, "oracle": "FP64 CPU restatement"}
        if plain is not None:
            parity["plain_replica0"] = {"du_kj_mol": abs(float(res_plain[0, pert]) - refs[0]["usc"]),
                                        "force_rms_rel": force_rms_rel(F_plain, refs[0]["forces"])}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_batched, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32",
                "precision": "f32 pair and grid arithmetic, i64 fixed-point force sums, compensated f32 / f64 energy "
                             "sums, f64 merge",
                "data": "synthetic (seeded water boxes + ligand chains)",
                "config": {"workload": f"abfe-pme-23558 x{R}: {R} replicas of 23,558 atoms (7,838 waters + 44-atom "
                                       "ligand), 6.2 nm box, PME rc 0.9 nm tol 5e-4 grid 56^3, 22-state schedule",
                           "global_batch": R * world, "mode": "difference path, one CUDA graph per step",
                           "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                           "l2": "flushed between timed steps (256 MB write)",
                           "autotune": tune_report.strip().splitlines()[-1],
                           "value_definition": "replica evaluations per second = replicas x launches/s"},
                "plain": plain,
                "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "gpu_launches": batch.launchCount() * args.steps,
                "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "clocks": clk.summary(), "md": md,
                "autotune_report": tune_report.strip().splitlines()}
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
