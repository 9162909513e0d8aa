"""Benchmark: particle-steps/s of the superellipsoid timestep on one GB300.

A step is one full timestep (collider gate and pass when triggered, narrowphase + contact
law, force reduction, integration) of a seeded synthetic assembly already resident in HBM.
Prints one JSON line.  ``--impl reference`` times the CPU restatement of the reference (the
oracle, OpenMP over all host cores) on the same workload instead.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, mixed/batched vs plain FP64 at stated force error"
UNIT = "particle-steps/s"

# HBM bytes one launch of the contact kernel must move (each item once): per body the
# state it gathers (pos 24, ori 32, vel 24, angVel 24, shape 48, info 16, bounds 48) and per
# table entry the history it reads (ids+flags 12, angle 16, depth 8, normal 24, shear 24,
# phys 24) and the fields it writes (flags 4, depth 8, angle 16, normal 24, contact point 24,
# shear 24, normal force 24, force 24).
BYTES_PER_BODY = 216
BYTES_PER_PAIR = 108 + 148


TILE = os.path.join(ROOT, "tests", "golden", "config1_tile.npz")
DEFAULT_WORKLOAD = "config1_dense"
# force-error bar of the mixed form (per touching contact, relative error of normal + shear force
# after one step from identical states, against the FP64 oracle)
MIXED_TOL, MIXED_FRAC = 1e-6, 0.999
# a contact above MIXED_TOL counts as within the bar when its error is within this factor of the
# reference's own spread at double-float precision (2^-47 relative noise on its transcendental
# results), as in tests/test_mixed.py
MIXED_SPREAD_REL, MIXED_SPREAD_FACTOR = 2.0 ** -47, 3.0


def workload_spec(name, seed):
    from sudodem_gb300 import assemblies
    if name == "config1_dense":
        # the dense end of config 1: 200,000 superellipsoids (half-axes U[0.8,1.2] mm, eps U[0.3,1.8])
        # in a periodic cell at 100 kPa mean stress (5^3 copies of a 1,600-particle cell the oracle
        # compressed under config 1's isotropic loading), still under velGrad = -1/s I
        return assemblies.config1_dense(TILE, tiles=5)
    if name.startswith("config1_dense_t"):
        return assemblies.config1_dense(TILE, tiles=int(name[15:]))
    if name == "sq200k_walled":
        # 200,000 superellipsoids with the size distribution of the plain-vs-mixed config
        # (half-axes U[0.8,1.2] mm, eps1/eps2 U[0.3,1.8]) deposited in a walled box.
        return assemblies.deposition_box(200_000, seed=seed, eps_range=(0.3, 1.8))
    if name in ("config1", "config1_loose"):
        # the start of config 1: 200,000 superellipsoids, half-axes U[0.8,1.2] mm, eps U[0.3,1.8],
        # jittered lattice in a periodic cell at solid fraction 0.3 under isotropic
        # strain-controlled compression (velGrad = -1/s I)
        return assemblies.config1(seed=seed)
    if name.startswith("config1_n"):
        return assemblies.periodic_cell(int(name[9:]), seed=seed)
    if name == "sq200k_dense":
        # same particles on a 2.1 mm lattice: most neighbours start in contact (a compressed state)
        return assemblies.walled_lattice(200_000, seed=seed, box=0.2, per_side=94, spacing=2.1e-3,
                                         eps_range=(0.3, 1.8))
    if name == "config4":
        # 1,000,000 superellipsoids, half-axes log-uniform [0.5, 2] mm, eps U[0.2, 1.0], 200 x 200 mm
        # walled box under gravity, size-sorted layers (the large deposition case)
        return assemblies.config4(seed=seed)
    if name.startswith("config4_n"):
        return assemblies.config4(seed=seed, n=int(name[9:]))
    if name == "sq20k_dense":
        return assemblies.walled_lattice(20_000, seed=seed, box=0.095, per_side=44, spacing=2.1e-3,
                                         eps_range=(0.3, 1.8))
    if name == "sq1k_config0":
        return assemblies.config0(seed=seed)
    if name == "config3":
        # 5,000 superellipsoids generated as in config 0, one material per body (the specimen of
        # the differentiation window, before its deposition)
        return assemblies.config3(seed=seed)
    if name in ("hm200k_dense", "hm20k_dense"):
        # Hertz-Mindlin contact model (SuperquadricsGeom2 Nelder-Mead geometry, HertzMindlinPhys,
        # SuperquadricsLaw2): superellipsoids with half-axes U[0.8,1.2] mm, eps U[0.5,1.5] on a
        # 2.1 mm lattice in a walled box (most neighbours start in contact), SuperquadricsMat2
        # G = 1 MPa, nu = 0.3; walls keep the linear Kn = 1e5 N/m
        n, box, per = (200_000, 0.2, 94) if name == "hm200k_dense" else (20_000, 0.095, 44)
        return assemblies.hertz_mindlin(
            assemblies.walled_lattice(n, seed=seed, box=box, per_side=per, spacing=2.1e-3, eps_range=(0.5, 1.5)),
            G=1e6, nu=0.3)
    if name.startswith("sq") and name.endswith("_walled"):
        n = int(float(name[2:-7].replace("k", "e3").replace("m", "e6")))
        return assemblies.deposition_box(n, seed=seed, eps_range=(0.3, 1.8))
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_search_traffic(workload):
    """DRAM bytes (read + write) per launch of each form's search kernel, from the committed ncu
    summary of that workload (one capture at full size); {} where none was captured."""
    p = os.path.join(ROOT, "profiles", f"traffic_search_kernels_{workload}.md")
    out = {}
    if os.path.exists(p):
        for ln in open(p):
            if ln.startswith("dram_bytes_per_launch "):
                form, v = ln.split()[1], ln.split()[2]
                out[form] = float(v)
    return out


def cpu_baseline(spec, budget_s=20.0, threads=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import OracleScene
    threads = threads or os.cpu_count()
    o = OracleScene.from_spec(spec, threads=threads)
    o.step(1)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 50:
            break
    np_ = spec.n_particles
    out = {"value": np_ * n / el, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"CPU oracle, {n} timesteps of the same {np_}-particle assembly after 1 warm-up step, "
                     f"{threads} OpenMP threads, {el:.1f} s"}
    if threads > 1:
        # the same oracle on one thread (the steps that follow the timed ones)
        o.set_threads(1)
        t0 = time.perf_counter()
        n1 = 0
        while True:
            o.step(1)
            n1 += 1
            el1 = time.perf_counter() - t0
            if el1 > budget_s / 2 or n1 >= 20:
                break
        out["value_1thread"] = np_ * n1 / el1
        out["sample_1thread"] = f"{n1} further timesteps on 1 thread, {el1:.1f} s"
    return out


def config2_workload(name, seed):
    """config2: 512 walled specimens (assemblies.config2); config2_s<K>: its first K specimens."""
    from sudodem_gb300 import assemblies
    specs, servo = assemblies.config2(seed=seed)
    if name.startswith("config2_s"):
        specs = specs[:int(name[9:])]
    return specs, servo


def _oracle_specimen(args):
    spec, servo, budget = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import OracleScene
    o = OracleScene.from_spec(spec, threads=1)
    o.set_servo(servo)
    o.step(1)
    t0 = time.perf_counter()
    n = 0
    while n < 200 and time.perf_counter() - t0 < budget:
        o.step(1)
        n += 1
    return spec.n_particles * n, time.perf_counter() - t0


def cpu_baseline_batch(specs, servo, budget_s=15.0):
    """The oracle on a sample of the specimens, one specimen per host core (1 thread each, as the
    reference runs one scene per process), for about budget_s of wall time."""
    import multiprocessing as mproc
    cores = os.cpu_count()
    sample = specs[:cores]
    t0 = time.perf_counter()
    with mproc.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_oracle_specimen, [(sp, servo, budget_s) for sp in sample])
    wall = time.perf_counter() - t0
    ps = sum(r[0] for r in res)
    el = max(r[1] for r in res)
    return {"value": ps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"CPU oracle with the CompressionEngine on the first {len(sample)} specimens "
                      f"({sum(sp.n_particles for sp in sample)} particles), one specimen per core, 1 thread each, "
                      f"{el:.1f} s timed of {wall:.1f} s wall"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    import torch
    rank = int(os.environ["RANK"])
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dist.init_process_group("nccl")
    return rank, ws, dist


def run_reference(args):
    rank, ws, dist = dist_setup()
    if rank != 0:
        return
    if args.workload.startswith("config2"):
        specs, servo = config2_workload(args.workload, args.seed)
        cb = cpu_baseline_batch(specs, servo, budget_s=min(30.0, 3.0 * max(args.steps, 1)))
        v = cb["value"]
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": args.workload, "specimens": len(specs),
                           "particles": int(sum(sp.n_particles for sp in specs)), "precision": "fp64"},
                "cpu_baseline": cb,
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    spec = workload_spec(args.workload, args.seed)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import OracleScene
    threads = os.cpu_count()
    o = OracleScene.from_spec(spec, threads=threads)
    o.step(max(1, min(args.warmup, 3)))
    budget = 120.0
    t0 = time.perf_counter()
    n = 0
    while n < args.steps:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    v = spec.n_particles * n / el
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": n, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(args.workload, spec),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} timesteps of the full workload (time budget {budget:.0f} s)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours_batch(args):
    """Batched specimens (config2): each rank steps its share of the specimens as one batch."""
    rank, ws, dist = dist_setup()
    from sudodem_gb300 import Batch
    from sudodem_gb300.partition import rank_share
    specs, servo = config2_workload(args.workload, args.seed)
    sizes = [sp.n_particles for sp in specs]
    mine = rank_share(sizes, rank, ws)
    my_specs = [specs[i] for i in mine]
    precision = "fp64" if args.precision == "both" else args.precision
    b = Batch(len(my_specs), device=0, precision=precision, contacts_per_body=args.contacts_per_body)
    for e in b.scenes:
        e.set_lm_spread(not args.no_lm_spread)
    b.load(my_specs, servo=servo)
    npart = sum(sp.n_particles for sp in my_specs)
    nbodies = sum(sp.n_bodies for sp in my_specs)
    b.step(args.warmup)
    b.sync()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    if dist:
        dist.barrier()
    clocks.start()
    ms = b.time_steps(args.steps)
    rep = b.sync()
    clk = clocks.stop()
    launches = b.launch_count() * args.steps
    total_particles = sum(sizes)
    if dist:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = total_particles * args.steps / (ms / 1e3)
    nentries = sum(len(e.interactions(True)) for e in b.scenes)
    peak, peak_kind = measured_peaks()
    alg_bytes = BYTES_PER_BODY * nbodies + BYTES_PER_PAIR * nentries
    step_ms = ms / args.steps
    achieved = alg_bytes / (step_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "batch step (all specimens' kernels, concurrent graph branches)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": None, "algorithmic_bytes": alg_bytes, "launch_ms": step_ms,
                "note": "contact-stage algorithmic bytes of all specimens per batch step over the step time"}
    import torch
    kin = np.concatenate([e.kinematics() for e in b.scenes])
    hin = torch.empty(kin.shape, dtype=torch.float64, pin_memory=True)
    hout = torch.empty(kin.shape, dtype=torch.float64, pin_memory=True)
    hin.numpy()[:] = kin
    e2e_steps = max(3, min(args.steps, 10))
    ems = b.time_e2e(e2e_steps, hin.data_ptr(), hout.data_ptr())
    if dist:
        t = torch.tensor([ems], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ems = float(t.item())
    e2e = {"value": total_particles * e2e_steps / (ems / 1e3), "unit": UNIT,
           "h2d_bytes_per_step": 128 * nbodies, "d2h_bytes_per_step": 128 * nbodies}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_batch(specs, servo, budget_s=min(args.cpu_budget, 15.0))
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f32+f64",
                "data": "synthetic",
                "config": {"workload": args.workload, "specimens": len(specs), "particles": total_particles,
                           "particles_rank0": npart, "table_entries_rank0": nentries, "precision": precision,
                           "parallelism": "specimens sharded across ranks (balanced particle counts)",
                           "engine": "CompressionEngine shear phase, lateral walls at 100 kPa",
                           "l2": f"inputs larger than L2: {nentries} table entries x >= 256 B on rank 0"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
                "report": rep}
        print(json.dumps(line))


def workload_config(name, spec):
    """The workload's description, the same dict in both arms (nothing measured in it)."""
    cfg = {"workload": name, "particles": spec.n_particles, "bodies": spec.n_bodies,
           "contact_model": spec.info.get("contact_model", "linear"), "parallelism": "replicas",
           "periodic": bool(spec.info.get("periodic", False)),
           "l2": f"inputs larger than L2: {spec.n_bodies} bodies x 256 B of state + a contact table of "
                 f"~6-12 entries per particle x 256 B, well above 129 MB"}
    if name == "config1_dense":
        cfg["state"] = (f"periodic cell of 5^3 copies of a 1,600-particle cell compressed to "
                        f"{spec.info['tile_mean_stress'] / 1e3:.0f} kPa mean stress (solid fraction "
                        f"{spec.info['tile_solid_fraction']:.3f}), under config 1's velGrad = -1/s I")
    return cfg


def pipe_flops_per_eval():
    """FP32 and FP64 flops of one Disfunction evaluation (double-float and FP64 forms), from the
    committed ncu summary of the pipe-peak kernels (2 x FMA + ADD + MUL instructions per thread,
    per evaluation)."""
    p = os.path.join(ROOT, "profiles", "pipe_peaks_flops.md")
    out = {}
    if os.path.exists(p):
        for ln in open(p):
            for key in ("fp32_flops_per_ff_eval", "fp64_flops_per_fp64_eval", "fp64_flops_per_ff_eval"):
                if ln.startswith(key + ":"):
                    out[key] = float(ln.split(":")[1])
    return out


def measure_form(spec, precision, args, rank, ws, dist):
    """Throughput of one precision form on the workload: CUDA-graph timesteps timed with CUDA
    events on the engine stream (max over ranks), per-stage and search-kernel device times from
    eager steps, and the end-to-end figure through the C ABI with pinned host buffers."""
    from sudodem_gb300 import Engine
    eng = Engine(device=0, precision=precision, contacts_per_body=args.contacts_per_body)
    eng.set_lm_spread(not args.no_lm_spread)
    eng.load(spec)
    tune = None
    if not args.no_autotune:
        # launch shapes of the contact stage picked on a second copy of the scene (shapes change
        # no result; the measured scene runs exactly the steps it runs untuned)
        tuner = Engine(device=0, precision=precision, contacts_per_body=args.contacts_per_body)
        tuner.set_lm_spread(not args.no_lm_spread)
        tuner.load(spec)
        tune = tuner.autotune(steps=3)
        tuner.close()
        eng.set_launch_shape(tune["search_blocks_per_sm"], tune["pass1_blocks_per_sm"])
    eng.step(args.warmup)
    eng.sync()
    l0 = eng.launch_count()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    if dist:
        dist.barrier()
    clocks.start()
    ms = eng.time_steps(args.steps)
    rep = eng.sync()
    clk = clocks.stop()
    launches = eng.launch_count() - l0
    if spec.info.get("contact_model") == "hertz_mindlin" and rep["nan_forces"]:
        raise SystemExit("the run stopped on a NaN contact force: timing invalid")
    if dist:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    npart = spec.n_particles
    nentries = len(eng.interactions(True))
    # eager steps: per-stage and search-kernel device times, evaluations per step
    eng.set_use_graph(False)
    k2 = 3
    eng.step(k2)
    st = eng.stage_times()
    srch = eng.search_times()
    rep2 = eng.sync()
    eng.set_use_graph(True)
    # end to end through the C ABI with pinned host buffers (kinematics in and out every step)
    import torch
    kin = eng.kinematics()
    hin = torch.empty((spec.n_bodies, 16), dtype=torch.float64, pin_memory=True)
    hout = torch.empty((spec.n_bodies, 16), dtype=torch.float64, pin_memory=True)
    hin.numpy()[:] = kin
    e2e_steps = max(3, min(args.steps, 20))
    ems = eng.time_e2e(e2e_steps, hin.data_ptr(), hout.data_ptr())
    return {"engine": eng, "value": ws * npart * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
            "e2e": {"value": ws * npart * e2e_steps / (ems / 1e3), "unit": UNIT,
                    "h2d_bytes_per_step": 128 * spec.n_bodies, "d2h_bytes_per_step": 128 * spec.n_bodies},
            "stage_ms_per_step": {"collider": st[0] / k2, "contacts": st[1] / k2, "integrate": st[2] / k2},
            "search_kernel_ms": srch[0] / k2, "fallback_kernel_ms": srch[1] / k2,
            "evals_per_step": {"double_float": rep2["evals_fp32"] / k2, "fp64": rep2["evals_fp64"] / k2},
            "fallback_searches_per_step": rep2["fallback_fp64"] / k2,
            "long_queue_searches_per_step": rep2["long_queue"] / k2,
            "table_entries": nentries, "launches": launches, "launch_shape": tune, "clocks": clk, "report": rep}


def oracle_spread(spec, state, threads, rel, seeds=(1, 2, 3)):
    """The reference's own conditioning at relative precision rel, per touching pair: the
    largest relative change of the oracle's contact force over a few seeds of last-bit noise
    on its transcendental results (oracle.set_math_noise), as tests/parity_util.oracle_spread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from oracle import OracleScene
    bodies, recs, scal, cell = state

    def step():
        o = OracleScene.from_spec(spec, threads=threads)
        o.set_bodies(bodies)
        o.set_interactions(recs)
        o.set_scalars(scal)
        if cell is not None:
            o.put_cell(cell)
        o.rebuild_sorted_bounds()
        o.step(1)
        f = {(int(r[0]), int(r[1])): (r[26:29] + r[29:32], r[4] > 0 and r[2] == 1) for r in o.interactions()}
        o.close()
        return f
    ref = step()
    out = {k: 0.0 for k, (f, t) in ref.items() if t}
    try:
        for sd in seeds:
            oracle.set_math_noise(sd, rel)
            N = step()
            for k in out:
                fr = ref[k][0]
                n = N.get(k)
                den = np.linalg.norm(fr)
                if n is None or not n[1]:
                    out[k] = np.inf
                else:
                    out[k] = max(out[k], float(np.linalg.norm(n[0] - fr) / (den if den > 0 else 1)))
    finally:
        oracle.set_math_noise(0)
    return out


def force_errors(spec, state, precisions, threads):
    """One step of the oracle and of a fresh engine per precision form from the same state
    (bodies, interactions, scalars, cell): per touching contact, the relative error of the
    normal + shear force against the oracle (the checker of the cpu_baseline leg)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import OracleScene
    from sudodem_gb300 import Engine
    bodies, recs, scal, cell = state
    o = OracleScene.from_spec(spec, threads=threads)
    o.set_bodies(bodies)
    o.set_interactions(recs)
    o.set_scalars(scal)
    if cell is not None:
        o.put_cell(cell)
    o.rebuild_sorted_bounds()
    o.step(1)
    R = {(int(r[0]), int(r[1])): r for r in o.interactions() if r[4] > 0 and r[2] == 1}
    spread = oracle_spread(spec, state, threads, MIXED_SPREAD_REL) if "mixed" in precisions else {}
    out = {}
    for prec in precisions:
        e = Engine(device=0, precision=prec)
        e.load(spec)
        e.put_body_state(bodies)
        e.put_interactions(recs)
        e.put_scalars(scal)
        if cell is not None:
            e.put_cell(cell)
        e.step(1)
        rep = e.sync()
        G = {(int(r[0]), int(r[1])): r for r in e.interactions(True)}
        keys = [k for k in R if k in G]
        g = np.array([G[k][26:29] + G[k][29:32] for k in keys])
        r = np.array([R[k][26:29] + R[k][29:32] for k in keys])
        den = np.linalg.norm(r, axis=1)
        err = np.linalg.norm(g - r, axis=1) / np.where(den > 0, den, 1)
        q = lambda p: float(np.quantile(err, p))
        out[prec] = {"touching": len(err), "median": q(0.5), "p99": q(0.99), "p999": q(0.999), "max": float(err.max()),
                     "frac_le_1e-6": float(np.mean(err <= 1e-6)), "frac_le_1e-10": float(np.mean(err <= 1e-10)),
                     "searches_deferred_to_fp64": int(rep["fallback_fp64"])}
        if spread:
            sp = np.array([spread.get(k, 0.0) for k in keys])
            ok = (err <= MIXED_TOL) | (err <= MIXED_SPREAD_FACTOR * sp)
            out[prec]["frac_within_bar"] = float(np.mean(ok))
            out[prec]["above_1e-6_within_oracle_spread"] = int(np.sum((err > MIXED_TOL) & ok))
        e.close()
    o.close()
    return out


def run_ours(args):
    if args.workload.startswith("config2"):
        return run_ours_batch(args)
    rank, ws, dist = dist_setup()
    from sudodem_gb300 import _native
    spec = workload_spec(args.workload, args.seed + rank)
    npart = spec.n_particles
    forms = ("fp64", "mixed") if args.precision == "both" else (args.precision,)
    res = {p: measure_form(spec, p, args, rank, ws, dist) for p in forms}
    peaks = _native.pipe_peaks(0)
    flops = pipe_flops_per_eval()
    traffic = profiled_search_traffic(args.workload)
    # the roofline of each form's dominant kernel (the search kernel): issue-bound on the pipe
    # its evaluations run on (FP64 for k_contacts_lm; FP32 for the double-float
    # k_contacts_lm_ff), against this GPU's measured FMA peak of that pipe
    for p, r in res.items():
        ev = r["evals_per_step"]["double_float" if p == "mixed" else "fp64"]
        kms = r["search_kernel_ms"]
        pipe = "fp32" if p == "mixed" else "fp64"
        fpe = flops.get("fp32_flops_per_ff_eval" if p == "mixed" else "fp64_flops_per_fp64_eval")
        peak = peaks["fp32_tflops" if p == "mixed" else "fp64_tflops"]
        peak_eval = peaks["disfunction_ff_geval_s" if p == "mixed" else "disfunction_fp64_geval_s"] * 1e9
        rate = ev / (kms / 1e3) if kms > 0 else 0.0
        achieved = rate * fpe / 1e12 if fpe else None
        r["roofline"] = {"bound": pipe, "kernel": "k_contacts_lm_ff" if p == "mixed" else "k_contacts_lm",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if achieved is not None else None,
                         "peak_source": "measured on this GPU by sqdem_pipe_peaks (FMA loop of that pipe)",
                         "traffic": traffic.get(p), "launch_ms": kms, "evaluations_per_launch": ev,
                         "flops_per_evaluation": fpe,
                         "evaluation_rate": rate, "peak_evaluation_rate": peak_eval,
                         "evaluation_rate_frac": rate / peak_eval if peak_eval else None,
                         "note": "Disfunction evaluations of the Levenberg-Marquardt searches dominate; flops per "
                                 "evaluation counted by ncu on the pipe-peak kernel that does nothing else"}
    cpu, ferr = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(spec, budget_s=args.cpu_budget)
        # force errors of each form against the oracle, one step from the state the FP64 engine
        # reached (the checker runs in this leg)
        e = res[forms[0]]["engine"]
        state = (e.body_state(), e.interactions(True), e.scalars(), e.cell() if spec.info.get("periodic") else None)
        ferr = force_errors(spec, state, forms, os.cpu_count())
    head = forms[0]
    if "mixed" in res and ferr and ferr["mixed"].get("frac_within_bar", ferr["mixed"]["frac_le_1e-6"]) >= MIXED_FRAC:
        head = "mixed"
    if rank == 0:
        h = res[head]
        line = {"metric": METRIC, "value": h["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64" if head == "mixed" else "f64", "data": "synthetic",
                "config": workload_config(args.workload, spec),
                "headline_form": head,
                "headline_rule": (f"mixed when at least {MIXED_FRAC:.1%} of touching contacts are within "
                                  f"{MIXED_TOL:g} relative force error of the FP64 oracle in this run, or within "
                                  f"{MIXED_SPREAD_FACTOR:g}x the oracle's own spread under 2^-47 relative noise "
                                  f"on its transcendental results (a contact the reference's arithmetic does not "
                                  f"determine to {MIXED_TOL:g} at that precision), else fp64"),
                "roofline": h["roofline"], "cpu_baseline": cpu, "e2e": h["e2e"], "clocks": h["clocks"],
                "gpu_launches": h["launches"],
                "forms": {p: {k: v for k, v in r.items() if k not in ("engine", "report", "clocks")}
                          for p, r in res.items()},
                "force_error": ferr,
                "peaks": peaks,
                "report": h["report"]}
        if "mixed" in res and "fp64" in res:
            line["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
        print(json.dumps(line))
    for r in res.values():
        r["engine"].close()


def config3_start(args):
    """Start of the config-3 window on the GPU engine: the specimen deposited for
    --deposit-steps steps and settled by --settle-rounds rounds of zeroed velocities
    (NewtonIntegrator.quiet_system_flag) 2,000 steps apart (with no viscous contact damping the
    collapsed column keeps bouncing at a few cm/s for hundreds of thousands of steps); the lid
    placed 0.05 mm above the highest particle's centre plus its largest half-axis (above every
    particle: a particle behind a wall would read as deeply penetrating it) and lowered at
    0.1 m/s, sweeping any particle still in flight ahead of it, until its force has stayed above
    0.5 N (about the bed's weight) for three checks in a row (20 steps apart); every velocity
    zeroed; then the lid brought to the preload --lid-force by a one-sided servo (every 20 steps
    it moves down at 5e-3 m/s per N of missing force, at most 1.5 mm/s, and stands still when the
    force is reached, so that it never pulls away from the bed) until the force has stayed above
    80% of the preload for 50 checks in a row (or --servo-max checks); then the lid set to the
    window's compression velocity (0.05/s x its height) for --precompress-steps steps.  The
    window is a slice of that ongoing compression."""
    from sudodem_gb300 import Engine, assemblies
    spec = assemblies.config3(seed=args.seed, n=args.particles)
    eng = Engine(device=0)
    eng.load(spec)
    eng.step(args.deposit_steps)
    for _ in range(args.settle_rounds):
        eng.set_quiet(True)
        eng.step(2000)
    b = eng.body_state()
    part = spec.kind == 0
    vp99 = float(np.percentile(np.linalg.norm(b[part, 7:10], axis=1), 99))
    b[5, 2] = float(np.max(b[part, 2] + np.max(spec.shape5[part, 0:3], axis=1))) + 0.05e-3
    b[5, 7:10] = [0.0, 0.0, -0.1]
    eng.put_body_state(b)
    held, k = 0, 0
    while held < 3 and k < args.approach_max:
        eng.step(20)
        k += 1
        held = held + 1 if abs(eng.body_state()[5, 18]) > 0.5 else 0
    reached = held >= 3
    eng.set_quiet(True)      # zeroes every body's velocity, the lid's too
    eng.step(1)
    target, gain, vmax = args.lid_force, 5e-3, 1.5e-3
    held, k2 = 0, 0
    while held < 50 and k2 < args.servo_max:
        b = eng.body_state()
        F = abs(b[5, 18])
        held = held + 1 if F >= 0.8 * target else 0
        b[5, 7:10] = [0.0, 0.0, -float(min(vmax, gain * max(0.0, target - F)))]
        eng.put_body_state(b)
        eng.step(20)
        k2 += 1
    b = eng.body_state()
    height = float(b[5, 2] - b[4, 2])
    b[5, 7:10] = [0.0, 0.0, -0.05 * height]
    eng.put_body_state(b)
    trace = []
    for k3 in range(0, args.precompress_steps, 10000):
        eng.step(min(10000, args.precompress_steps - k3))
        trace.append(round(float(abs(eng.body_state()[5, 18])), 4))
    b = eng.body_state()
    force0 = float(abs(b[5, 18]))
    recs = eng.interactions(include_potential=True)
    eng.close()
    lid = recs[(recs[:, 0] == 5) | (recs[:, 1] == 5)]
    return spec, b, recs, {"deposit_steps": args.deposit_steps, "settle_rounds": args.settle_rounds,
                           "particle_speed_p99_after_settling_m_s": vp99, "lid_steps": 20 * k, "lid_reached": bool(reached),
                           "servo_steps": 20 * k2, "servo_held": bool(held >= 50), "preload_n": target,
                           "precompress_steps": args.precompress_steps, "lid_force_every_10000_steps_n": trace,
                           "lid_height_m": height, "lid_velocity_m_s": -0.05 * height, "lid_force_n": force0,
                           "lid_pairs": int(len(lid)), "lid_pairs_touching": int(np.sum(lid[:, 4] > 0))}


# HBM bytes of one reverse step, each item once: per pair the taped state it reads (ids 8,
# flag 4, depth 8, angle 16, normal 32, shear 32, phys 32, Fv 32, contact point 32, code 4),
# its adjoints read and written (angle 16, normal 32, shear 32, twice), the contributions it
# writes (8 x 32) and the parameter accumulators (2 x 32, read and written); per body its taped
# state (5 x 32), shape/mass/eps (80) and adjoints (7 x 32, read and written twice).
ADJ_BYTES_PER_PAIR = 8 + 4 + 8 + 16 + 32 + 32 + 32 + 32 + 32 + 4 + 2 * 80 + 256 + 4 * 32
ADJ_BYTES_PER_BODY = 160 + 80 + 4 * 224


def run_ours_adjoint(args):
    """Config 3: gradient of the final lid force over a window of --window steps with respect
    to per-particle friction and exponents and the stiffnesses, through the adjoint."""
    rank, ws, dist = dist_setup()
    from sudodem_gb300.adjoint import AdjointWindow, window_loss
    spec, bodies, recs, start = config3_start(args)
    n = spec.n_bodies
    npart = spec.n_particles
    wF = np.zeros((n, 3))
    wF[5, 2] = 1.0
    wX = None
    if args.loss_heights:   # plus the particles' mean final height
        wX = np.zeros((n, 3))
        wX[spec.kind == 0, 2] = 1.0 / npart
    w = AdjointWindow(0)
    w.load(spec, bodies, recs)
    eps0 = spec.shape5[:, 3:5].copy()
    mu0 = np.tan(spec.materials["frictionAngle"])
    Kn0, Ks0 = spec.materials["Kn"].copy(), spec.materials["Ks"].copy()
    # warm-up, and the shape of the pairs' reverse-step kernel timed on a short window (every
    # shape gives bitwise the same gradients): the fastest is kept
    loss1, _ = w.forward(1, 1, wF, wX)
    shapes = {}
    nt = min(args.window, 50)
    for shape in ((1, 2, 3, 0) if args.replay_shape < 0 else (args.replay_shape,)):
        w.set_replay(shape)
        w.forward(nt, min(args.checkpoint, nt), wF, wX)
        w.backward()
        shapes[AdjointWindow.REPLAY_SHAPES[shape]] = w.report()["backward_ms"] / nt
    best = min(shapes, key=shapes.get)
    w.set_replay([k for k, v in AdjointWindow.REPLAY_SHAPES.items() if v == best][0])
    # resident blocks per SM of the grouped reverse kernel (the lanes' replayed state in L2 at 1)
    blocks = {}
    for nbk in ((1, 2, 0) if args.replay_blocks < 0 else (args.replay_blocks,)):
        w.set_replay_blocks(nbk)
        w.forward(nt, min(args.checkpoint, nt), wF, wX)
        w.backward()
        blocks[nbk] = w.report()["backward_ms"] / nt
    best_blocks = min(blocks, key=blocks.get)
    w.set_replay_blocks(best_blocks)
    clocks = ClockSampler(0)
    clocks.start()
    loss, sig = w.forward(args.window, args.checkpoint, wF, wX)
    g = w.backward()
    clk = clocks.stop()
    rep = w.report()
    ms = rep["forward_ms"] + rep["backward_ms"]
    value = npart * args.window / (ms / 1e3)
    # end to end: the torch autograd function from host parameters to host gradients
    import torch
    te = torch.tensor(eps0, dtype=torch.float64, requires_grad=True)
    tm = torch.tensor(mu0, dtype=torch.float64, requires_grad=True)
    tkn = torch.tensor(Kn0, dtype=torch.float64, requires_grad=True)
    tks = torch.tensor(Ks0, dtype=torch.float64, requires_grad=True)
    t0 = time.perf_counter()
    L = window_loss(w, te, tm, tkn, tks, args.window, args.checkpoint, wF, wX)
    L.backward()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": npart * args.window / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (2 * n + 3 * n) * 8 / args.window,
           "d2h_bytes_per_step": (2 * n + 3 * n) * 8 / args.window,
           "note": "torch.autograd.Function: parameters from host tensors, loss and gradients back to host"}
    # divergence of the window's trajectory: one particle moved by 1e-13 m at the start; the
    # separation of the two runs' positions at the end, per step (the time over which a
    # finite-difference check of the gradient can hold)
    # divergence of the trajectory: one particle moved by 1e-13 m at the start; the separation
    # of the two runs' positions after the finite-difference window and after the whole window,
    # per step (the e-folding time bounds the window over which a difference at a relative step
    # of 1e-6 stays linear)
    divergence = None
    fd, fd_summary = [], None
    if args.fd_dirs:
        fdw = min(args.fd_window, args.window)
        base = {}
        for nst in sorted({fdw, args.window}):
            w.forward(nst, args.checkpoint, wF, wX)
            base[nst] = w.state()
        pb = bodies.copy()
        ip = int(np.nonzero(spec.kind == 0)[0][npart // 2])
        pb[ip, 0] += 1e-13
        w.load(spec, pb, recs)
        divergence = {"perturbation_m": 1e-13}
        for nst in sorted(base):
            w.forward(nst, args.checkpoint, wF, wX)
            sep = float(np.max(np.abs(w.state()[:, 0:3] - base[nst][:, 0:3])))
            divergence[f"after_{nst}_steps"] = {"max_separation_m": sep,
                                                "growth_per_step": math.log(max(sep, 1e-300) / 1e-13) / nst}
        w.load(spec, bodies, recs)
        # central differences over --fd-window steps along --fd-dirs seeded directions over every
        # parameter (the kinds cycling eps, mu, Kn, Ks), at the relative step --fd-h, in FP64 on the
        # GPU: (a) runs forced onto the base run's recorded branches (sqdem_adj_set_branches), the
        # differences of the branch whose derivative the reverse pass computes; (b) the same runs
        # evaluated naturally, which count when they took the base run's branches (signature)
        w.set_branches(AdjointWindow.BRANCH_RECORD)
        Lb, sigb = w.forward(fdw, args.checkpoint, wF, wX)
        gb = w.backward()
        decisions = w.branch_report()["decisions"]
        w.set_branches(AdjointWindow.BRANCH_FORCE)
        rng = np.random.default_rng(args.seed)
        noise = 0.0   # rounding noise of the loss: runs perturbed by 1e-13, whose linear change is below it
        for k in range(4):
            d = rng.normal(size=mu0.shape) * mu0
            w.set_materials(Kn0, Ks0, mu0 + 1e-13 * d)
            ln, _ = w.forward(fdw, args.checkpoint, wF, wX)
            noise = max(noise, abs(ln - Lb - 1e-13 * float(np.sum(gb["mu"] * d))))
        part = (spec.kind == 0)[:, None]
        kinds = ("eps", "mu", "Kn", "Ks")
        h = args.fd_h
        scan = sorted({h, h / 2, *[float(x) for x in args.fd_scan.split(",") if x]}, reverse=True)

        def central(mode, dE, dmu, dKn, dKs, hh):
            w.set_branches(mode)
            vals, sigs, dis, cross = [], [], 0, 0
            for sgn in (1, -1):
                w.set_materials(Kn0 + sgn * hh * dKn, Ks0 + sgn * hh * dKs, mu0 + sgn * hh * dmu)
                w.set_eps(eps0 + sgn * hh * dE)
                lv, sv = w.forward(fdw, args.checkpoint, wF, wX)
                vals.append(lv)
                sigs.append(sv)
                if mode == AdjointWindow.BRANCH_FORCE:
                    br = w.branch_report()
                    dis += br["disagreements"]
                    cross += br["surface_sign_changes"]
            return (vals[0] - vals[1]) / (2 * hh), sigs, dis, cross

        for k in range(args.fd_dirs):
            name = kinds[k % 4]
            dE = rng.normal(size=eps0.shape) * eps0 * part if name == "eps" else 0 * eps0
            dmu = rng.normal(size=mu0.shape) * mu0 if name == "mu" else 0 * mu0
            dKn = rng.normal(size=Kn0.shape) * Kn0 if name == "Kn" else 0 * Kn0
            dKs = rng.normal(size=Ks0.shape) * Ks0 if name == "Ks" else 0 * Ks0
            ad = float(np.sum(gb["eps"] * dE) + np.sum(gb["mu"] * dmu) + np.sum(gb["Kn"] * dKn) + np.sum(gb["Ks"] * dKs))
            row = {"param": name, "adjoint": ad, "forced": {}}
            for hh in scan:
                f, _, dis, cross = central(AdjointWindow.BRANCH_FORCE, dE, dmu, dKn, dKs, hh)
                row["forced"][f"{hh:.0e}"] = {"fd": f, "rel_err": abs(f - ad) / max(abs(ad), 1e-300),
                                              "decisions_forced_against_their_natural_outcome": dis,
                                              "pair_steps_crossing_a_surface_singularity": cross,
                                              "noise_bound_rel": noise / hh / max(abs(ad), 1e-300)}
            best = min(row["forced"], key=lambda x: row["forced"][x]["rel_err"])
            row["forced_best"] = {"h": float(best), "rel_err": row["forced"][best]["rel_err"]}
            # Richardson extrapolation of the central differences at h and h/2 (their error is
            # c h^2 on a smooth branch): (4 D(h/2) - D(h)) / 3
            rich = (4 * row["forced"][f"{h / 2:.0e}"]["fd"] - row["forced"][f"{h:.0e}"]["fd"]) / 3
            row["forced_richardson"] = {"h": h, "fd": rich, "rel_err": abs(rich - ad) / max(abs(ad), 1e-300)}
            f, sigs, _, _ = central(AdjointWindow.BRANCH_NATURAL, dE, dmu, dKn, dKs, h)
            row["natural"] = {"h": h, "fd": f, "rel_err": abs(f - ad) / max(abs(ad), 1e-300),
                              "same_branches": bool(sigs[0] == sigs[1] == sigb)}
            fd.append(row)
        w.set_branches(AdjointWindow.BRANCH_NATURAL)
        at_h = [x["forced"][f"{h:.0e}"] for x in fd]
        fd_summary = {"directions": len(fd), "h_relative": h, "h_scanned": scan, "window_steps": fdw, "loss": Lb,
                      "decisions_per_run": decisions, "loss_rounding_noise": noise,
                      "forced_within_1e-5_at_h": int(sum(x["rel_err"] <= 1e-5 for x in at_h)),
                      "forced_max_rel_err_at_h": max(x["rel_err"] for x in at_h),
                      "forced_within_1e-5_or_noise_at_h": int(sum(x["rel_err"] <= 1e-5 + 2 * x["noise_bound_rel"]
                                                                  for x in at_h)),
                      "forced_at_h_without_surface_crossing": int(sum(x["pair_steps_crossing_a_surface_singularity"] == 0
                                                                      for x in at_h)),
                      "forced_within_1e-5_at_h_without_surface_crossing": int(sum(
                          x["rel_err"] <= 1e-5 for x in at_h if x["pair_steps_crossing_a_surface_singularity"] == 0)),
                      "forced_richardson_within_1e-5": int(sum(x["forced_richardson"]["rel_err"] <= 1e-5 for x in fd)),
                      "forced_within_1e-5_best_h": int(sum(x["forced_best"]["rel_err"] <= 1e-5 for x in fd)),
                      "forced_max_rel_err_best_h": max(x["forced_best"]["rel_err"] for x in fd),
                      "natural_same_branches": int(sum(x["natural"]["same_branches"] for x in fd)),
                      "natural_within_1e-5": int(sum(x["natural"]["rel_err"] <= 1e-5 for x in fd))}
    w.set_materials(Kn0, Ks0, mu0)
    w.set_eps(eps0)
    cpu = None
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from oracle import OracleScene
        threads = os.cpu_count()
        o = OracleScene.from_spec(spec, threads=threads)
        o.set_bodies(bodies)
        o.set_interactions(recs)
        o.reset_phys()
        o.set_frozen(True)
        t0 = time.perf_counter()
        nst = 0
        while nst < args.window and time.perf_counter() - t0 < args.cpu_budget:
            o.step(1)
            nst += 1
        el = time.perf_counter() - t0
        cpu = {"value": npart * nst / el, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{nst} steps of the frozen-pair window (forward only) from the same start state; a "
                         f"finite-difference gradient needs two such windows per parameter direction"}
    peak, peak_kind = measured_peaks()
    P = w.num_pairs()
    alg = ADJ_BYTES_PER_PAIR * P + ADJ_BYTES_PER_BODY * n
    step_s = rep["backward_ms"] / 1e3 / args.window
    achieved = alg / step_s / 1e9
    roofline = {"bound": "hbm", "kernel": "reverse step (k_bwd_integrate, k_bwd_contacts, k_bwd_gather, with the "
                                          "segment recompute)", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None, "algorithmic_bytes": alg,
                "note": "bound by the FP64 issue rate of the dual-number replay of the narrowphase, not by bytes"}
    launches = args.window * 2 + 1 + args.window * 5
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.window, "warmup": 1,
            "ms_per_step": ms / args.window, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "config3", "particles": npart, "bodies": n, "pairs": P, "window_steps": args.window,
                       "checkpoint_every": args.checkpoint, "parameters": {"eps": 2 * npart, "mu": n, "Kn": n, "Ks": n},
                       "loss": "final lid normal force" + (" + mean final particle height" if args.loss_heights else ""),
                       "start": start,
                       "replay_shape": best, "replay_ms_per_step_by_shape": shapes,
                       "replay_blocks_per_sm": best_blocks,
                       "replay_ms_per_step_by_blocks_per_sm": {str(k): v for k, v in blocks.items()},
                       "what": "particle-steps/s of forward + reverse window (one gradient)",
                       "l2": "state and tape larger than L2"},
            "loss": loss, "loss_after_one_step": loss1, "forward_ms": rep["forward_ms"], "backward_ms": rep["backward_ms"],
            "replay_mismatches": rep["replay_mismatches"], "grad_norms": {k: float(np.linalg.norm(v)) for k, v in g.items()},
            "fd_check": fd, "fd_summary": fd_summary,
            "divergence": divergence, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": launches}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--precision", default="both", choices=["fp64", "mixed", "both"],
                    help="single-scene workloads: time one form or both (default; the headline is the mixed form "
                         "when it meets its force-error bar in this run)")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--contacts-per-body", type=int, default=16)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes of the contact stage (no tuning steps)")
    ap.add_argument("--no-lm-spread", action="store_true",
                    help="one Levenberg-Marquardt evaluation point per lane and round (same results)")
    ap.add_argument("--window", type=int, default=2000, help="config3: steps of the differentiated window")
    ap.add_argument("--checkpoint", type=int, default=100, help="config3: steps between checkpoints")
    ap.add_argument("--particles", type=int, default=5000, help="config3: particles")
    ap.add_argument("--deposit-steps", type=int, default=200000, help="config3: deposition steps before the window")
    ap.add_argument("--fd-dirs", type=int, default=0,
                    help="config3: finite-difference directions, cycling over eps, mu, Kn, Ks")
    ap.add_argument("--fd-h", type=float, default=1e-6, help="config3: relative finite-difference step")
    ap.add_argument("--replay-shape", type=int, default=-1,
                    help="config3: shape of the reverse kernel (AdjointWindow.REPLAY_SHAPES; -1: time each, keep the fastest)")
    ap.add_argument("--replay-blocks", type=int, default=-1,
                    help="config3: resident blocks per SM of the reverse kernel (-1: time 1, 2, unbounded, keep the fastest)")
    ap.add_argument("--fd-scan", default="1e-4,1e-5,1e-7,1e-8",
                    help="config3: further relative steps of the forced central differences (comma-separated)")
    ap.add_argument("--fd-window", type=int, default=200,
                    help="config3: steps of the finite-difference check's window (at most --window)")
    ap.add_argument("--approach-max", type=int, default=20000,
                    help="config3: at most this many 20-step checks while the lid is lowered onto the bed")
    ap.add_argument("--precompress-steps", type=int, default=50000,
                    help="config3: steps of the compression at 0.05/s before the window")
    ap.add_argument("--settle-rounds", type=int, default=10,
                    help="config3: rounds of zeroed velocities, 2,000 steps apart, after the deposition")
    ap.add_argument("--lid-force", type=float, default=0.5, help="config3: lid preload (N) before the compression")
    ap.add_argument("--servo-max", type=int, default=10000,
                    help="config3: at most this many 20-step checks while the lid is brought to its preload")
    ap.add_argument("--loss-heights", action="store_true", help="config3: add the particles' mean final height to the loss")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "config3":
        run_ours_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
