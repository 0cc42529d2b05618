"""Benchmark of the bonded-lattice XPBD fracture substep on one GB300.

Workload (default, --workload impact): the single large lattice impact -- a
256x128x128 block of cells (4,194,304 nodes, 37,340,160 face+edge bonds, FP32)
on a ground plane, struck by a rigid iron sphere (r 0.2 m, 10 m/s) at a seeded
point, per-bond lognormal break strain (median 1.5e-3, sigma 0.3), plastic
yield at 60% of the median, 32 z-slabs, dt = 1/240 s in 10 substeps with 4
colour sweeps. Synthetic, generated from those constants (banjo_gb300.scenes).

A step is one rigid step: 10 substeps. The metric is bond projections/s: one
projection is one XPBD bond solve on a live bond, so a substep makes
4 x live bonds of them.

  value   device time (CUDA events on the backend's stream) of K steps, state
          resident in HBM; the working set (about 6 GB) is far larger than L2.
  e2e     the same metric through the C ABI from host buffers: upload of the
          host LatticeState, K steps, download, timed on the host clock.
  roofline  the projection sweep, the dominant phase: algorithmic bytes of one
          substep's sweeps (4 x (N x 24 + B x 40)) over its event-timed
          duration, against the measured HBM copy bandwidth.
  cpu_baseline  the CPU checker (a restatement of the reference CPU lane) on the
          same lattice, all host threads, steady-state substeps only.

--impl reference times the reference's CPU lane on the same workload and metric.
The reference tree does not travel to the GPU machine, so there it is the CPU
restatement of that lane (oracle/), all host threads, one substep per step.

--gpus N (torchrun, one rank per GPU): the path does not shard (one lattice);
each rank runs an independent replica and value is the sum of the replicas'
projections over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bond projections/s"
ITERATIONS = 4
SUBSTEPS_PER_STEP = 10


def peaks() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.tmp.flush()

    def summary(self) -> dict:
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_case(workload: str) -> tuple[dict, str]:
    from banjo_gb300 import scenes

    if workload == "impact":
        return scenes.impact_block(), "impact 256x128x128, 4194304 nodes, 37340160 bonds, 32 slabs, sphere 10 m/s"
    if workload == "cantilever":
        return scenes.cantilever(), "cantilever 32x8x8, 2048 nodes, 15648 bonds, pinned, loaded"
    if workload == "impact_mid":
        # The impact scene at an eighth of the volume, for profiler captures.
        case = scenes.impact_block(nx=128, ny=64, nz=64, radius=0.1)
        return case, f"impact 128x64x64, {int(case['node_count'][0])} nodes, {int(case['bond_count'][0])} bonds, 32 slabs"
    raise SystemExit(f"unknown workload {workload}")


def bytes_per_substep(n: int, b: int, plastic: bool) -> dict:
    """Algorithmic bytes of one FP32 substep: every compulsory array counted once
    per pass that needs it."""
    nodes = n * (44 + 24)
    strain = n * (36 + 12 + 1)
    bond_const = b * 56
    bond_state = b * (34 + (16 if plastic else 0))
    sweep = ITERATIONS * (n * 24 + b * 40)
    return {"total": nodes + strain + bond_const + bond_state + sweep, "sweep": sweep}


def cpu_baseline(case: dict, threads: int, substeps: int = 3) -> dict:
    """The CPU checker on `substeps` substeps of the workload; the first substep
    (the post-upload restart) is left out of the rate."""
    import oracle

    sample = dict(case)
    sample["steps"] = np.array([substeps], dtype=np.uint64)
    out = oracle.run_port(sample, threads=threads)
    secs = out["substep_seconds"][1:]
    live = int(case["bond_count"][0]) - int(out["status_u64"][4])
    rate = ITERATIONS * live * len(secs) / float(np.sum(secs))
    return {"value": rate, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{substeps} substeps of the same lattice on {threads} host threads, the first "
                      f"(restart) substep excluded; {float(np.sum(secs)):.2f} s timed"}


# ---------------------------------------------------------------------------
# Batched and served trials: drop trials of uneven sizes (edges uniform on
# 8..48 per axis, compliance log-uniform 1e-8..1e-5, break strain uniform
# 1e-3..5e-3, drop height uniform 0.1..1 m onto a ground plane; the seeded
# draws of banjo_gb300.scenes.trial_parameters), built by the library's box
# builder on host threads.
# ---------------------------------------------------------------------------
TRIAL_SPACING = 0.01


def trial_specs(count: int, seed: int = 3) -> list:
    from banjo_gb300 import scenes

    edges, comp, strain, height = scenes.trial_parameters(count=count, seed=seed)
    return [(int(e[0]), int(e[1]), int(e[2]), float(c), float(s), float(h))
            for e, c, s, h in zip(edges, comp, strain, height)]


def build_trial(lattice, spec):
    nx, ny, nz, comp, strain, height = spec
    inf = float("inf")
    lift = height + 0.5 * ny * TRIAL_SPACING
    box = lattice.build_box(nx, ny, nz, TRIAL_SPACING, center=(0.0, lift, 0.0), compliance=comp,
                            threshold=(strain, strain, inf, inf, inf, inf))
    sched = lattice.box_schedule(box)
    return sched, lattice.box_state(box, sched)


def trial_settings(lattice):
    from banjo_gb300 import scenes

    return lattice.step_settings(scenes.settings(planes=[scenes.plane((0.0, 0.0, 0.0),
                                                                      node_radius=0.5 * TRIAL_SPACING)]))


def host_threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def trial_cpu_baseline(specs, substeps: int = 2) -> dict:
    """The CPU checker with trial-level parallelism: one serial lane per host
    thread, each running whole trials of the same draw one after another (the
    stronger CPU arrangement for many small lattices). Each trial's first
    (restart) substep is left out of the rate; the rate is every timed
    projection over the timed seconds shared by the threads."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    from banjo_gb300 import scenes

    threads = host_threads()

    def one(spec):
        nx, ny, nz, comp, strain, height = spec
        case = scenes.drop_trial(nx, ny, nz, compliance=comp, break_strain=strain, drop_height=height, steps=1,
                                 substeps=substeps + 1)
        out = oracle.run_port(case, threads=1)
        secs = float(np.sum(out["substep_seconds"][1:]))
        live = int(case["bond_count"][0]) - int(out["status_u64"][4])
        return ITERATIONS * live * substeps, secs

    with ThreadPoolExecutor(threads) as ex:
        results = list(ex.map(one, specs))
    proj = sum(p for p, _ in results)
    secs = sum(t for _, t in results)
    return {"value": proj / (secs / threads), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(specs)} trials of the same draw, {substeps} substeps each after the restart, one "
                      f"serial lane per thread on {threads} threads; {secs:.1f} thread-seconds timed"}


def batched_leg(args, lattice) -> dict:
    """Config-3 trials in one batch against the same trials run one lattice at
    a time through the single-lattice backend ("plain")."""
    from concurrent.futures import ThreadPoolExecutor

    specs = trial_specs(args.trials)
    settings = trial_settings(lattice)
    batch = lattice.Batch()
    t0 = time.perf_counter()

    def add(spec):
        sched, state = build_trial(lattice, spec)
        batch.add(sched, state, lattice.Sphere())  # prepared on this thread, placed under the batch's lock
        return state.node_count, state.bond_count

    with ThreadPoolExecutor(host_threads()) as ex:
        sizes = list(ex.map(add, specs))
    build_s = time.perf_counter() - t0
    batch.settle(settings)
    tuning = None
    if not args.no_tune:
        # The autotuner: sweep launch shapes timed on these lattices (state unchanged).
        t0 = time.perf_counter()
        tuning = batch.tune()
        tuning["tune_s"] = time.perf_counter() - t0
    nodes = sum(n for n, _ in sizes)
    bonds = sum(b for _, b in sizes)
    w, k = args.warmup * SUBSTEPS_PER_STEP, args.steps * SUBSTEPS_PER_STEP
    batch.run(lattice.RunControl(max_steps=w))
    before = [batch.status(i) for i in range(len(specs))]
    batch.run(lattice.RunControl(max_steps=k))
    after = [batch.status(i) for i in range(len(specs))]
    device_s = after[0].kernel_seconds - before[0].kernel_seconds
    live = sum(b - a.broken_bonds for (_, b), a in zip(sizes, after))
    value = ITERATIONS * live * k / device_s
    launches = batch.kernels_per_substep()
    phases = batch.profile_phases(1)
    del batch

    # Plain: the first trials of the same draw, one backend at a time.
    plain_n = min(args.plain_trials, len(specs))
    plain_proj, plain_s = 0.0, 0.0
    for spec in specs[:plain_n]:
        sched, state = build_trial(lattice, spec)
        be = lattice.make_gb300_lattice_backend(sched)
        be.upload(state, settings, lattice.Sphere())
        be.run(lattice.RunControl(max_steps=w))
        st0 = be.status()
        st1 = be.run(lattice.RunControl(max_steps=k))
        plain_s += st1.kernel_seconds - st0.kernel_seconds
        plain_proj += ITERATIONS * (state.bond_count - st1.broken_bonds) * k
    plain = plain_proj / plain_s
    cpu = None if args.no_cpu_baseline else trial_cpu_baseline(specs[:args.cpu_trials])
    return {"value": value, "unit": "projections/s", "trials": len(specs), "nodes": nodes, "bonds": bonds,
            "cpu_baseline": cpu,
            "ms_per_step": device_s / args.steps * 1e3, "gpu_launches_per_substep": launches,
            "host_build_s": build_s, "host_threads": host_threads(),
            "plain": {"value": plain, "unit": "projections/s", "trials": plain_n,
                      "note": "the first trials of the same draw, each alone through the single-lattice backend "
                              "(its own captured substep graph), device time summed"},
            "speedup_vs_plain": value / plain, "tuning": tuning,
            "phase_ms_per_substep": {name: v for name, v in phases.items() if v > 0},
            "workload": f"{len(specs)} drop trials, edges 8..48 per axis (seeded), one batch; step = "
                        f"{SUBSTEPS_PER_STEP} substeps, I={ITERATIONS}; device time of {args.steps} steps"}


def served_leg(args, lattice) -> dict:
    """Config-4 requests: Poisson arrivals, 90% config-3 trials and 10% 128^3
    lattices, admitted against a device memory budget, stepped together."""
    import threading

    rng = np.random.default_rng(11)
    small = trial_specs(args.served_pool)
    large_specs = [(128, 128, 128, s[3], s[4], s[5]) for s in trial_specs(2, seed=5)]
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(host_threads()) as ex:
        pool_small = list(ex.map(lambda sp: build_trial(lattice, sp), small))
        pool_large = list(ex.map(lambda sp: build_trial(lattice, sp), large_specs))
    arrivals = np.cumsum(rng.exponential(1.0 / args.served_rate, size=int(args.served_rate * args.served_window * 3)))
    arrivals = arrivals[arrivals < args.served_window]
    kinds = rng.random(arrivals.size) < 0.1
    picks = [(pool_large[int(rng.integers(len(pool_large)))] if big else pool_small[int(rng.integers(len(pool_small)))])
             for big in kinds]
    horizon = args.served_substeps
    server = lattice.Server(trial_settings(lattice), int(args.served_budget_gb * (1 << 30)))
    sphere = lattice.Sphere()
    tickets = [None] * arrivals.size
    start = time.perf_counter()

    # Clients submit from a pool of host threads, each request at its arrival
    # (submission prepares the request's sweep order on the submitting
    # thread; the library's parallel loops share the host's cores).
    clients = ThreadPoolExecutor(max(1, host_threads() - 2))

    def submit(i):
        sched, state = picks[i]
        # Borrowed: the pool's states outlive the leg, so the device reads
        # them at admission and no host image is written per request.
        tickets[i] = server.submit(sched, state, sphere, horizon, borrow=not args.served_copy)

    def produce():
        for i, t in enumerate(arrivals):
            delay = start + float(t) - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            clients.submit(submit, i)
        clients.shutdown(wait=True)

    producer = threading.Thread(target=produce)
    producer.start()
    done, latency, wait, proj = set(), {}, {}, 0.0
    steps, step_s, poll_s = 0, 0.0, 0.0
    while len(done) < arrivals.size:
        t0 = time.perf_counter()
        st = server.step(args.served_chunk)
        step_s += time.perf_counter() - t0
        steps += 1
        if st.running == 0 and st.queued == 0:
            time.sleep(0.0005)  # nothing admitted yet: wait for the next arrival
        t0 = time.perf_counter()
        for i, t in enumerate(tickets):
            if t is None or i in done:
                continue
            info = server.poll(t)
            if info.phase == lattice.REQUEST_DONE:
                _, st = server.take(t, None)
                finished = time.perf_counter() - start
                latency[i] = finished - float(arrivals[i])
                wait[i] = info.admitted_s - info.submitted_s
                b = picks[i][1].bond_count
                proj += ITERATIONS * (b - st.broken_bonds) * horizon
                done.add(i)
        poll_s += time.perf_counter() - t0
        if not producer.is_alive() and all(t is not None for t in tickets) and len(done) == arrivals.size:
            break
    producer.join()
    wall = time.perf_counter() - start
    stats = server.stats()
    lat = np.array([latency[i] for i in range(arrivals.size)])
    wq = np.array([wait[i] for i in range(arrivals.size)])
    return {"value": proj / wall, "unit": "projections/s", "requests": int(arrivals.size),
            "large_requests": int(kinds.sum()), "substeps_per_request": horizon,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "p50_admission_wait_s": float(np.percentile(wq, 50)), "p99_admission_wait_s": float(np.percentile(wq, 99)),
            "wall_s": wall, "device_s": stats.device_seconds, "budget_gb": args.served_budget_gb,
            "steps": steps, "host_step_s": step_s, "host_poll_s": poll_s, "server_admit_s": stats.admit_seconds,
            "server_retire_s": stats.retire_seconds, "server_run_s": stats.run_seconds,
            "chunk_substeps": args.served_chunk, "submission": "copied" if args.served_copy else "borrowed",
            "workload": f"Poisson arrivals at {args.served_rate:g}/s for {args.served_window:g} s; 90% drawn from "
                        f"{len(pool_small)} config-3 trials, 10% 128^3 lattices; {horizon} substeps each (a bounded "
                        f"horizon: the full 2400 would hold the GPU for hours at this arrival rate); latency = "
                        "finish - scheduled arrival, wall clock"}


def fp64_error(case: dict, gpu: dict, cpu64: dict) -> dict:
    """FP32 device run against the FP64 CPU restatement on the same case:
    position error over the lattice extent, ledger relative errors, and the
    bonds whose broken state differs."""
    ref = case["ref_pos"].reshape(-1, 3)
    extent = float(np.max(ref.max(axis=0) - ref.min(axis=0)))
    du = np.abs(gpu["u"].astype(np.float64) - cpu64["u"]).max()
    rel = lambda a, b: abs(a - b) / max(abs(b), 1e-300)  # noqa: E731
    return {"max_position_error_over_extent": float(du / extent),
            "removed_energy_rel_error": rel(float(gpu["status_f64"][0]), float(cpu64["status_f64"][0])),
            "plastic_work_rel_error": rel(float(gpu["status_f64"][2]), float(cpu64["status_f64"][2])),
            "broken_bonds_fp32": int(gpu["status_u64"][4]), "broken_bonds_fp64": int(cpu64["status_u64"][4]),
            "broken_state_differs": int(np.count_nonzero(gpu["alive"] != cpu64["alive"]))}


def cascade_leg(args, lattice) -> dict:
    """Config 5: the notched bar (energy-scaled law, plastic flow, horizon 2)
    under its ramped end load on the device, and its error against the FP64
    CPU restatement over the first steps."""
    import oracle
    from banjo_gb300 import scenes

    case = scenes.notched_bar(steps=args.cascade_steps)
    n, b = int(case["node_count"][0]), int(case["bond_count"][0])
    sched = lattice.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = lattice.build_lattice_state(case, sched)
    be = lattice.make_gb300_lattice_backend(sched)
    be.upload(state, lattice.step_settings(case["settings"]), lattice.Sphere())
    base = case["forces"]
    per = SUBSTEPS_PER_STEP
    proj, device_s = 0.0, 0.0
    for step in range(args.cascade_steps):
        scale = float(case["force_ramp_scale"][0]) * step / float(case["force_ramp_steps"][0])
        be.set_external_forces(scale * base, per)
        before = be.status()
        st = be.run(lattice.RunControl(max_steps=per))
        device_s += st.kernel_seconds - before.kernel_seconds
        proj += ITERATIONS * (b - st.broken_bonds) * per
    out = {"value": proj / device_s, "unit": "projections/s", "nodes": n, "bonds": b,
           "steps": args.cascade_steps, "broken_bonds": int(st.broken_bonds),
           "removed_energy_j": st.removed_energy_j, "plastic_work_j": st.plastic_work_j,
           "max_plastic_stretch": st.max_plastic_stretch,
           "workload": f"notched bar 128x32x32 (slot at mid-length, lower half), horizon 2, energy-scaled law + "
                       f"plastic flow compiled in FP64; end load ramped 0 -> 2x(45 MPa x 0.1024 m^2) over 10000 "
                       f"steps, the first {args.cascade_steps} steps run; device time"}
    if args.cascade_fp64_steps > 0:
        short = scenes.notched_bar(steps=args.cascade_fp64_steps)
        gpu = lattice.run_case(short)
        cpu64 = oracle.run_port(short, precision="double", threads=os.cpu_count() or 1)
        out["fp64_check"] = dict(fp64_error(short, gpu, cpu64), steps=args.cascade_fp64_steps,
                                 note="device FP32 vs the CPU restatement in FP64 (direct arithmetic), same case")
    return out


def distributed():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # One GPU per rank, made the only visible device before any CUDA call,
        # so the lattice library and torch agree on it without coordination.
        visible = os.environ.get("CUDA_VISIBLE_DEVICES")
        if visible:
            os.environ["CUDA_VISIBLE_DEVICES"] = visible.split(",")[local]
        else:
            os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
        return rank, world, 0, dist, torch
    return rank, world, local, None, None


def barrier(dist, torch):
    if dist is not None:
        dist.barrier()
        torch.cuda.synchronize()


def max_over_ranks(x: float, dist, torch) -> float:
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, dist, torch) -> float:
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_gb300(args) -> None:
    rank, world, local, dist, torch = distributed()
    from banjo_gb300 import build as lib_build
    from banjo_gb300 import lattice

    lib_build.build()
    case, desc = make_case(args.workload)
    n, b = int(case["node_count"][0]), int(case["bond_count"][0])
    sched = lattice.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = lattice.build_lattice_state(case, sched)
    settings = lattice.step_settings(case["settings"])
    sphere = lattice.sphere_state(case["sphere"])
    backend = lattice.make_gb300_lattice_backend(sched)
    backend.upload(state, settings, sphere)
    if "forces" in case:
        backend.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    substeps_w = args.warmup * SUBSTEPS_PER_STEP
    substeps_k = args.steps * SUBSTEPS_PER_STEP
    backend.run(lattice.RunControl(max_steps=substeps_w))
    launches = backend.kernels_per_substep()

    # Timed region: K steps, device-timed with the backend's CUDA events.
    before = backend.status()
    sampler = ClockSampler(local)
    barrier(dist, torch)
    with sampler:
        t0 = time.perf_counter()
        st = backend.run(lattice.RunControl(max_steps=substeps_k))
        host_s = time.perf_counter() - t0
    barrier(dist, torch)
    device_s = st.kernel_seconds - before.kernel_seconds
    # Live bonds counted after each failure round of the window (a lower bound
    # on projections: a bond that breaks in a substep was live through it).
    live_end = b - st.broken_bonds
    projections = ITERATIONS * live_end * substeps_k
    device_s_max = max_over_ranks(device_s, dist, torch)
    total_proj = sum_over_ranks(float(projections), dist, torch)
    clocks = sampler.summary()

    # Roofline of the projection sweep: event-timed phases of a few substeps.
    phases = backend.profile_phases(args.profile_substeps)
    sweep_ms = (phases["sweep_interior"] + phases["sweep_boundary"]) / args.profile_substeps
    plastic = float(case["settings"][8]) > 0.0
    algo = bytes_per_substep(n, b, plastic)
    peak, peak_kind = peaks()
    achieved = algo["sweep"] / (sweep_ms * 1e-3) / 1e9
    # DRAM bytes of one substep's sweep (its 116 level launches), measured by
    # ncu (dram__bytes_read.sum + dram__bytes_write.sum, warm caches) on the
    # impact workload at 128x64x64 (4,616,704 bonds): 759.26 MB, scaled here by
    # bonds (the traffic grows with the bonds processed).
    traffic = 759.26e6 * b / 4616704.0 if args.workload.startswith("impact") else None
    sub_per_s = substeps_k / device_s
    total_gbs = algo["total"] * sub_per_s / 1e9

    # e2e: through the C ABI from host buffers (upload, K steps, download).
    e2e_state = lattice.build_lattice_state(case, sched)
    e2e_backend = lattice.make_gb300_lattice_backend(sched)
    t0 = time.perf_counter()
    e2e_backend.upload(e2e_state, settings, sphere)
    t1 = time.perf_counter()
    e2e_st = e2e_backend.run(lattice.RunControl(max_steps=substeps_k))
    t2 = time.perf_counter()
    e2e_backend.download(e2e_state)
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"upload_s": t1 - t0, "run_s": t2 - t1, "download_s": e2e_s - (t2 - t0)}
    e2e_proj = ITERATIONS * (b - e2e_st.broken_bonds) * substeps_k
    e2e_s_max = max_over_ranks(e2e_s, dist, torch)
    e2e_total = sum_over_ranks(float(e2e_proj), dist, torch)
    # Bytes copied: upload takes the state's own arrays as they are (the device
    # converts them) -- 14 doubles per node; per neighbour slot the rest
    # vector, weight, alive flag, other node and bond; per bond 19 arrays
    # (ends, slots, flags, rest data, thresholds, damage state) and the
    # storage order -- and download returns u, u_prev, v and 8 bond arrays.
    d = max(1, state.view.max_degree)
    h2d = n * 14 * 8 + n * d * 41 + b * (164 + 4)
    d2h = n * 3 * 24 + b * (2 + 6 * 8)

    line = {
        "metric": METRIC,
        "value": total_proj / device_s_max,
        "unit": "projections/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": device_s_max / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (f64 ledgers)",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": desc, "substeps_per_step": SUBSTEPS_PER_STEP, "iterations": ITERATIONS,
                   "nodes": n, "bonds": b, "parallelism": f"replicas{world}" if world > 1 else "single lattice",
                   "l2": "working set ~6 GB >> 129 MB L2 (no flush needed)",
                   "live_bonds_end": live_end, "broken_in_window": st.broken_bonds - before.broken_bonds},
        "e2e": {"value": e2e_total / e2e_s_max, "unit": "projections/s", "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps,
                "note": "one upload of the host LatticeState (converted on the device), K steps, one download; wall clock", **e2e_parts},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_per": "substep sweep (bytes)",
                     "algorithmic_bytes_per_substep_sweep": algo["sweep"],
                     "peak_kind": peak_kind, "kernel": "kSolve (projection sweep)",
                     "sweep_ms_per_substep": sweep_ms, "whole_substep_gbs": total_gbs,
                     "whole_substep_frac": total_gbs / peak},
        # The reference scene's own rate, bonds x substeps / time
        # (TileImpactScene.cpp:867-868), over the same device and e2e windows.
        "bond_updates_per_s": {"device": world * b * substeps_k / device_s_max,
                               "e2e": world * b * substeps_k / e2e_s_max},
        "gpu_launches": launches * substeps_k,
        "clocks": clocks,
        "host_seconds": host_s,
        "phase_ms_per_substep": {k: v / args.profile_substeps for k, v in phases.items() if v > 0},
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(case, os.cpu_count() or 1)
        # The serial lane as well (one host thread), on one substep after the restart.
        line["cpu_baseline_serial"] = cpu_baseline(case, 1, substeps=2)
    del backend, e2e_backend, state, e2e_state, case
    if args.trials > 0:
        line["batched"] = batched_leg(args, lattice)
    if args.served_window > 0:
        line["served"] = served_leg(args, lattice)
    if args.cascade_steps > 0:
        line["cascade"] = cascade_leg(args, lattice)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    oracle.build_port()
    case, desc = make_case(args.workload)
    threads = os.cpu_count() or 1
    b = int(case["bond_count"][0])
    # One step = one substep of the workload (bounded so the run ends in minutes);
    # warm-up substeps (including the post-upload restart) are run, not timed.
    sample = dict(case)
    sample["steps"] = np.array([args.warmup + args.steps], dtype=np.uint64)
    out = oracle.run_port(sample, threads=threads)
    secs = out["substep_seconds"][args.warmup:]
    live = b - int(out["status_u64"][4])
    value = ITERATIONS * live * len(secs) / float(np.sum(secs))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "projections/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": float(np.mean(secs)) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (f64 ledgers)",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": desc, "substeps_per_step": 1, "iterations": ITERATIONS},
        "cpu_baseline": {"value": value, "unit": "projections/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} substeps after {args.warmup} warm-up substeps, {threads} threads; "
                                   "the reference tree is absent here, so its CPU lane runs as the restatement"},
        "e2e": {"value": value, "unit": "projections/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=6)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="impact", choices=["impact", "impact_mid", "cantilever"])
    p.add_argument("--profile-substeps", type=int, default=3)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--trials", type=int, default=4096, help="batched leg: trials in one batch (0: skip)")
    p.add_argument("--plain-trials", type=int, default=64, help="batched leg: trials timed one at a time")
    p.add_argument("--no-tune", action="store_true", help="batched leg: keep the default launch shapes")
    p.add_argument("--cpu-trials", type=int, default=96,
                   help="batched leg: trials in the trial-parallel CPU baseline sample")
    p.add_argument("--served-copy", action="store_true",
                   help="served leg: submit copied states (a host image per request) instead of borrowed ones")
    p.add_argument("--served-window", type=float, default=0.25, help="served leg: seconds of arrivals (0: skip)")
    p.add_argument("--served-rate", type=float, default=2000.0)
    p.add_argument("--served-substeps", type=int, default=40)
    p.add_argument("--served-chunk", type=int, default=10)
    p.add_argument("--served-pool", type=int, default=256)
    p.add_argument("--served-budget-gb", type=float, default=80.0)
    p.add_argument("--cascade-steps", type=int, default=200, help="notched-bar leg: ramp steps run (0: skip)")
    p.add_argument("--cascade-fp64-steps", type=int, default=10, help="notched-bar leg: steps of the FP64 check")
    args = p.parse_args()
    if args.warmup < 3:
        raise SystemExit("warm-up must be at least 3 steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
