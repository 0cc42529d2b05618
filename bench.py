"""Benchmark of the bonded-lattice XPBD fracture substep on one GB300.

The headline workload (--workload impact) is the single large lattice impact:
a 256x128x128 block of cells (4,194,304 nodes, 37,340,160 face+edge bonds,
FP32) on a ground plane, struck by a rigid iron sphere (r 0.2 m, 10 m/s) at a
seeded point, per-bond lognormal break strain (median 1.5e-3, sigma 0.3),
plastic yield at 60% of the median, 32 z-slabs, dt = 1/240 s in 10 substeps
with 4 colour sweeps. Every input is synthetic, generated from those constants
(banjo_gb300.scenes); no dataset exists for it.

A step is one rigid step: 10 substeps. The metric is bond projections/s: one
projection is one XPBD solve of a live bond; a substep makes iterations x the
bonds alive when its sweep starts. Both the device and the CPU restatement
count them exactly (RunStatus::bond_projections, its port counterpart).

Main line (the impact):
  value     device time (CUDA events on the backend's stream) of K steps with
            the state resident in HBM (a ~6 GB working set, far above L2).
  e2e       the same metric through the C ABI from host buffers: upload of the
            host LatticeState, K steps, download, on the host clock.
  roofline  the projection sweep, the dominant kernel: algorithmic bytes per
            substep, iterations x (nodes x 24 + live bonds x 40), over its
            event-timed duration, against the measured HBM copy bandwidth.
  parity    the first steps of the same impact on the device and in the CPU
            restatement (all host threads): every state array bit for bit, the
            substep each bond broke, every RunStatus counter, and the FP64
            ledgers within the bound another summation order allows.
  fp64_error  the device (FP32) against the restatement in FP64 on the first
            steps: position and velocity error, ledger relative errors, bonds
            whose state differs.
  cpu_baseline  the restatement's rate on the parity prefix (substeps after the
            post-upload restart), all host threads.

Legs (each with its own parity, FP64 error and CPU baseline where it applies):
  cantilever  32x8x8 pinned beam under its load, 240 steps.
  batched   4096 drop trials of uneven size in one batch against the same
            trials one backend at a time ("plain"), device time and through
            the API (e2e).
  served    requests (90% drop trials, 10% 128^3 lattices, 2400 substeps
            each) arriving as a Poisson process at 50,
            80 and 95% of the batched capacity, with p50/p99 latency, admission
            wait and admission's share of wall time; a 2000/s stress point with
            a short horizon; a sample of requests checked against the same
            request run alone.
  cascade   the 128x32x32 notched bar under its ramped end load.

--impl reference times the reference's CPU lane on the same workload, metric
and window (the substeps of the same K steps after the same W warm-up steps).
The reference tree does not travel to the GPU machine, so there it runs as the CPU
restatement of that lane (oracle/), on all host threads.

--gpus N (torchrun, one rank per GPU): the path does not shard (one lattice);
each rank runs an independent replica and value is the sum of the replicas'
projections over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
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


def host_threads() -> int:
    return max(1, min(64, os.cpu_count() or 1))


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


def sweep_bytes(n: int, live: float) -> float:
    """Algorithmic bytes of one substep's projection sweeps: per iteration,
    every node's position read and written (16 + 8: the w lane is read only)
    and every live bond's ends, rest data, rest edge and compliance (32) and
    its multiplier read and written (8)."""
    return ITERATIONS * (n * 24 + live * 40)


def prefix(case: dict, substeps: int) -> dict:
    c = dict(case)
    c["steps"] = np.array([substeps], dtype=np.uint64)
    return c


# ---------------------------------------------------------------------------
# Parity and FP64 error (the oracle is the checker here, never the thing timed
# on the device side).
# ---------------------------------------------------------------------------
def parity_report(cpu: dict, gpu: dict, break_step: bool) -> dict:
    from oracle.compare import STATE_KEYS, ledger_report, mismatches, status_mismatches

    keys = STATE_KEYS + (["break_step"] if break_step else [])
    bad_state = mismatches(cpu, gpu, keys)
    bad_status = status_mismatches(cpu, gpu, skip=("removed_energy_j", "plastic_work_j"))
    ledgers = ledger_report(cpu, gpu)
    proj_equal = int(cpu["bond_projections"][0]) == int(gpu["bond_projections"][0])
    return {"ok": not bad_state and not bad_status and ledgers["within"] and proj_equal,
            "state_bit_exact": not bad_state, "state_mismatches": bad_state,
            "break_step_equal": break_step and "break_step" not in bad_state,
            "status_equal": not bad_status, "status_mismatches": bad_status, "ledgers": ledgers,
            "bond_projections_equal": proj_equal, "broken_bonds": int(cpu["status_u64"][4]),
            "substeps": int(cpu["status_u64"][0])}


def fp64_error(case: dict, gpu: dict, cpu64: dict) -> dict:
    """FP32 device run against the FP64 CPU restatement on the same case:
    position error over the lattice extent, velocity error over the largest
    FP64 speed, ledger relative errors, and the bonds whose state differs."""
    ref = np.asarray(case["ref_pos"]).reshape(-1, 3)
    extent = float(np.max(ref.max(axis=0) - ref.min(axis=0)))
    du = float(np.abs(np.asarray(gpu["u"], np.float64) - cpu64["u"]).max())
    dv = float(np.abs(np.asarray(gpu["v"], np.float64) - cpu64["v"]).max())
    vmax = float(np.abs(cpu64["v"]).max())
    rel = lambda a, b: abs(a - b) / max(abs(b), 1e-300)  # noqa: E731
    return {"max_position_error_over_extent": du / extent,
            "max_velocity_error_over_max_speed": dv / vmax if vmax > 0 else dv,
            "removed_energy_rel_error": rel(float(gpu["status_f64"][0]), float(cpu64["status_f64"][0])),
            "plastic_work_rel_error": rel(float(gpu["status_f64"][2]), float(cpu64["status_f64"][2])),
            "broken_bonds_fp32": int(gpu["status_u64"][4]), "broken_bonds_fp64": int(cpu64["status_u64"][4]),
            "broken_state_differs": int(np.count_nonzero(np.asarray(gpu["alive"]) != cpu64["alive"])),
            "substeps": int(cpu64["status_u64"][0])}


def port_rate(out: dict, skip: int = 1) -> tuple[float, float]:
    """The restatement's projections per second over its substeps after the
    first `skip` (by default the post-upload restart), from its per-substep
    wall times and exact per-substep projection counts; and the seconds
    timed."""
    secs = np.asarray(out["substep_seconds"], np.float64)[skip:]
    proj = np.asarray(out["substep_projections"], np.float64)[skip:]
    return float(np.sum(proj)) / float(np.sum(secs)), float(np.sum(secs))


# ---------------------------------------------------------------------------
# The impact (main line)
# ---------------------------------------------------------------------------
def impact_parity(args, lattice, case) -> tuple[dict, dict, dict]:
    """Parity prefix, FP64 error prefix and the CPU baseline taken from the
    parity run of the restatement."""
    import oracle

    threads = host_threads()
    p_sub = args.parity_steps * SUBSTEPS_PER_STEP
    t0 = time.perf_counter()
    cpu = oracle.run_port(prefix(case, p_sub), threads=threads, per_substep=True)
    cpu_s = time.perf_counter() - t0
    gpu = lattice.run_case(prefix(case, p_sub), per_substep=True)
    parity = parity_report(cpu, gpu, break_step=True)
    parity.update(steps=args.parity_steps, threads=threads, cpu_wall_s=cpu_s,
                  note="the first steps of the benchmarked lattice, impact inside; device run one substep per call "
                       "to record the substep each bond broke")
    rate, timed = port_rate(cpu)
    baseline = {"value": rate, "unit": METRIC, "cores": threads, "kind": "port",
                "sample": f"substeps 2-{p_sub} of the parity prefix of the same lattice (the first, post-upload "
                          f"restart substep left out), {threads} host threads, {timed:.1f} s timed; "
                          "the restatement's threaded lane runs within 1.15x of the reference's threaded lane at "
                          "equal threads (calibration test tests/test_port_speed.py)"}
    del cpu, gpu
    gc.collect()
    fp = None
    if args.fp64_steps > 0:
        # The FP64 run is the device's double lane (direct arithmetic), which
        # the restatement's double lane and the reference's double fixtures
        # hold bit for bit (tests/test_gpu_parity.py, test_gpu_edges.py): at
        # this size the restatement in double would need more host memory
        # than the benchmark may take.
        f_sub = args.fp64_steps * SUBSTEPS_PER_STEP
        gpu32 = lattice.run_case(prefix(case, f_sub))
        gpu64 = lattice.run_case(prefix(case, f_sub), precision="double")
        fp = dict(fp64_error(case, gpu32, gpu64), steps=args.fp64_steps,
                  note="device FP32 against the device's FP64 lane (direct arithmetic, bit-identical to the "
                       "restatement's FP64 lane), same case and substeps")
        del gpu32, gpu64
        gc.collect()
    return parity, fp, baseline


def run_gb300(args) -> None:
    rank, world, local, dist, torch = distributed()
    from banjo_gb300 import build as lib_build
    from banjo_gb300 import lattice

    lib_build.build()
    case, desc = make_case(args.workload)
    n, b = int(case["node_count"][0]), int(case["bond_count"][0])
    sched = lattice.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = lattice.build_lattice_state(case, sched)
    # The caller's state for the e2e run, built up front as a caller's would
    # be, before the main lattice's memory is freed and reused. The upload
    # copies it through page-locked staging slices on the host's threads.
    e2e_state = lattice.build_lattice_state(case, sched)
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
    projections = st.bond_projections - before.bond_projections
    device_s_max = max_over_ranks(device_s, dist, torch)
    total_proj = sum_over_ranks(float(projections), dist, torch)
    clocks = sampler.summary()

    # Roofline of the projection sweep: event-timed phases of a few substeps
    # after the timed region, counted on the bonds alive in them.
    p0 = backend.status()
    phases = backend.profile_phases(args.profile_substeps)
    p1 = backend.status()
    live_prof = (p1.bond_projections - p0.bond_projections) / (ITERATIONS * args.profile_substeps)
    sweep_ms = (phases["sweep_interior"] + phases["sweep_boundary"]) / args.profile_substeps
    peak, peak_kind = peaks()
    algo = sweep_bytes(n, live_prof)
    achieved = algo / (sweep_ms * 1e-3) / 1e9
    achieved_all = sweep_bytes(n, b) / (sweep_ms * 1e-3) / 1e9
    # DRAM bytes of one substep's sweep (its 116 level launches), from ncu
    # (dram__bytes_read.sum + dram__bytes_write.sum) on the impact at 128x64x64
    # (4,616,704 bonds) and scaled by bonds: traffic grows with the records
    # streamed.
    traffic = args.sweep_traffic_per_bond * b if args.workload.startswith("impact") else None

    d = max(1, state.view.max_degree)
    del backend, state  # host and device memory for the e2e lattice
    gc.collect()
    # e2e: through the C ABI from host buffers (upload, K steps, download).
    e2e_backend = lattice.make_gb300_lattice_backend(sched)
    t0 = time.perf_counter()
    e2e_backend.upload(e2e_state, settings, sphere)
    if "forces" in case:
        e2e_backend.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    t1 = time.perf_counter()
    e2e_st = e2e_backend.run(lattice.RunControl(max_steps=substeps_k))
    t2 = time.perf_counter()
    e2e_backend.download(e2e_state)
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"upload_s": t1 - t0, "run_s": t2 - t1, "download_s": e2e_s - (t2 - t0)}
    e2e_s_max = max_over_ranks(e2e_s, dist, torch)
    e2e_total = sum_over_ranks(float(e2e_st.bond_projections), dist, torch)
    # Bytes copied: upload takes the state's own arrays as they are (the device
    # converts them) -- 14 doubles per node; per neighbour slot the rest
    # vector, weight, alive flag, other node and bond; per bond 19 arrays
    # (ends, slots, flags, rest data, thresholds, damage state) and the
    # storage order -- and download returns u, u_prev, v and 8 bond arrays.
    h2d = n * 14 * 8 + n * d * 41 + b * (164 + 4)
    d2h = n * 3 * 24 + b * (2 + 6 * 8)
    del e2e_backend, e2e_state, sched
    gc.collect()

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
                   "timed_substeps": f"{substeps_w}-{substeps_w + substeps_k}",
                   "broken_in_window": st.broken_bonds - before.broken_bonds,
                   "live_bonds_end": b - st.broken_bonds},
        "e2e": {"value": e2e_total / e2e_s_max, "unit": "projections/s", "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps,
                "note": "one upload of the host LatticeState (converted on the device), K steps from upload, one "
                        "download; wall clock", **e2e_parts},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_per": "substep sweep (bytes)",
                     "algorithmic_bytes_per_substep_sweep": algo, "peak_kind": peak_kind,
                     "kernel": "kSolve (projection sweep)", "sweep_ms_per_substep": sweep_ms,
                     "live_bonds_profiled": live_prof,
                     "achieved_all_records": achieved_all, "frac_all_records": achieved_all / peak,
                     "note": "algorithmic bytes count live bonds only; the all-records figure counts every record "
                             "the sweep streams, dead ones included"},
        "bond_updates_per_s": {"device": world * b * substeps_k / device_s_max,
                               "e2e": world * b * substeps_k / e2e_s_max},
        "gpu_launches": launches * substeps_k,
        "clocks": clocks,
        "host_seconds": host_s,
        "phase_ms_per_substep": {k: v / args.profile_substeps for k, v in phases.items() if v > 0},
    }
    if rank == 0 and args.parity_steps > 0:
        parity, fp, baseline = impact_parity(args, lattice, case)
        line["parity"] = parity
        if fp is not None:
            line["fp64_error"] = fp
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = baseline
    del case
    legs = [("cantilever", args.cantilever, cantilever_leg), ("batched", args.trials > 0, batched_leg),
            ("served", args.served_points > 0 or args.stress_window > 0, served_leg),
            ("cascade", args.cascade_steps > 0, cascade_leg)]
    for name, on, fn in legs:
        if on and name not in args.skip:
            if name == "served":
                line[name] = fn(args, lattice, line.get("batched"))
            else:
                line[name] = fn(args, lattice)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# The cantilever
# ---------------------------------------------------------------------------
def cantilever_leg(args, lattice) -> dict:
    import oracle
    from banjo_gb300 import scenes

    case = scenes.cantilever()
    n, b = int(case["node_count"][0]), int(case["bond_count"][0])
    total = int(case["steps"][0])
    sched = lattice.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = lattice.build_lattice_state(case, sched)
    settings = lattice.step_settings(case["settings"])
    be = lattice.make_gb300_lattice_backend(sched)
    t0 = time.perf_counter()
    be.upload(state, settings, lattice.sphere_state(case["sphere"]))
    be.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    st = be.run(lattice.RunControl(max_steps=total))
    be.download(state)
    e2e_s = time.perf_counter() - t0
    phases = be.profile_phases(3)
    gpu = lattice.run_case(case)
    threads = host_threads()
    cpu = oracle.run_port(case, threads=threads)
    cpu1 = oracle.run_port(case, threads=1)
    cpu64 = oracle.run_port(case, precision="double", threads=1)
    rate1, _ = port_rate(cpu1, skip=0)
    rate, _ = port_rate(cpu, skip=0)
    ledger_ms = phases.get("sphere_exit", 0.0) / 3
    # Before the first failure the two lanes integrate the same loaded beam;
    # after it they are different trajectories of a fracture.
    first = int(cpu["status_u64"][1])
    pre = prefix(case, first)
    pre_err = dict(fp64_error(pre, lattice.run_case(pre), oracle.run_port(pre, precision="double", threads=1)),
                   note=f"the first {first} substeps, up to the first failure")
    return {"value": st.bond_projections / st.kernel_seconds, "unit": "projections/s", "nodes": n, "bonds": b,
            "substeps": total, "ms_per_substep": st.kernel_seconds / total * 1e3,
            "e2e": {"value": st.bond_projections / e2e_s, "unit": "projections/s", "wall_s": e2e_s},
            "parity": parity_report(cpu, gpu, break_step=False),
            "fp64_error": dict(fp64_error(case, gpu, cpu64), note="whole run, device FP32 vs restatement FP64; "
                               "after the first failure the two runs break different bonds and the pieces fly "
                               "apart differently"),
            "fp64_error_before_failure": pre_err,
            "cpu_baseline": {"value": max(rate, rate1), "unit": METRIC, "cores": threads if rate >= rate1 else 1,
                             "kind": "port",
                             "sample": f"the whole run ({total} substeps); the serial lane ({rate1:.3g}/s) and the "
                                       f"{threads}-thread lane ({rate:.3g}/s) both timed, the faster reported"},
            "phase_ms_per_substep": {k: v / 3 for k, v in phases.items() if v > 0},
            "ledger_ms_per_substep": ledger_ms,
            "workload": "cantilever 32x8x8 (2048 nodes, 15648 bonds), x=0 face pinned, end load, 240 steps x 10 "
                        "substeps from upload; device time of the whole run"}


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


def trial_case(spec, substeps: int) -> dict:
    """The same trial as a scene case (the generator the box builder is held
    to bit for bit), for the CPU restatement."""
    from banjo_gb300 import scenes

    nx, ny, nz, comp, strain, height = spec
    case = scenes.drop_trial(nx, ny, nz, compliance=comp, break_strain=strain, drop_height=height, steps=1,
                             substeps=1)
    case["steps"] = np.array([substeps], dtype=np.uint64)
    return case


def trial_settings(lattice):
    from banjo_gb300 import scenes

    return lattice.step_settings(scenes.settings(planes=[scenes.plane((0.0, 0.0, 0.0),
                                                                      node_radius=0.5 * TRIAL_SPACING)]))


def trial_cpu_baseline(specs, substeps: int = 2) -> dict:
    """The CPU restatement with trial-level parallelism: one serial lane per
    host thread, each running whole trials of the same draw one after another
    (the stronger CPU arrangement for many small lattices). Each trial's first
    (restart) substep is left out; the rate is every timed projection over the
    timed seconds shared by the threads."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    threads = host_threads()

    def one(spec):
        out = oracle.run_port(trial_case(spec, substeps + 1), threads=1)
        secs = float(np.sum(out["substep_seconds"][1:]))
        return float(np.sum(out["substep_projections"][1:])), secs

    with ThreadPoolExecutor(threads) as ex:
        results = list(ex.map(one, specs))
    proj = sum(p for p, _ in results)
    secs = sum(t for _, t in results)
    return {"value": proj / (secs / threads), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(specs)} trials of the same draw, {substeps} substeps each after the restart, one "
                      f"serial lane per thread on {threads} threads; {secs:.1f} thread-seconds timed"}


class ScratchDownload:
    """Download targets for lattices of any size up to a bound, sharing one
    set of host arrays: a view with a lattice's counts whose pointers lead
    into the shared arrays (download writes positions, velocities and the
    bond state, nothing else). Keeps a 4096-trial batch's downloads from
    holding every trial's state in host memory at once."""

    def __init__(self, lattice, max_nodes: int, max_bonds: int):
        import ctypes as C

        self._C = C
        self.lattice = lattice
        self.nodes3 = [np.zeros(3 * max_nodes) for _ in range(3)]
        self.bytes = [np.zeros(max_bonds, np.uint8) for _ in range(2)]
        self.doubles = [np.zeros(max_bonds) for _ in range(6)]
        self.view = lattice.StateView()

    def target(self, nodes: int, bonds: int, degree: int):
        C = self._C
        v = self.view
        v.node_count, v.bond_count, v.max_degree = nodes, bonds, degree
        f64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        u8 = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint8))  # noqa: E731
        v.u, v.u_prev, v.v = (f64(a) for a in self.nodes3)
        v.alive, v.failure_mode = (u8(a) for a in self.bytes)
        (v.damage, v.prev_tensile, v.prev_compressive, v.prev_shear, v.plastic_extension,
         v.plastic_strain) = (f64(a) for a in self.doubles)
        return self


def batched_leg(args, lattice) -> dict:
    """Drop trials in one batch against the same trials run one lattice at
    a time through the single-lattice backend ("plain")."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    specs = trial_specs(args.trials)
    settings = trial_settings(lattice)
    # Parity sample: 8 seeded members, the largest among them.
    rng = np.random.default_rng(17)
    largest = int(np.argmax([nx * ny * nz for nx, ny, nz, *_ in specs]))
    sample = sorted({largest, *[int(x) for x in rng.choice(len(specs), size=7, replace=False)]})[:8]
    keep = {}
    batch = lattice.Batch()
    t_start = time.perf_counter()

    def make(i):
        # Built and added on host threads; only the sample's states are kept.
        sched, state = build_trial(lattice, specs[i])
        k = batch.add(sched, state, lattice.Sphere())
        if i in sample:
            keep[i] = state
        return k, state.node_count, state.bond_count, state.view.max_degree

    with ThreadPoolExecutor(host_threads()) as ex:
        added = list(ex.map(make, range(len(specs))))
    index_of = [a[0] for a in added]
    counts = [a[1:] for a in added]
    batch.settle(settings)
    upload_s = time.perf_counter() - t_start
    tuning = None
    if not args.no_tune:
        # The autotuner: sweep launch shapes timed on these lattices (state unchanged).
        t0 = time.perf_counter()
        tuning = batch.tune()
        tuning["tune_s"] = time.perf_counter() - t0
    nodes = sum(c[0] for c in counts)
    bonds = sum(c[1] for c in counts)
    w, k = args.warmup * SUBSTEPS_PER_STEP, args.steps * SUBSTEPS_PER_STEP
    t0 = time.perf_counter()
    batch.run(lattice.RunControl(max_steps=w))
    before = [batch.status(i) for i in range(len(specs))]
    batch.run(lattice.RunControl(max_steps=k))
    run_wall = time.perf_counter() - t0
    after = [batch.status(i) for i in range(len(specs))]
    device_s = after[0].kernel_seconds - before[0].kernel_seconds
    proj = sum(a.bond_projections - p.bond_projections for a, p in zip(after, before))
    proj_all = sum(a.bond_projections for a in after)
    value = proj / device_s
    launches = batch.kernels_per_substep()

    # Download of every trial (the sample into their own states, the rest
    # into shared scratch arrays), then the sample against the restatement
    # run from upload over the same W + K substeps.
    scratch = ScratchDownload(lattice, max(c[0] for c in counts), max(c[1] for c in counts))
    outs = {}
    t0 = time.perf_counter()
    for i in range(len(specs)):
        if i in keep:
            sp = batch.download(index_of[i], keep[i])
            outs[i] = lattice.state_outputs(keep[i], sp, batch.first_failure_bonds(index_of[i]),
                                            batch.status(index_of[i]))
        else:
            batch.download(index_of[i], scratch.target(*counts[i]))
    download_s = time.perf_counter() - t0
    e2e_s = upload_s + run_wall + download_s
    parity, fp = {}, {}
    threads = host_threads()
    for i in sample:
        case = trial_case(specs[i], w + k)
        cpu = oracle.run_port(case, threads=threads)
        rep = parity_report(cpu, outs[i], break_step=False)
        parity[str(i)] = {"ok": rep["ok"], "bonds": counts[i][1], "state_mismatches": rep["state_mismatches"],
                          "status_mismatches": rep["status_mismatches"], "ledgers_within": rep["ledgers"]["within"]}
        if args.fp64_steps > 0:
            cpu64 = oracle.run_port(case, precision="double", threads=threads)
            fp[str(i)] = fp64_error(case, outs[i], cpu64)
    del outs, keep, scratch
    gc.collect()
    phases = batch.profile_phases(1)
    sweep_ms = phases["sweep_interior"] + phases["sweep_boundary"]
    live_now = sum(c[1] - a.broken_bonds for c, a in zip(counts, after))
    algo = sum(sweep_bytes(c[0], 0) for c in counts) + ITERATIONS * 40 * live_now
    peak, peak_kind = peaks()
    del batch
    gc.collect()

    # Plain: the first trials of the same draw, one backend at a time; device
    # time, and through the API (backend creation, upload, W + K steps,
    # download) on the host clock.
    plain_n = min(args.plain_trials, len(specs))
    plain_proj, plain_s, plain_wall, plain_api_proj = 0.0, 0.0, 0.0, 0.0
    for spec in specs[:plain_n]:
        sched, state = build_trial(lattice, spec)
        t0 = time.perf_counter()
        be = lattice.make_gb300_lattice_backend(sched)
        be.upload(state, settings, lattice.Sphere())
        be.run(lattice.RunControl(max_steps=w))
        st0 = be.status()
        st1 = be.run(lattice.RunControl(max_steps=k))
        be.download(state)
        plain_wall += time.perf_counter() - t0
        plain_s += st1.kernel_seconds - st0.kernel_seconds
        plain_proj += st1.bond_projections - st0.bond_projections
        plain_api_proj += st1.bond_projections
        del be
    plain = plain_proj / plain_s
    plain_e2e = plain_api_proj / plain_wall
    batch_e2e = proj_all / e2e_s
    cpu = None if args.no_cpu_baseline else trial_cpu_baseline(specs[:args.cpu_trials])
    return {"value": value, "unit": "projections/s", "trials": len(specs), "nodes": nodes, "bonds": bonds,
            "cpu_baseline": cpu,
            "ms_per_step": device_s / args.steps * 1e3, "gpu_launches_per_substep": launches,
            "host_threads": host_threads(),
            "e2e": {"value": batch_e2e, "unit": "projections/s", "wall_s": e2e_s,
                    "build_and_upload_s": upload_s, "run_s": run_wall, "download_s": download_s,
                    "note": "every trial built by the box builder and added on host threads (upload), W + K "
                            "steps, every trial downloaded; all projections over that wall time"},
            "plain": {"value": plain, "unit": "projections/s", "trials": plain_n,
                      "e2e": plain_e2e,
                      "note": "the first trials of the same draw, each alone through the single-lattice backend "
                              "(its own captured substep graph); device time of K steps, and the API wall time of "
                              "backend creation, upload, W + K steps and download (e2e)"},
            "speedup_vs_plain": value / plain, "e2e_speedup_vs_plain": batch_e2e / plain_e2e,
            "roofline": {"bound": "hbm", "achieved": algo / (sweep_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (sweep_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                         "kernel": "kSweepLattice + kSolve (the batch's projection sweep)",
                         "sweep_ms_per_substep": sweep_ms, "algorithmic_bytes_per_substep_sweep": algo},
            "parity": {"ok": all(v["ok"] for v in parity.values()), "members": parity,
                       "substeps": w + k, "largest_member_bonds": counts[largest][1],
                       "note": "8 seeded members (the largest included) after the timed window against the CPU "
                               "restatement run from upload over the same substeps"},
            "fp64_error": {"members": fp, "max_position_error_over_extent":
                           max((v["max_position_error_over_extent"] for v in fp.values()), default=None)},
            "tuning": tuning,
            "phase_ms_per_substep": {name: v for name, v in phases.items() if v > 0},
            "workload": f"{len(specs)} drop trials, edges 8..48 per axis (seeded), one batch; step = "
                        f"{SUBSTEPS_PER_STEP} substeps, I={ITERATIONS}; device time of {args.steps} steps"}


# ---------------------------------------------------------------------------
# Served requests
# ---------------------------------------------------------------------------
class ServedRun:
    """One arrival process against a fresh server: clients submit each
    request at its scheduled arrival from host threads, the serving loop
    steps the server and collects finished requests."""

    def __init__(self, lattice, settings, budget, picks, arrivals, horizon, chunk, copy, keep=()):
        self.lattice = lattice
        self.server = lattice.Server(settings, budget)
        self.picks = picks
        self.arrivals = arrivals
        self.horizon = horizon
        self.chunk = chunk
        self.copy = copy
        self.keep = set(keep)  # requests whose results are kept for the parity check
        self.results = {}

    def run(self) -> dict:
        from concurrent.futures import ThreadPoolExecutor

        lattice = self.lattice
        server = self.server
        count = len(self.arrivals)
        tickets = [None] * count
        sphere = lattice.Sphere()
        clients = ThreadPoolExecutor(max(1, host_threads() - 2))
        start = time.perf_counter()

        def submit(i):
            sched, state, _ = self.picks[i]
            # Copied: the request's device image is prepared on the client's
            # thread, so admission is a copy; borrowed: the caller's arrays
            # are copied as they are and converted on the device at admission.
            tickets[i] = server.submit(sched, state, sphere, self.horizon, borrow=not self.copy and i not in self.keep)

        def produce():
            for i, t in enumerate(self.arrivals):
                delay = start + float(t) - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                clients.submit(submit, i)
            clients.shutdown(wait=True)

        producer = threading.Thread(target=produce)
        producer.start()
        done, latency, wait, service, proj = set(), {}, {}, {}, 0
        while len(done) < count:
            st = server.step(self.chunk)
            if st.running == 0 and st.queued == 0:
                time.sleep(0.0005)  # nothing admitted: wait for the next arrival
            for i, t in enumerate(tickets):
                if t is None or i in done:
                    continue
                info = server.poll(t)
                if info.phase == lattice.REQUEST_DONE:
                    finished = time.perf_counter() - start
                    out_state = None
                    if i in self.keep:
                        out_state = self.picks[i][2]()
                    sp, rs = server.take(t, out_state)
                    if i in self.keep:
                        self.results[i] = lattice.state_outputs(out_state, sp, np.zeros(0, np.uint32), rs)
                    latency[i] = finished - float(self.arrivals[i])
                    wait[i] = info.admitted_s - info.submitted_s
                    service[i] = info.finished_s - info.admitted_s
                    proj += rs.bond_projections
                    done.add(i)
        producer.join()
        wall = time.perf_counter() - start
        stats = server.stats()
        lat = np.array([latency[i] for i in range(count)])
        wq = np.array([wait[i] for i in range(count)])
        sv = np.array([service[i] for i in range(count)])
        return {"requests": count, "value": proj / wall, "unit": "projections/s",
                "completed_per_s": count / wall,
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "p50_admission_wait_s": float(np.percentile(wq, 50)),
                "p99_admission_wait_s": float(np.percentile(wq, 99)),
                "p50_service_s": float(np.percentile(sv, 50)), "p99_service_s": float(np.percentile(sv, 99)),
                "wall_s": wall, "device_s": stats.device_seconds, "device_busy": stats.device_seconds / wall,
                "admit_s": stats.admit_seconds, "admit_share_of_wall": stats.admit_seconds / wall,
                "retire_s": stats.retire_seconds, "run_s": stats.run_seconds}


def served_leg(args, lattice, batched: dict | None) -> dict:
    """Served requests: Poisson arrivals of 90% drop trials and 10% 128^3
    lattices, 2400 substeps each, admitted against an HBM budget and stepped
    together; a load sweep at fractions of the batched capacity."""
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(11)
    small = trial_specs(args.served_pool)
    large = [(128, 128, 128, s[3], s[4], s[5]) for s in trial_specs(2, seed=5)]
    specs = small + large

    def make(spec):
        sched, state = build_trial(lattice, spec)
        return sched, state, (lambda sp=spec: build_trial(lattice, sp)[1])

    with ThreadPoolExecutor(host_threads()) as ex:
        pool = list(ex.map(make, specs))
    settings = trial_settings(lattice)
    budget = int(args.served_budget_gb * (1 << 30))
    horizon = args.served_substeps
    bonds_small = float(np.mean([pool[i][1].bond_count for i in range(len(small))]))
    bonds_large = float(np.mean([pool[len(small) + j][1].bond_count for j in range(len(large))]))
    mean_proj = ITERATIONS * horizon * (0.9 * bonds_small + 0.1 * bonds_large)
    capacity_proj = batched["value"] if batched else args.served_capacity
    capacity = capacity_proj / mean_proj  # requests/s the batched rate carries
    out = {"substeps_per_request": horizon, "budget_gb": args.served_budget_gb,
           "mean_request_projections": mean_proj,
           "capacity_requests_per_s": capacity,
           "capacity_note": "the batched leg's device rate over the mean request's projections (no breakage)",
           "submission": "copied (device image prepared on client threads)" if args.served_copy else
           "borrowed (converted on the device at admission)"}

    def draw(count):
        kinds = rng.random(count) < 0.1
        return [len(small) + int(rng.integers(len(large))) if big else int(rng.integers(len(small)))
                for big in kinds]

    points = []
    parity_done = False
    for frac in (0.5, 0.8, 0.95)[:args.served_points]:
        rate = frac * capacity
        count = args.served_completions
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
        which = draw(count)
        keep = ()
        if not parity_done and args.served_parity > 0:
            # The parity sample: seeded requests of this point, one large among them.
            big = [i for i, w in enumerate(which) if w >= len(small)]
            if not big:
                which[0] = len(small)
                big = [0]
            rest = [i for i in range(count) if i not in big[:1]]
            keep = sorted([big[0], *[int(x) for x in rng.choice(rest, size=args.served_parity - 1, replace=False)]])
        run = ServedRun(lattice, settings, budget, [pool[w] for w in which], arrivals, horizon, args.served_chunk,
                        args.served_copy, keep=keep)
        res = run.run()
        res.update(load_fraction=frac, offered_requests_per_s=rate,
                   large_requests=int(sum(w >= len(small) for w in which)))
        points.append(res)
        if keep:
            picks = [pool[which[i]] for i in keep]
            out["parity"] = served_parity(lattice, settings, picks, run.results, keep, horizon)
            if args.fp64_steps > 0:
                out["fp64_error"] = served_fp64(lattice, settings, picks, run.results, keep, horizon)
            parity_done = True
    out["load_sweep"] = points
    if points:
        out["value"] = points[-1]["value"]
        out["unit"] = "projections/s"
        out["p50_latency_s"] = points[-1]["p50_latency_s"]
        out["p99_latency_s"] = points[-1]["p99_latency_s"]
    if args.stress_window > 0:
        arrivals = np.cumsum(rng.exponential(1.0 / args.stress_rate, size=int(args.stress_rate * args.stress_window * 3)))
        arrivals = arrivals[arrivals < args.stress_window]
        which = draw(arrivals.size)
        run = ServedRun(lattice, settings, budget, [pool[w] for w in which], arrivals, args.stress_substeps,
                        args.served_chunk, args.served_copy)
        res = run.run()
        res.update(label="stress: arrivals far above capacity; latency here is queueing",
                   offered_requests_per_s=args.stress_rate, window_s=args.stress_window,
                   substeps_per_request=args.stress_substeps)
        out["stress"] = res
    out["workload"] = (f"Poisson arrivals of {args.served_completions} requests per point at 50/80/95% of the "
                       f"batched capacity; 90% drawn from {len(small)} drop trials, 10% 128^3 lattices; "
                       f"{horizon} substeps each; latency = finish observed by the client - scheduled arrival")
    return out


def served_parity(lattice, settings, picks, results, keep, horizon) -> dict:
    """Each kept request's served result against the same lattice run alone
    through the single-lattice backend for the same substeps."""
    from oracle.compare import STATE_KEYS, mismatches, status_mismatches

    members = {}
    for (sched, state, fresh), i in zip(picks, keep):
        be = lattice.make_gb300_lattice_backend(sched)
        be.upload(state, settings, lattice.Sphere())
        st = be.run(lattice.RunControl(max_steps=horizon))
        alone_state = fresh()
        sp = be.download(alone_state)
        alone = lattice.state_outputs(alone_state, sp, np.zeros(0, np.uint32), st)
        served = results[i]
        bad = mismatches(alone, served, [k for k in STATE_KEYS if k != "first_failure_bonds"])
        bad_status = status_mismatches(alone, served)
        members[str(i)] = {"ok": not bad and not bad_status, "bonds": state.bond_count,
                           "state_mismatches": bad, "status_mismatches": bad_status,
                           "broken_bonds": int(st.broken_bonds)}
        del be
    return {"ok": all(m["ok"] for m in members.values()), "members": members,
            "largest_member_bonds": max(m["bonds"] for m in members.values()),
            "note": "seeded requests of the first load point (one 128^3 among them), bit for bit against the same "
                    "request run alone"}


def served_fp64(lattice, settings, picks, results, keep, horizon, members: int = 4) -> dict:
    """The FP32 served results of the smallest kept requests against the
    device's FP64 lane (direct arithmetic, which the restatement's FP64 lane
    holds bit for bit) on the same requests alone: over the whole horizon,
    and over the substeps before the request's first bond failure (after it
    the two precisions are different trajectories of a chaotic process)."""
    s64 = type(settings).from_buffer_copy(settings)
    s64.direct_arithmetic = 1

    def alone(sched, state, fresh, s, precision, substeps):
        be = lattice.make_gb300_lattice_backend(sched, precision)
        be.upload(state, s, lattice.Sphere())
        st = be.run(lattice.RunControl(max_steps=substeps))
        out = fresh()
        sp = be.download(out)
        del be
        return lattice.state_outputs(out, sp, np.zeros(0, np.uint32), st)

    order = sorted(range(len(keep)), key=lambda q: picks[q][1].bond_count)[:members]
    fp = {}
    for q in order:
        sched, state, fresh = picks[q]
        ref = {"ref_pos": np.asarray(state.x0, np.float64)}
        served = results[keep[q]]
        row = dict(fp64_error(ref, served, alone(sched, state, fresh, s64, "double", horizon)),
                   bonds=state.bond_count)
        first = int(served["status_u64"][1])
        if 0 < first < horizon:
            row["before_failure"] = fp64_error(ref, alone(sched, state, fresh, settings, "float", first),
                                               alone(sched, state, fresh, s64, "double", first))
        fp[str(keep[q])] = row
    pre = [v["before_failure"]["max_position_error_over_extent"] for v in fp.values() if "before_failure" in v]
    return {"members": fp,
            "max_position_error_over_extent": max((v["max_position_error_over_extent"] for v in fp.values()),
                                                  default=None),
            "max_position_error_over_extent_before_failure": max(pre, default=None),
            "note": f"the {len(fp)} smallest requests of the parity sample, served FP32 against the device's FP64 "
                    f"lane on the same request alone, over {horizon} substeps and up to the first bond failure"}


# ---------------------------------------------------------------------------
# The notched bar
# ---------------------------------------------------------------------------
def cascade_leg(args, lattice) -> dict:
    """The notched bar (energy-scaled law, plastic flow, horizon 2) under its
    ramped end load on the device, with parity and FP64 error over its first
    steps. The full 10,000-step horizon is held to the reference's own run by
    tests/test_gpu_cascade_long.py."""
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
    device_s = 0.0
    for step in range(args.cascade_steps):
        scale = float(case["force_ramp_scale"][0]) * step / float(case["force_ramp_steps"][0])
        be.set_external_forces(scale * base, per)
        before = be.status()
        st = be.run(lattice.RunControl(max_steps=per))
        device_s += st.kernel_seconds - before.kernel_seconds
    phases = be.profile_phases(3)
    out = {"value": st.bond_projections / device_s, "unit": "projections/s", "nodes": n, "bonds": b,
           "steps": args.cascade_steps, "broken_bonds": int(st.broken_bonds),
           "removed_energy_j": st.removed_energy_j, "plastic_work_j": st.plastic_work_j,
           "max_plastic_stretch": st.max_plastic_stretch,
           "phase_ms_per_substep": {k: v / 3 for k, v in phases.items() if v > 0},
           "workload": f"notched bar 128x32x32 (slot at mid-length, lower half), horizon 2, energy-scaled law + "
                       f"plastic flow compiled in FP64; end load ramped 0 -> 2x(45 MPa x 0.1024 m^2) over 10000 "
                       f"steps, the first {args.cascade_steps} steps run; device time"}
    if args.cascade_check_steps > 0:
        short = scenes.notched_bar(steps=args.cascade_check_steps)
        gpu = lattice.run_case(short)
        threads = host_threads()
        cpu = oracle.run_port(short, threads=threads)
        out["parity"] = dict(parity_report(cpu, gpu, break_step=False), steps=args.cascade_check_steps)
        cpu64 = oracle.run_port(short, precision="double", threads=threads)
        out["fp64_error"] = dict(fp64_error(short, gpu, cpu64), steps=args.cascade_check_steps,
                                 note="device FP32 vs the CPU restatement in FP64 (direct arithmetic), same case")
        out["cpu_baseline"] = {"value": port_rate(cpu, skip=0)[0], "unit": METRIC, "cores": threads, "kind": "port",
                               "sample": f"the parity run: {args.cascade_check_steps} ramp steps, {threads} threads"}
    return out


# ---------------------------------------------------------------------------
# Ranks
# ---------------------------------------------------------------------------
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


def _reduce_device(dist) -> str:
    # NCCL reduces device tensors; gloo (the CPU tests of this logic) host ones.
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier(dist, torch):
    if dist is not None:
        dist.barrier()
        if torch.cuda.is_available():
            torch.cuda.synchronize()


def max_over_ranks(x: float, dist, torch) -> float:
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, dist, torch) -> float:
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args) -> None:
    """The reference's CPU lane on the GPU arm's workload and window: the
    restatement (the reference tree is absent on the GPU machine) on all host
    threads, the substeps of the K timed steps after the W warm-up steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    oracle.build_port()
    case, desc = make_case(args.workload)
    threads = host_threads()
    w, k = args.warmup * SUBSTEPS_PER_STEP, args.steps * SUBSTEPS_PER_STEP
    out = oracle.run_port(prefix(case, w + k), threads=threads)
    value, timed = port_rate(out, skip=w)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "projections/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": timed / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (f64 ledgers)",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": desc, "substeps_per_step": SUBSTEPS_PER_STEP, "iterations": ITERATIONS,
                   "timed_substeps": f"{w}-{w + k}", "same_config": True},
        "cpu_baseline": {"value": value, "unit": "projections/s", "cores": threads, "kind": "port",
                         "sample": f"substeps {w}-{w + k} (the GPU arm's timed window) of the same lattice, {threads} "
                                   "threads; the reference tree is absent here, so its CPU lane runs as the "
                                   "restatement, whose threaded lane is held within 1.15x of the reference's"},
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
    p.add_argument("--sweep-traffic-per-bond", type=float, default=759.26e6 / 4616704.0,
                   help="ncu DRAM bytes of one substep's sweep per bond (impact 128x64x64)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--parity-steps", type=int, default=5, help="impact: steps of the parity prefix (0: skip)")
    p.add_argument("--fp64-steps", type=int, default=2, help="impact and batch: steps of the FP64 error check")
    p.add_argument("--skip", nargs="*", default=[], choices=["cantilever", "batched", "served", "cascade"])
    p.add_argument("--cantilever", type=int, default=1, help="cantilever leg (0: skip)")
    p.add_argument("--trials", type=int, default=4096, help="batched leg: trials in one batch (0: skip)")
    p.add_argument("--plain-trials", type=int, default=64, help="batched leg: trials timed one at a time")
    p.add_argument("--no-tune", action="store_true", help="batched leg: keep the default launch shapes")
    p.add_argument("--cpu-trials", type=int, default=96,
                   help="batched leg: trials in the trial-parallel CPU baseline sample")
    p.add_argument("--served-copy", type=int, default=1,
                   help="served leg: 1 submits copied states (device image prepared on client threads), 0 borrowed")
    p.add_argument("--served-points", type=int, default=3, help="served leg: load points of 50/80/95%% (0: none)")
    p.add_argument("--served-completions", type=int, default=200, help="served leg: requests per load point")
    p.add_argument("--served-substeps", type=int, default=2400)
    p.add_argument("--served-chunk", type=int, default=10)
    p.add_argument("--served-pool", type=int, default=256)
    p.add_argument("--served-budget-gb", type=float, default=80.0)
    p.add_argument("--served-parity", type=int, default=16, help="served leg: requests checked against alone runs")
    p.add_argument("--served-capacity", type=float, default=3.5e10,
                   help="served leg: projections/s taken as the batched capacity when the batched leg is skipped")
    p.add_argument("--stress-rate", type=float, default=2000.0)
    p.add_argument("--stress-window", type=float, default=0.25, help="served stress point: seconds of arrivals")
    p.add_argument("--stress-substeps", type=int, default=40)
    p.add_argument("--cascade-steps", type=int, default=200, help="notched-bar leg: ramp steps run (0: skip)")
    p.add_argument("--cascade-check-steps", type=int, default=10,
                   help="notched-bar leg: steps of the parity and FP64 checks")
    args = p.parse_args()
    if args.warmup < 3:
        raise SystemExit("warm-up must be at least 3 steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
