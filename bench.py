#!/usr/bin/env python
"""Throughput of the per-step physics path on GB300: particle-steps/s.

Workload (--n, default 1,000,000): a differentiated Earth-Theia-like impact,
800k-particle target + 200k impactor, Iron core 30 % of mass + Granite
mantle, radial density from a 1-D hydrostatic integration, mass ratio 0.1,
1.1 v_esc at 45 degrees, strength and damage on, plain Barnes-Hut at
theta = 0.5 (seeded synthetic bodies; no dataset exists for this).

A step is one Simulation::step kernel sequence (reduce-dt, kick, drift,
sort + tree build, SPH pass 1, EOS, gravity, SPH pass 2, kick, EOS) on the
whole particle set, through the library's fused C-ABI step.

  value      N * steps / device time of the timed steps, inputs resident
  e2e        same metric through the C-ABI with the simulation state on
             the host: every step uploads the state's input fields from
             pinned host memory, steps, and reads the state and the fields
             the engine's telemetry reads back
  roofline   the gravity kernel (dominant): 23 FLOP per evaluated pair
             interaction (device counter) / CUDA-event launch time, against
             the FP32 FMA throughput measured in this process
  cpu_baseline  the reference algorithm's FP64 host path (oracle/, OpenMP
             on the host cores): two full steps of the same workload
  other_configs  the 4M Plummer sphere (gravity only: plain against the
             far-field modes at their FP64 errors) and the 16M gas-giant
             impact (full steps), run as --workload c3 / c5 child processes
  reference_cuda  the reference's own CUDA kernels (compiled for sm_100
             from its checkout into oracle/_ref) stepping the same initial
             state on the same GPU, CUDA-event timed, and this library's
             speed-up over them

--impl reference prints the CPU reference arm on the same workload and
metric: full FP64 host steps, W untimed and K timed; beside them, in
"reference_cuda", the reference's own CUDA kernels (compiled for sm_100 from
its checkout) stepping the same workload on this GPU, when that build is
present.  Under torchrun each rank runs an independent replica
(the path has no cross-GPU exchange; "replicas only"); value aggregates all
ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "astraea-impact-sim_gb300"))

METRIC = "particle-steps/s at N=1M, learned-θ vs plain BH at equal force error"
UNIT = "particle-steps/s"
FLOP_PER_INTERACTION = 23        # 20 force + 3 potential (rsqrt counted once)
def kernels_per_step(n):
    """Launches of one fused step: kick, drift, histogram, 8 onesweep,
    permute + Karras, the refit (block, scan, one launch per three
    sparse-table levels above the first, cross), neighbour lists, pass 1,
    EOS, gravity, pass 2, kick."""
    nb = max(1, (n + 255) // 256)
    levels = nb.bit_length()                   # levels 0 .. floor(log2 nb)
    return 18 + 3 + (levels - 1 + 2) // 3
# Fields a fused step reads (uploaded every e2e step) and the fields the
# engine's per-step telemetry reads back (engine/simulation.cpp:948-1000).
E2E_IN = ["posX", "posY", "posZ", "velX", "velY", "velZ", "accX", "accY", "accZ", "mass", "h", "h0", "rho",
          "drhoDt", "pressure", "soundSpeed", "u", "duDt", "tempK", "sXX", "sYY", "sZZ", "sXY", "sXZ", "sYZ",
          "dSXX", "dSYY", "dSZZ", "dSXY", "dSXZ", "dSYZ", "damage", "damageCbrt", "dDamageCbrtDt", "epsFail",
          "materialId", "phaseId", "bodyId", "originalId", "tracerIndex"]
E2E_OUT = ["posX", "posY", "posZ", "velX", "velY", "velZ", "mass", "rho", "u", "phiGrav", "tempK", "pressure",
           "radPowerW", "damage", "bodyId", "materialId", "originalId"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None,
                    help="particles (default: 1M for c2, 4M for c3, 16M for c5)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c5", "planet", "verify"],
                    help="c2: the 1M differentiated impact (the headline line); c3: 4M Plummer sphere, "
                         "gravity only, plain vs quadrupole and learned far field; c5: 16M gas-giant core impact; "
                         "planet: scenario construction only (the planet_builder field); verify: the engine's "
                         "headless --verify-conservation run (preset scenario, 100 steps) on the device path")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--max-dt-sec", type=float, default=5.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-far-field", action="store_true", help="skip the far-field comparison (quadrupole and learned)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-planet", action="store_true", help="skip the planet-construction measurement")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default block shape of the tree walks")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the 4M Plummer (c3) and 16M gas-giant (c5) runs summarised in the c2 line")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip timing the reference's own CUDA kernels (oracle/_ref cubin) beside this library")
    ap.add_argument("--eager", action="store_true",
                    help="time the steps as separate C-ABI calls instead of replaying a captured two-step graph")
    ap.add_argument("--far-field", type=int, default=0, choices=[0, 1],
                    help="far-field model of the timed steps: 0 monopole (the engine's), 1 + quadrupole")
    return ap.parse_args()


def workload_config(n, theta, far_field=0, workload="c2"):
    if workload == "c5":
        name = ("gas-giant core impact, N=%d: HydrogenHelium n=1 polytrope envelope over an Iron+Granite core "
                "(10%% of the target mass, 10 Earth masses), Regolith impactor of %d particles (mass ratio 0.1) "
                "at 2.0 v_esc and 30 deg" % (n, n // 8))
    else:
        name = ("differentiated Earth-Theia-like impact, N=%d (target %d + impactor %d), Iron core 30%% "
                "+ Granite mantle, hydrostatic radial density, mass ratio 0.1, 1.1 v_esc at 45 deg, strength "
                "+ damage on" % (n, n - int(round(0.2 * n)), int(round(0.2 * n))))
    return {
        "workload": name,
        "n_particles": n,
        "traversal": ("plain Barnes-Hut theta=%.2f (monopole, the engine's kernel)" % theta if far_field == 0 else
                      "Barnes-Hut theta=%.2f, monopole + quadrupole far field" % theta),
        "max_dt_psu": None,
        "l2": "inputs larger than L2: particle SoA %.0f MB + tree/neighbour scratch ~%.0f MB (L2 129 MB)"
              % (2 * n * 212 / 1e6, n * 1.15e3 / 1e6),
        "parallelism": "replicas only (one independent simulation per GPU)",
    }


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        with open(self.path) as fh:
            rows = [r.split(",") for r in fh.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------- GPU arm
def replica_rate(local_units, local_ms, dist=None, device="cpu"):
    """Whole-job throughput of independent replicas: the particle-steps of all
    ranks over the slowest rank's time (max over ranks).  Returns
    (units per second, slowest ms)."""
    import torch
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    ms = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(units, op=dist.ReduceOp.SUM)
        dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    return float(units.item()) / (float(ms.item()) / 1.0e3), float(ms.item())


def run_gpu(args):
    import numpy as np
    import torch
    from astraea_gb300 import engine, scenarios

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = args.n
    max_dt = max(1.0e-5, args.max_dt_sec) / 1.0e3
    engine.set_far_field(args.far_field)
    if args.workload == "c5":
        st, info = scenarios.gas_giant_impact(n_total=n, n_impactor=n // 8, seed=42 + rank)
    else:
        st, info = scenarios.differentiated_impact(n_total=n, seed=42 + rank)
    sim = engine.Simulation(n)
    sim.load_state(st)
    engine.reserve(sim.bvh, n)
    sim.evaluate_initial_forces(args.theta)
    tuning = None
    if not args.no_autotune:                   # block shape of the two walks, then fresh forces
        tuning = engine.autotune(sim.p, sim.bvh, args.theta)
        sim.evaluate_initial_forces(args.theta)
    for _ in range(max(args.warmup, 0)):
        sim.step(max_dt, args.theta)
    torch.cuda.synchronize()
    dt_host = torch.zeros(1, dtype=torch.float32).pin_memory()
    prev = sim.prev_dt
    # Two fused steps captured in one CUDA graph (the step makes no host
    # synchronisation or allocation after astraea_gb300_reserve; after two
    # steps the particle buffers and device dt slots are back where they
    # started, so the graph replays as is): the step's ~25 launches go to the
    # GPU as one graph launch.  Capture and one replay are untimed.
    graph = None
    if not args.eager:
        cap = torch.cuda.Stream()
        graph = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(graph, stream=cap):
                engine.set_stream(cap)
                for _ in range(2):
                    engine.step(sim.p, sim.alt, sim.bvh, prev, max_dt, args.theta, dt_host.data_ptr())
        finally:
            engine.set_stream(None)
        graph.replay()
        torch.cuda.synchronize()

    # ---- timed region: fused steps, state resident in HBM
    engine.reset_device_status()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    if graph is not None:
        for _ in range(args.steps // 2):
            graph.replay()
        for _ in range(args.steps % 2):
            engine.step(sim.p, sim.alt, sim.bvh, prev, max_dt, args.theta, dt_host.data_ptr())
    else:
        for _ in range(args.steps):
            engine.step(sim.p, sim.alt, sim.bvh, prev, max_dt, args.theta, dt_host.data_ptr())
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    flags, counters = engine.read_device_status()
    value, ms_max = replica_rate(n * args.steps, ms, dist, "cuda")
    sim.prev_dt = float(dt_host[0])

    # ---- dominant kernel: gravity, timed standalone on the current tree
    reps = 5
    engine.gravity_barnes_hut(sim.p, sim.bvh, args.theta)
    torch.cuda.synchronize()
    engine.reset_device_status()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(reps):
        engine.gravity_barnes_hut(sim.p, sim.bvh, args.theta)
    g1.record()
    torch.cuda.synchronize()
    _, gc = engine.read_device_status()
    grav_ms = g0.elapsed_time(g1) / reps
    inter = gc["gravity_interactions"] / reps
    fp32_scalar, fp32_packed = engine.measure_fp32_peaks()
    fp32_peak = max(fp32_scalar, fp32_packed)
    achieved = FLOP_PER_INTERACTION * inter / (grav_ms * 1e-3) / 1e12
    traffic = None
    issue = None
    tpath = os.path.join(ROOT, "profiles", "gravity_traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as fh:
                tr = json.load(fh)
            ipg = tr.get("warp_instructions_per_group")
            if ipg:
                # the bound the kernel actually meets: warp-instruction issue
                # (4 schedulers per SM, one instruction per clock each)
                props = torch.cuda.get_device_properties(torch.cuda.current_device())
                sm_hz = float((clk or {}).get("sm_mhz") or 2070.0) * 1e6
                peak_issue = props.multi_processor_count * 4 * sm_hz
                groups = (n + 31) // 32
                tests_ref = tr.get("node_tests_per_group_at_capture") or 0.0
                tests_now = gc.get("gravity_node_tests", 0) / reps / groups
                inst = ipg * groups * ((tests_now / tests_ref) if tests_ref and tests_now else 1.0)
                issue = {"bound": "instruction issue", "warp_instructions_per_launch": inst,
                         "achieved": inst / (grav_ms * 1e-3), "peak": peak_issue, "unit": "warp instructions/s",
                         "frac": inst / (grav_ms * 1e-3) / peak_issue,
                         "source": "instructions per group from the 262k ncu capture (profiles/gravity_c2_262k.md), "
                                   "scaled by this run's node tests per group and group count (an estimate); "
                                   "peak = SMs x 4 schedulers x the sampled SM clock"}
            # measured per launch at this N when the capture is of this size,
            # else scaled by the particle count (the records are read once)
            if tr.get("n") == n and tr.get("dram_bytes_per_launch"):
                traffic = float(tr["dram_bytes_per_launch"])
            else:
                traffic = tr.get("bytes_per_particle") and tr["bytes_per_particle"] * n
        except ValueError:
            traffic = None

    # ---- per-stage times of the fused step (events between its stages)
    stages = stage_breakdown(sim, engine, torch, args, max_dt, n, fp32_peak)

    # ---- force error of the plain path vs an FP64 direct sum (sampled targets)
    truth = fp64_truth(sim, torch, samples=1024)
    err_rms = force_error_fp64(sim, engine, torch, np, truth=truth, theta=args.theta)

    frame = frame_stages(sim, engine, torch, np, n)
    far = None
    if not args.no_far_field:
        learned = train_learned(engine, torch, [scenarios.differentiated_impact(n_total=262_144, seed=s)[0]
                                                for s in (901, 902)])
        far = far_field_scan(sim, engine, torch, np, args, max_dt, truth, learned=learned)
    ens = None if (args.no_ensemble or world > 1) else ensemble_run(engine, scenarios, torch, max_dt, args.theta)
    planet = None if (args.no_planet or world > 1) else planet_stage(engine, torch, np)

    # ---- e2e through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sim, engine, torch, args, max_dt, world, dist)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 in drift, refit moments)",
        "data": "synthetic (seeded hydrostatic bodies)",
        "config": workload_config(n, args.theta, args.far_field, args.workload),
        "gpu_launches": kernels_per_step(n) * args.steps,
        "clocks": clk,
        "roofline": {"kernel": "gravity (Barnes-Hut group walk + pair evaluation)", "bound": "fp32",
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if fp32_peak else None, "traffic": traffic,
                     "peak_source": "measured in-process: the larger of scalar fmaf (%.1f) and packed "
                                    "fma.rn.f32x2 (%.1f) FMA chains; the bf16/HBM peaks of MEASURED_PEAKS.json "
                                    "do not bound this kernel" % (fp32_scalar, fp32_packed),
                     "interactions_per_launch": inter, "launch_ms": grav_ms, "issue": issue},
        "step_hbm": step_hbm_roofline(n, ms_max / args.steps),
        "stages": stages,
        "force_error_rms_vs_fp64": err_rms,
        "step_counters_per_particle": {k: v / (args.steps * n) for k, v in counters.items()
                                       if k != "gravity_stack_peak"},
        "gravity_stack_peak": counters.get("gravity_stack_peak"),
        "device_flags": flags,
        "frame_stages": frame,
        "far_field": far,
        "ensemble": ens,
        "planet_builder": planet,
        "e2e": e2e,
    }
    out["config"]["max_dt_psu"] = max_dt
    out["config"]["autotuned_walks"] = tuning
    out["config"]["launch"] = ("eager C-ABI calls, one per step" if graph is None else
                               "two fused steps captured in one CUDA graph, replayed (the library's graph-capturable "
                               "step; the e2e number below is eager calls through the C-ABI)")
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(st, args, max_dt)
    if rank == 0 and world == 1 and args.workload == "c2" and not args.no_other_configs:
        out["other_configs"] = other_configs(args)
    if rank == 0 and world == 1 and args.workload == "c2" and not args.no_reference_cuda:
        # the reference's own kernels on the same GPU and initial state, after
        # everything above (their buffers are separate and freed afterwards)
        ref = reference_cuda(n, st)
        out["reference_cuda"] = ref
        if isinstance(ref, dict):
            out["reference_cuda"]["speedup_of_this_library"] = ref["ms_per_step_median"] / (ms_max / args.steps)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def other_configs(args):
    """The 4M Plummer sphere (gravity only, plain against the far-field
    modes, errors against the FP64 direct sum) and the 16M gas-giant core
    impact (full fused steps), each run as `bench.py --workload c3|c5` in a
    child process after this line's own measurements, summarised here."""
    res = {}
    for wl, extra in (("c3", ["--steps", "6", "--warmup", "1"]), ("c5", ["--steps", "5", "--warmup", "3"])):
        try:
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--workload", wl] + extra,
                               capture_output=True, text=True, timeout=900)
            line = json.loads(r.stdout.strip().splitlines()[-1])
        except Exception as exc:                # report, never fail the headline line
            res[wl] = "unavailable: %s" % str(exc).splitlines()[0][:200]
            continue
        if wl == "c3":
            keep = ("theta", "far_field", "gravity_ms", "force_rms_vs_fp64", "gravity_speedup_vs_plain",
                    "theta_far", "gamma", "leaf_bucket")
            res[wl] = {"config": line["config"]["workload"],
                       "runs": [{k: r0[k] for k in keep if k in r0} for r0 in line["runs"]],
                       "equal_error_choice": line.get("equal_error_choice")}
        else:
            res[wl] = {k: line.get(k) for k in ("metric", "value", "unit", "ms_per_step", "force_error_rms_vs_fp64",
                                                 "clocks")}
            res[wl]["config"] = line["config"]["workload"]
            res[wl]["gravity"] = {k: line["roofline"].get(k) for k in ("launch_ms", "achieved", "frac", "unit")}
    return res


def ensemble_run(engine, scenarios, torch, max_dt, theta, replays=25, eager_pairs=4):
    """The batched-ensemble workload: 64 independent impacts, N log-uniform
    in [8k, 128k] (2.76M particles in all), angle 0..75 deg, 1..3 v_esc,
    materials Iron / Granite / WaterIce / Regolith.  Eager fused steps
    instance after instance vs one CUDA graph holding two steps of every
    instance on its own stream."""
    states = [scenarios.ensemble_impact(**c)[0] for c in scenarios.ensemble_configs()]
    ens = engine.Ensemble(states, max_dt, theta)
    ens.step_sequential(2)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    ens.step_sequential(2 * eager_pairs)
    ev[1].record()
    ens.capture()
    torch.cuda.synchronize()
    ens.replay(1)
    torch.cuda.synchronize()
    ev[2].record()
    ens.replay(replays)
    ev[3].record()
    torch.cuda.synchronize()
    steps = 2 * replays
    eager_ms = ev[0].elapsed_time(ev[1]) / (2 * eager_pairs)
    graph_ms = ev[2].elapsed_time(ev[3]) / steps
    total = ens.particles
    tuned = {"2^%d" % k: v for k, v in sorted(ens.tuning.items())}
    del ens
    torch.cuda.empty_cache()
    return {"instances": len(states), "particles": total, "steps": steps,
            "eager_ms_per_step": eager_ms, "graph_ms_per_step": graph_ms,
            "eager_particle_steps_per_s": total / (eager_ms * 1e-3),
            "graph_particle_steps_per_s": total / (graph_ms * 1e-3),
            "graph_speedup": eager_ms / graph_ms,
            "autotuned_walks": tuned}


def planet_stage(engine, torch, np, reps=3):
    """Scenario construction (PlanetBuilder::buildPlanet + the body upload)
    for the two-body setups of the 1M and 16M workloads: target and
    impactor written straight into one particle buffer by
    astraea_gb300_build_planet (wall time, median of `reps`), against the
    oracle's serial restatement of the reference builder on this host (one
    run; bit-identical to the reference library where that was built)."""
    orc = _oracle()
    cases = {
        "1M: LivingTerra 800k (6x16x16 tracers) + ProtoTheia 200k": [(0, 800_000, 0, 16, 42, None),
                                                                    (5, 200_000, 1, 0, 43, 0.025 * 5.97219e24)],
        "16M: GasGiant 14M + ProtoTheia 2M": [(4, 14_000_000, 0, 0, 42, None), (5, 2_000_000, 1, 0, 43, None)],
    }
    out = {}
    for name, bodies in cases.items():
        total = sum(b[1] for b in bodies)
        p = engine.DeviceParticles(total)
        times = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            off = 0
            for a, n, body, grid, seed, mass in bodies:
                engine.build_planet(engine.body_spec(a, mass_kg=mass), n, p, offset=off, body_id=body,
                                    tracer_grid_res=grid, seed=seed)
                off += n
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        del p
        torch.cuda.empty_cache()
        t0 = time.perf_counter()
        for a, n, body, grid, seed, mass in bodies:
            orc.build_planet(engine.body_spec(a, mass_kg=mass), n, body, grid, seed)
        cpu_s = time.perf_counter() - t0
        dev_s = float(np.median(times))
        out[name] = {"particles": total, "device_s": dev_s, "oracle_cpu_s": cpu_s,
                     "device_particles_per_s": total / dev_s, "cpu_particles_per_s": total / cpu_s,
                     "speedup": cpu_s / dev_s}
    return out


def frame_stages(sim, engine, torch, np, n, reps=5):
    """Per-frame work outside the step: the telemetry reduction (FP64 device
    passes; about 219 B per particle over its seven passes) and one PCLS
    frame (about 47 B read + 21 B written per particle), median of `reps`."""
    from astraea_gb300 import abi
    tele = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        engine.reduce_telemetry(sim.p, 1.0, True)          # blocks until the result is on the host
        tele.append((time.perf_counter() - t0) * 1e3)
    size = engine.pcls_frame_bytes(n, 0, True)
    buf = torch.empty(size, dtype=torch.uint8, device="cuda")
    info = abi.PclsFrameInfo()
    info.withSpeed = 1
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    pk = []
    for _ in range(reps):
        ev[0].record()
        engine.pack_pcls_frame(sim.p, info, buf)
        ev[1].record()
        torch.cuda.synchronize()
        pk.append(ev[0].elapsed_time(ev[1]))
    tm, pm = float(np.median(tele)), float(np.median(pk))
    return {"telemetry_ms": tm, "telemetry_gbs": 219.0 * n / (tm * 1e-3) / 1e9,
            "pcls_frame_ms": pm, "pcls_frame_bytes": size, "pcls_frame_gbs": 68.0 * n / (pm * 1e-3) / 1e9}


def hbm_peak():
    """Measured STREAM-style copy bandwidth of the GB300s (GB/s)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def step_hbm_roofline(n, ms):
    """Compulsory bytes per particle-step of the reference SoA (1.58 KB, the
    per-stage sum of the engine's reads/writes) against measured HBM."""
    peak = hbm_peak()
    achieved = 1580.0 * n / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "bytes_per_particle_step": 1580.0}


# Compulsory bytes per particle of each fused-step stage for the reference SoA
# (drift 44; bounds 12 + Morton 24 + sort 200; permute 428; build + refit 172;
# pass 1 68; EOS 26 per evaluation; gravity 32; pass 2 171; kick 169 per
# half kick; dt 41 with the closing kick): 1,582 B per particle-step.
STAGE_BYTES = {"kick": 169, "drift": 44, "sort": 236, "permute": 428, "refit": 172, "pass1": 68, "eos": 26,
               "gravity": 32, "pass2": 171, "kick_eos": 236}
# FP32 operations per in-range pair, counted from the restated formulas
# (every term; a sqrt, a quotient and a Wendland evaluation count as the
# operations written): pass 1 65, pass 2 189 (with the viscosity, delta-SPH
# and tensile terms), XSPH drift 41.
PAIR_FLOP = {"pass1": 65, "pass2": 189, "drift": 41}


def stage_breakdown(sim, engine, torch, args, max_dt, n, fp32_peak, steps=3):
    """CUDA-event time of every stage of the fused step (astraea_gb300_
    set_stage_timing), averaged over a few steps after the timed region, with
    each stage's compulsory bytes against measured HBM and, for the SPH pair
    loops, the in-range pairs (device counters) times their FLOP count
    against the measured FP32 FMA peak."""
    from astraea_gb300 import abi
    acc = dict.fromkeys(abi.STAGES, 0.0)
    # one untimed step first: the stage calls before this may have left the
    # step cache invalid, which would put a refresh into the first timed step
    engine.step(sim.p, sim.alt, sim.bvh, sim.prev_dt, max_dt, args.theta, None)
    engine.reset_device_status()
    engine.set_stage_timing(True)
    try:
        for _ in range(steps):
            engine.step(sim.p, sim.alt, sim.bvh, sim.prev_dt, max_dt, args.theta, None)
            for k, v in engine.read_stage_times(sim.bvh).items():
                acc[k] += v / steps
    finally:
        engine.set_stage_timing(False)
    counters = engine.read_device_counters()
    peak = hbm_peak()
    out = {}
    for k, ms in acc.items():
        e = {"ms": ms}
        if k in STAGE_BYTES and ms > 0.0:
            gbs = STAGE_BYTES[k] * n / (ms * 1e-3) / 1e9
            e.update(bytes_per_particle=STAGE_BYTES[k], gbs=gbs, frac_hbm=gbs / peak)
        if k in PAIR_FLOP and ms > 0.0:
            pairs = counters[k + "_pairs"] / steps
            tf = PAIR_FLOP[k] * pairs / (ms * 1e-3) / 1e12
            e.update(pairs_per_particle=pairs / n, flop_per_pair=PAIR_FLOP[k], tflops=tf,
                     frac_fp32=tf / fp32_peak if fp32_peak else None)
        out[k] = e
    out["hbm_peak_gbs"] = peak
    out["total_ms"] = sum(acc.values())
    return out


def force_error_fp64(sim, engine, torch, np, samples=1024, truth=None, theta=0.5):
    """RMS of |a - a_FP64| / |a_FP64| over sampled targets of the gravity of
    the timed configuration; the FP64 direct sum runs on the GPU in float64."""
    engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
    torch.cuda.synchronize()
    return rms_vs_truth(sim, torch, truth or fp64_truth(sim, torch, samples))


def rms_vs_truth(sim, torch, truth):
    tgt, acc = truth
    n = sim.p.count
    A = sim.p.arrays
    bh = torch.stack([A["accX"][:n][tgt], A["accY"][:n][tgt], A["accZ"][:n][tgt]], 1).double()
    rel = (bh - acc).norm(dim=1) / acc.norm(dim=1)
    return float(torch.sqrt((rel * rel).mean()))


def fp64_truth(sim, torch, samples=1024):
    """Sampled targets and their FP64 direct-sum accelerations (eps_ij
    softening, G_PSU), on the GPU in torch float64."""
    n = sim.p.count
    A = sim.p.arrays
    g = torch.Generator(device="cpu").manual_seed(1234)
    tgt = torch.randperm(n, generator=g)[:samples].cuda()
    pos = torch.stack([A["posX"][:n], A["posY"][:n], A["posZ"][:n]], 1).double()
    m = A["mass"][:n].double()
    eps = 0.8 * torch.clamp(A["h0"][:n].double(), min=1e-6)
    G = 6.67430e-11 * 1e24 * 1e6 / 1e18
    acc = torch.zeros(samples, 3, dtype=torch.float64, device="cuda")
    pt, et = pos[tgt], eps[tgt]
    for s0 in range(0, n, 1 << 16):
        s1 = min(n, s0 + (1 << 16))
        d = pt[:, None, :] - pos[None, s0:s1, :]
        e = 0.5 * (et[:, None] + eps[None, s0:s1])
        r2 = (d * d).sum(-1) + e * e
        w = m[None, s0:s1] * r2.rsqrt() ** 3
        idx = torch.arange(s0, s1, device="cuda")
        w = torch.where(tgt[:, None] == idx[None, :], torch.zeros_like(w), w)
        acc -= G * (w[:, :, None] * d).sum(1)
    return tgt, acc


def train_learned(engine, torch, states, steps=1500):
    """Trains the far-field network of mode 2 on the GPU on other snapshots
    of the same kind of workload (never the measured one)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows, hist = engine.train_far_field(states, steps=steps, batch=8192, lr=2e-3, seed=1)
    torch.cuda.synchronize()
    return {"training_rows": rows, "training_steps": steps, "loss_first": hist[0][1], "loss_last": hist[-1][1],
            "training_s": time.perf_counter() - t0, "snapshots": len(states)}


FAR_CONFIGS = (
    {"theta": 0.5, "mode": 0},
    {"theta": 0.6, "mode": 1}, {"theta": 0.7, "mode": 1}, {"theta": 0.8, "mode": 1},
    {"theta": 0.5, "mode": 2, "theta_far": 0.9, "gamma": 0.3},
    {"theta": 0.5, "mode": 2, "theta_far": 1.2, "gamma": 0.3},
    {"theta": 0.5, "mode": 2, "theta_far": 0.9, "gamma": 0.5},
    {"theta": 0.7, "mode": 3, "bucket": "auto", "gamma": 0.3},
    {"theta": 0.7, "mode": 3, "bucket": 16, "gamma": 0.2},
    {"theta": 0.75, "mode": 3, "bucket": "auto", "gamma": 0.2},
    {"theta": 0.75, "mode": 3, "bucket": "auto", "gamma": 0.3},
    {"theta": 0.8, "mode": 3, "bucket": "auto", "gamma": 0.2},
)
FAR_NAMES = {0: "monopole", 1: "monopole+quadrupole", 2: "monopole+learned correction",
             3: "quadrupole+leaf buckets+group expansion"}


def set_mode(engine, sim, cfg, theta, tune=False):
    """Far-field mode of one scan entry; mode 3 with bucket "auto" tunes the
    leaf bucket on the current tree; with tune, the block shape of the
    gravity walk this mode runs at theta is tuned too (each walk variant
    keeps its own).  Returns the bucket used (mode 3)."""
    mode = cfg["mode"]
    if mode == 2:
        engine.ff_configure(theta_far=cfg["theta_far"], gamma=cfg["gamma"], gate_tolerance=0.0)
    engine.set_far_field(mode)
    bucket = None
    if mode == 3:
        bucket = 16 if cfg["bucket"] == "auto" else int(cfg["bucket"])
        engine.set_far_field_expansion(bucket, cfg["gamma"])
    engine.sort_and_build_bvh(sim.p, sim.alt, sim.bvh)
    if mode == 3 and cfg["bucket"] == "auto":
        bucket, _ = engine.autotune_expansion(sim.p, sim.bvh, theta)
    if tune:
        engine.autotune(sim.p, sim.bvh, theta)
    return bucket


def far_field_scan(sim, engine, torch, np, args, max_dt, truth, configs=FAR_CONFIGS, learned=None):
    """Plain monopole at theta 0.5 (the engine's kernel) against the
    quadrupole far field (mode 1) at larger opening angles and the learned
    correction (mode 2: far nodes taken at theta_far with the network's
    residual and Jacobian): gravity time, interactions and RMS force error
    vs the FP64 direct sum on the same tree (mode 2 also without the
    correction, the network zeroed), then the whole fused step."""
    out = []
    if learned is not None:
        params, scale = engine.ff_get_params()
    for cfg in configs:
        theta, mode = cfg["theta"], cfg["mode"]
        if mode == 2 and learned is None:
            continue
        bucket = set_mode(engine, sim, cfg, theta, tune=not args.no_autotune)   # sorted already: identity permutation
        engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
        torch.cuda.synchronize()
        engine.reset_device_status()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(5):
            engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
        ev[1].record()
        torch.cuda.synchronize()
        _, gc = engine.read_device_status()
        rec = {"theta": theta, "far_field": FAR_NAMES[mode], "gravity_ms": ev[0].elapsed_time(ev[1]) / 5,
               "interactions_per_particle": gc["gravity_interactions"] / 5 / sim.p.count,
               "force_rms_vs_fp64": rms_vs_truth(sim, torch, truth)}
        if mode == 3:
            cc = engine.read_device_counters()
            rec.update({"leaf_bucket": bucket, "leaf_bucket_autotuned": cfg["bucket"] == "auto",
                        "gamma": cfg["gamma"],
                        "expansion_terms_per_particle": cc["gravity_group_evals"] / 5 / sim.p.count,
                        "bucket_terms_per_particle": cc["gravity_bucket_leaves"] / 5 / sim.p.count})
        if mode == 2:
            rec.update({"theta_far": cfg["theta_far"], "gamma": cfg["gamma"]})
            engine.ff_set_params(np.zeros_like(params), scale)
            engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
            rec["force_rms_without_correction"] = rms_vs_truth(sim, torch, truth)
            engine.ff_set_params(params, scale)
            # where the time of the mode goes (no gate: spot check and fallback 0)
            parts = [engine.ff_profile(sim.p, sim.bvh, theta) for _ in range(3)]
            rec["gravity_parts_ms"] = {k: float(np.median([q[k] for q in parts])) for k in parts[0]}
            engine.ff_configure(theta_far=cfg["theta_far"], gamma=cfg["gamma"], gate_tolerance=1.0, gate_targets=64,
                                gate_fp64_pairs=True)
            gated = engine.ff_profile(sim.p, sim.bvh, theta)
            engine.ff_configure(theta_far=cfg["theta_far"], gamma=cfg["gamma"], gate_tolerance=1.0, gate_targets=64)
            gated32 = engine.ff_profile(sim.p, sim.bvh, theta)
            engine.ff_configure(theta_far=cfg["theta_far"], gamma=cfg["gamma"], gate_tolerance=0.0)
            rec["gate_ms"] = {"fp64_spot_check_64_targets": gated["gate"],
                              "fp32_pairs_spot_check_64_targets": gated32["gate"],
                              "skipped_fallback_walk": gated["fallback"]}
            engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
        out.append(rec)
    # whole steps (the state advances; e2e re-uploads its own inputs afterwards)
    dt_host = torch.zeros(1, dtype=torch.float32).pin_memory()
    for rec in out:
        mode = {v: k for k, v in FAR_NAMES.items()}[rec["far_field"]]
        cfg = {"mode": mode, "theta_far": rec.get("theta_far"), "gamma": rec.get("gamma"),
               "bucket": rec.get("leaf_bucket")}
        set_mode(engine, sim, cfg, rec["theta"])
        engine.invalidate_step_cache(sim.bvh)
        for _ in range(2):
            engine.step(sim.p, sim.alt, sim.bvh, sim.prev_dt, max_dt, rec["theta"], dt_host.data_ptr())
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        k = max(3, args.steps // 2)
        ev[0].record()
        for _ in range(k):
            engine.step(sim.p, sim.alt, sim.bvh, sim.prev_dt, max_dt, rec["theta"], dt_host.data_ptr())
        ev[1].record()
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / k
        rec["step_ms"] = ms
        rec["particle_steps_per_s"] = sim.p.count / (ms * 1e-3)
    engine.set_far_field(0)
    engine.set_far_field_expansion(16, 0.3)
    engine.sort_and_build_bvh(sim.p, sim.alt, sim.bvh)
    engine.invalidate_step_cache(sim.bvh)
    base = out[0]
    ok = [r for r in out[1:] if r["force_rms_vs_fp64"] <= base["force_rms_vs_fp64"]]
    best = max(ok, key=lambda r: r["particle_steps_per_s"]) if ok else None
    lr = [r for r in out if r["far_field"] == FAR_NAMES[2]]
    grav_share = base["gravity_ms"] / base["step_ms"]
    for r in out:
        r["gravity_speedup_vs_plain"] = base["gravity_ms"] / r["gravity_ms"]
    return {"runs": out, "learned_training": learned,
            "gravity_share_of_plain_step": grav_share,
            "amdahl_bound_step_speedup": 1.0 / (1.0 - grav_share),
            "learned_best_gravity_vs_plain": max(r["gravity_speedup_vs_plain"] for r in lr) if lr else None,
            "equal_error_gravity_best": max((r["gravity_speedup_vs_plain"] for r in ok), default=None),
            "equal_error_choice": best and {"theta": best["theta"], "far_field": best["far_field"],
                                            "theta_far": best.get("theta_far"),
                                            "speedup_vs_plain_theta05": best["particle_steps_per_s"] /
                                            base["particle_steps_per_s"]},
            "learned_best_vs_plain": (max(r["particle_steps_per_s"] for r in lr) / base["particle_steps_per_s"])
                                     if lr else None}


def run_e2e(sim, engine, torch, args, max_dt, world, dist):
    """The same fused step through the C-ABI with the simulation state held
    on the host: every step uploads the state's input fields from pinned
    host memory into the particle arrays, steps, and reads the state back
    (the input fields and the engine's telemetry fields) together with dt.
    Two device states alternate, so the copies run on their own streams (H2D
    and D2H in both copy engines) and overlap the kernels of the step on the
    other state: step k uploads into state k mod 2 while step k-1 computes
    on the other one, and reads its results back while step k+1 computes.
    What a step uploads is what the previous step on that state read back,
    so the library's tree still bounds it; the step cache is invalidated all
    the same (the library cannot know that), so every step rebuilds its dt
    and neighbour lists from the uploaded state."""
    n = sim.p.count
    sims = [sim, engine.Simulation(n)]
    sims[1].load_state(sim.p.download())
    engine.reserve(sims[1].bvh, n)
    sims[1].evaluate_initial_forces(args.theta)
    fields_out = E2E_IN + [f for f in E2E_OUT if f not in E2E_IN]
    host = [{f: torch.empty_like(sim.p.arrays[f][:n], device="cpu").pin_memory() for f in fields_out}
            for _ in range(2)]
    for b in range(2):
        for f in fields_out:
            host[b][f].copy_(sims[b].p.arrays[f][:n])
    dt_host = torch.zeros(2, dtype=torch.float32).pin_memory()
    bi = sum(host[0][f].numel() * host[0][f].element_size() for f in E2E_IN)
    bo = sum(host[0][f].numel() * host[0][f].element_size() for f in fields_out) + 4
    comp, h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev = lambda: torch.cuda.Event()
    in_ready, out_ready, out_read = [ev(), ev()], [ev(), ev()], [ev(), ev()]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    engine.set_stream(comp)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(comp)

    def upload(b, k):
        with torch.cuda.stream(h2d):
            h2d.wait_event(e0)
            if k >= 2:
                h2d.wait_event(out_read[b])         # state b read back after step k-2
            for f in E2E_IN:
                sims[b].p.arrays[f][:n].copy_(host[b][f], non_blocking=True)
            in_ready[b].record(h2d)

    upload(0, 0)
    for k in range(args.steps):
        b = k & 1
        if k + 1 < args.steps:
            upload(b ^ 1, k + 1)
        st = sims[b]
        with torch.cuda.stream(comp):
            comp.wait_event(in_ready[b])
            engine.invalidate_step_cache(st.bvh)
            engine.step(st.p, st.alt, st.bvh, st.prev_dt, max_dt, args.theta, dt_host[b:].data_ptr())
            out_ready[b].record(comp)
        with torch.cuda.stream(d2h):
            d2h.wait_event(out_ready[b])
            for f in fields_out:
                host[b][f].copy_(st.p.arrays[f][:n], non_blocking=True)
            out_read[b].record(d2h)
    comp.wait_stream(d2h)
    e1.record(comp)
    torch.cuda.synchronize()
    engine.set_stream(None)
    ms = e0.elapsed_time(e1)
    rate, _ = replica_rate(n * args.steps, ms, dist, "cuda")
    sims[1].bvh.free()
    del sims[1], st
    return {"value": rate, "unit": UNIT,
            "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
            "note": "the simulation state lives on the host: every step uploads its input fields from pinned "
                    "memory into the particle arrays, runs the fused step (step cache invalidated: neighbour "
                    "lists and dt recomputed from the uploaded state) and reads the state and the engine's "
                    "telemetry fields back with dt; two device states alternate so the copies run on their "
                    "own streams beside the other state's step"}


def run_c3(args):
    """Gravity-only traversal on a seeded Plummer sphere (a = 1, G = 1,
    softening 1e-3): plain monopole theta = 0.5 and the quadrupole far field
    at larger opening angles, RMS force error against the FP64 direct sum on
    65,536 sampled targets (the library's FP64 kernel)."""
    import numpy as np
    import torch
    from astraea_gb300 import engine, scenarios
    n = args.n
    st = scenarios.plummer_sphere(n)
    sim = engine.Simulation(n)
    sim.load_state(st)
    engine.reserve(sim.bvh, n)
    engine.set_far_field(0)
    engine.sort_and_build_bvh(sim.p, sim.alt, sim.bvh)
    g = torch.Generator(device="cpu").manual_seed(4321)
    tgt = torch.randperm(n, generator=g)[: min(65536, n)].cuda()
    t0 = time.perf_counter()
    acc64, _ = engine.direct_gravity_f64(sim.p, tgt)
    torch.cuda.synchronize()
    truth_s = time.perf_counter() - t0
    learned = train_learned(engine, torch, [scenarios.plummer_sphere(524_288, seed=s) for s in (901, 902)])
    params, scale = engine.ff_get_params()
    runs = []
    configs = [(t, m, None, None) for t, m in ((0.5, 0), (0.6, 0), (0.7, 0), (0.8, 0), (0.6, 1), (0.7, 1), (0.8, 1),
                                                (0.9, 1))]
    configs += [(0.5, 2, tf, gm) for tf, gm in ((0.9, 0.3), (1.2, 0.3), (0.9, 0.5))]
    configs += [(th, 3, None, gm) for th, gm in ((0.7, 0.3), (0.75, 0.2), (0.75, 0.3), (0.8, 0.2), (0.8, 0.3))]
    for theta, mode, theta_far, gamma in configs:
        bucket = set_mode(engine, sim, {"mode": mode, "theta_far": theta_far, "gamma": gamma, "bucket": "auto"},
                          theta, tune=not args.no_autotune)
        engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
        torch.cuda.synchronize()
        engine.reset_device_status()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(max(args.steps // 2, 3)):
            engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
        ev[1].record()
        torch.cuda.synchronize()
        reps = max(args.steps // 2, 3)
        ms = ev[0].elapsed_time(ev[1]) / reps
        _, c = engine.read_device_status()
        A = sim.p.arrays
        bh = torch.stack([A["accX"][:n][tgt], A["accY"][:n][tgt], A["accZ"][:n][tgt]], 1).double()
        rel = (bh - acc64).norm(dim=1) / acc64.norm(dim=1)
        rec = {"theta": theta, "far_field": FAR_NAMES[mode],
               "gravity_ms": ms, "particles_per_s": n / (ms * 1e-3),
               "interactions_per_particle": c["gravity_interactions"] / reps / n,
               "force_rms_vs_fp64": float(torch.sqrt((rel * rel).mean())),
               "force_p99_vs_fp64": float(torch.quantile(rel.float(), 0.99))}
        if mode == 3:
            cc = engine.read_device_counters()
            rec.update({"leaf_bucket": bucket, "gamma": gamma,
                        "expansion_terms_per_particle": cc["gravity_group_evals"] / reps / n,
                        "bucket_terms_per_particle": cc["gravity_bucket_leaves"] / reps / n})
        if mode == 2:
            rec.update({"theta_far": theta_far, "gamma": gamma})
            engine.ff_set_params(np.zeros_like(params), scale)
            engine.gravity_barnes_hut(sim.p, sim.bvh, theta)
            bh0 = torch.stack([A["accX"][:n][tgt], A["accY"][:n][tgt], A["accZ"][:n][tgt]], 1).double()
            rel0 = (bh0 - acc64).norm(dim=1) / acc64.norm(dim=1)
            rec["force_rms_without_correction"] = float(torch.sqrt((rel0 * rel0).mean()))
            engine.ff_set_params(params, scale)
        runs.append(rec)
    engine.set_far_field(0)
    engine.set_far_field_expansion(16, 0.3)
    base = runs[0]
    for r in runs:
        r["gravity_speedup_vs_plain"] = r["particles_per_s"] / base["particles_per_s"]
    ok = [r for r in runs[1:] if r["force_rms_vs_fp64"] <= base["force_rms_vs_fp64"]]
    best = max(ok, key=lambda r: r["particles_per_s"]) if ok else None
    print(json.dumps({
        "workload": "c3", "metric": "gravity traversals: particles/s at equal force error", "unit": "particles/s",
        "config": {"workload": "Plummer sphere N=%d (a=1, G=1 via m/G_PSU, softening 1e-3 => h0=1.25e-3), "
                               "gravity only" % n, "targets_fp64": int(tgt.numel()), "truth_seconds": truth_s},
        "runs": runs, "learned_training": learned,
        "equal_error_choice": best and {"theta": best["theta"], "far_field": best["far_field"],
                                        "theta_far": best.get("theta_far"),
                                        "speedup_vs_plain_theta05": best["particles_per_s"] /
                                        base["particles_per_s"]}}))


# ------------------------------------------------------------- CPU arm
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def cpu_fp64_step_rate(st, max_dt, steps=1, warmup=0):
    """Particle-steps/s of the reference algorithm's FP64 host path
    (oracle_step_f64: the reference's stage sequence restated for the CPU, the
    tree walks with FP64 pair arithmetic and sums, the reference's FP64 EOS,
    OpenMP over all host cores) on the full workload: every particle, every
    stage, `warmup` untimed and `steps` timed full steps after the initial
    forces.  Returns (rate, median step seconds, seconds of CPU work spent)."""
    oracle = _oracle()
    o = oracle.Oracle(st)
    oracle.set_group_stride(1)
    t_all = time.perf_counter()
    o.initial_forces()
    times = []
    for k in range(warmup + steps):
        c = time.perf_counter()
        o.step_f64(max_dt)
        if k >= warmup:
            times.append(time.perf_counter() - c)
    n = len(st["posX"])
    per_step = statistics.median(times)
    return n / per_step, per_step, time.perf_counter() - t_all


def host_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline(st, args, max_dt):
    n = len(st["posX"])
    rate, per_step, spent = cpu_fp64_step_rate(st, max_dt, steps=2)
    return {"value": rate, "unit": UNIT, "cores": host_threads(), "kind": "port",
            "sample": "2 full steps (every particle, every stage) of the same N=%d workload after its initial "
                      "forces, on the reference algorithm's FP64 host path (the oracle's restatement of the "
                      "reference kernels, FP64 pair arithmetic, OpenMP); median step %.2f s, %.1f s of CPU work"
                      % (n, per_step, spent)}


def reference_cuda(n, st, steps=10, warmup=3):
    """The reference's own CUDA kernels (engine/sph_gravity.cu + eos.cu,
    compiled unmodified for sm_100 from the reference checkout into
    oracle/_ref) stepping the same workload on this GPU, timed with CUDA
    events over the gpuStepMs span (engine/simulation.cpp:1719-1739)."""
    cubin = os.path.join(ROOT, "oracle", "_ref", "ref_kernels_sm100.cubin")
    if not os.path.exists(cubin):
        return "unavailable: oracle/_ref/ref_kernels_sm100.cubin is absent (it is compiled from the reference " \
               "checkout, which this machine does not have)"
    try:
        import torch
        if not torch.cuda.is_available():
            return "unavailable: no CUDA device visible"
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import ref_gpu
        rec = ref_gpu.bench(n, steps, warmup, st=st)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return rec
    except Exception as exc:                    # report, never fail the CPU arm
        return "unavailable: %s" % str(exc).splitlines()[0][:200]


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from astraea_gb300 import scenarios
    n = args.n
    max_dt = max(1.0e-5, args.max_dt_sec) / 1.0e3
    st, _ = scenarios.differentiated_impact(n_total=n, seed=42)
    ref_cuda = reference_cuda(n, st)
    rate, per_step, spent = cpu_fp64_step_rate(st, max_dt, steps=max(args.steps, 1), warmup=max(args.warmup, 0))
    cores = host_threads()
    sample = ("%d warm-up + %d timed full steps (every particle, every stage) of the N=%d workload after its "
              "initial forces, on the reference algorithm's FP64 host path: the oracle's restatement of the "
              "reference kernels (the reference has no CPU kernels of its own) with FP64 pair arithmetic and "
              "sums and the reference's FP64 EOS, OpenMP on %d host threads" % (args.warmup, args.steps, n, cores))
    cfg = workload_config(n, args.theta)
    cfg["max_dt_psu"] = max_dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (reference algorithm restated; FP64 pair arithmetic and EOS)",
        "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": ref_cuda, "cpu_seconds": spent,
    }))


if __name__ == "__main__":
    a = parse()
    if a.n is None:
        a.n = {"c2": 1_000_000, "c3": 4_000_000, "c5": 16_000_000}.get(a.workload, 0)
    if a.workload != "c2":
        a.no_cpu_baseline = a.no_ensemble = a.no_far_field = a.no_planet = True
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "c3":
        run_c3(a)
    elif a.workload == "verify":
        from astraea_gb300 import headless
        res = headless.run_headless("LivingGaiaAsteroidCataclysm", particles=a.n or 100000, steps=100)
        print(json.dumps({"workload": "verify", "metric": "conservation over 100 steps (engine thresholds)",
                          **res}))
        sys.exit(0 if res["ok"] else 1)
    elif a.workload == "planet":
        import numpy as np
        import torch
        from astraea_gb300 import engine
        print(json.dumps({"workload": "planet", "metric": "particles placed per second (wall)",
                          "planet_builder": planet_stage(engine, torch, np, reps=max(1, a.steps // 3))}))
    else:
        run_gpu(a)
