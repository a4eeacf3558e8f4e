"""Benchmark: MLS-MPM particle-substeps/s on the 1,000,000-particle lattice
(128^3 grid), GB300.

A step is one execute() of the reference (mls-mpm/mls-mpm.ts:245-268): two
substeps of clearGrid, p2g_1, p2g_2, updateGrid, g2p and copyPosition over
all particles.  Prints ONE JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm (default):
  value   device-resident throughput: per-step CUDA events on the launch
          stream, inputs resident in HBM, L2 flushed (256 MiB write) between
          timed steps, summed over K steps; max over ranks.
  e2e     the same metric through the public API with host buffers: each
          step sets the box from host memory (changeBoxSize), runs execute()
          and reads posvel back into pinned host memory; the read-back of a
          step overlaps the next step (downloadPosvelAsync into two
          alternating buffers) and one event pair spans all K steps and the
          last copy (no L2 flush: a step streams ~300 MB through the 129 MB
          L2).  `serialized_value`: a blocking read-back per step, per-step
          events, L2 flushed between steps outside them.
  roofline  the dominant kernel's algorithmic bytes per launch over its mean
          CUDA-event duration, against the measured HBM copy bandwidth;
          issue_roofline: its warp-instructions per launch against the SMs'
          issue rate; path_roofline: the whole substep's algorithmic bytes
          as the reference's six dispatches define them (204 B per
          particle + 100 B per grid cell) at the measured substep rate.
          The profiling pass and both e2e loops restart from the timed
          region's state (upload + the same warm-up).
  cpu_baseline  the C oracle (oracle/) on the host cores, bounded sample.
--impl reference: the oracle (the CPU restatement of the reference's kernels)
on all host threads, same workload and metric.  Under torchrun, rank 0 alone
runs it.
Multi-GPU: each rank runs its own replica (the path has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "MLS-MPM particle-substeps/s at 1M (bit-exact grid)"
UNIT = "particle-substeps/s"
SUBSTEPS = 2                  # per execute(), mls-mpm/mls-mpm.ts:247
AUTOTUNE_SUBSTEPS = 8         # timed per (block size, task size, lane-table threshold) candidate
N_PER_AXIS = 100              # 100^3 = 1,000,000 particles
ORIGIN, SPACING, JITTER, SEED = 4.0, 0.5, 0.05, 20240601
BOX = [128.0, 128.0, 128.0]
WORKLOAD = ("jittered lattice dam-break: 1,000,000 particles (100^3, spacing 0.5, "
            "jitter +-0.05, filling [4,54)^3), 128^3 grid, 2 substeps/step")
DTYPE = "f32 particle state, i32 fixed-point grid (x1e7)"
L2_FLUSH_BYTES = 256 << 20


def measured_peaks() -> dict:
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[4 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_scene(pkg):
    return pkg.scene_lattice(N_PER_AXIS, ORIGIN, SPACING, JITTER, SEED)


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def time_oracle(parts, steps: int, warmup: int, budget_s: float, nthreads: int, box=None):
    """Runs the oracle for warmup + up to `steps` execute() calls (2 substeps
    each), stopping when `budget_s` of timed work is exceeded."""
    from oracle import oracle
    sim = oracle.OracleSim(parts, BOX if box is None else box)
    for _ in range(warmup):
        sim.execute(SUBSTEPS, nthreads)
    done, t0 = 0, time.perf_counter()
    while done < steps:
        sim.execute(SUBSTEPS, nthreads)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done, dt


def cpu_model() -> str:
    """The host CPU's name from /proc/cpuinfo (model name on x86; implementer
    and part numbers on Arm), else the machine type."""
    import platform
    fields = {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if ":" in line:
                    k, v = line.split(":", 1)
                    fields.setdefault(k.strip(), v.strip())
    except OSError:
        pass
    if fields.get("model name"):
        return fields["model name"]
    if fields.get("CPU part"):
        return (f"{platform.machine()} CPU implementer {fields.get('CPU implementer', '?')} "
                f"part {fields['CPU part']}")
    return platform.machine()


def cpu_baseline_detail(pkg, budget_s: float = 3.0) -> dict:
    """The oracle on the 64,000-particle / 64^3 lattice (40^3 points from 3,
    spacing 0.5) and on the 1M-particle / 128^3 workload, on one host thread
    and on all of them, each a bounded sample from the initial state."""
    nt = cpu_threads()
    out = {"cpu": cpu_model(), "nproc": os.cpu_count(), "threads_all": nt,
           "budget_s_per_case": budget_s}
    cases = {"64k_64": (pkg.scene_lattice(40, 3.0, SPACING, JITTER, SEED), [64.0, 64.0, 64.0]),
             "1M_128": (make_scene(pkg), BOX)}
    for name, (parts, box) in cases.items():
        for threads in (1, nt):
            done, dt = time_oracle(parts, 1000, 0, budget_s, threads, box)
            out[f"{name}_{threads}t"] = {
                "particle_substeps_per_s": len(parts) * SUBSTEPS * done / dt,
                "substeps": done * SUBSTEPS, "seconds": dt}
    return out


PARITY_FRAMES = (1, 5, 25, 100, 200)


def cpu_baseline_and_parity(pkg, parts, stream, skip_parity: bool = False):
    """One oracle run of the benchmarked configuration from its initial
    state on all host threads.  Its first ~10 s are the timed CPU baseline;
    unless skipped, it continues for the configuration's full 200 frames
    and the GPU's grid, particles and posvel (a fresh simulator, same scene,
    sorted engine, CUDA graphs) are compared with it bit for bit after
    frames 1, 5, 25, 100 and 200."""
    import numpy as np
    from oracle import oracle
    nt = cpu_threads()
    n = len(parts)
    snaps = {}
    if not skip_parity:
        sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=n, maxGrid=(128, 128, 128))
        sim.upload(parts, BOX)
        for frame in range(1, PARITY_FRAMES[-1] + 1):
            sim.execute(stream)
            if frame in PARITY_FRAMES:
                stream.synchronize()
                snaps[frame] = (sim.downloadGrid(), sim.downloadParticles(), sim.downloadPosvel())
        sim.close()
    ref = oracle.OracleSim(parts, BOX)
    frames_timed, timed_s, t0 = 0, None, time.perf_counter()
    compare_s = 0.0  # comparisons inside the timed window are not CPU-baseline time
    results = {}
    last = PARITY_FRAMES[-1] if snaps else 10 ** 9
    for frame in range(1, last + 1):
        ref.execute(SUBSTEPS, nt)
        if timed_s is None:
            frames_timed = frame
            if time.perf_counter() - t0 - compare_s > 10.0:
                timed_s = time.perf_counter() - t0 - compare_s
                if not snaps:
                    break
        if frame in snaps:
            c0 = time.perf_counter()
            g, p, pv = snaps.pop(frame)
            results[frame] = {
                "grid": bool(np.array_equal(g, ref.cells)),
                "particles": bool(np.array_equal(p.view(np.uint32),
                                                 ref.particles.view(np.uint32))),
                "posvel": bool(np.array_equal(pv.view(np.uint32), ref.posvel.view(np.uint32)))}
            compare_s += time.perf_counter() - c0
    if timed_s is None:
        timed_s = time.perf_counter() - t0 - compare_s
    cpu = {"value": n * SUBSTEPS * frames_timed / timed_s, "unit": UNIT, "cores": nt,
           "kind": "port",
           "sample": f"the first {frames_timed} steps of the same 1M-particle workload from its "
                     f"initial state ({frames_timed * SUBSTEPS} substeps, {timed_s:.1f} s) on "
                     f"{nt} host threads"}
    parity = None
    if results:
        parity = {"vs_oracle_frames": sorted(results),
                  "vs_oracle_bit_exact": all(all(v.values()) for v in results.values()),
                  "vs_oracle": {str(k): v for k, v in sorted(results.items())},
                  "vs_oracle_what": "grid, particles and posvel of the benchmarked 1M / 128^3 "
                                    "configuration (seed 20240601) after frames 1, 5, 25, 100 "
                                    "and 200 of a fresh run, against the CPU oracle"}
    return cpu, parity


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, dist, device: str) -> float:
    """Max of a per-rank time over all ranks (identity without a process group)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, particles: int, steps: int, slowest_ms: float) -> float:
    """Whole-job particle-substeps/s when each of `world` ranks runs its own
    replica: every rank's units over the slowest rank's time."""
    return world * particles * SUBSTEPS * steps / (slowest_ms / 1e3)


def run_reference(args) -> None:
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    # Only the oracle is built and loaded here: the scene comes from its own
    # builder (bit-identical to the library's, tested), so this arm maps no
    # file of the product.
    from oracle import oracle, scene
    oracle.build()
    parts = scene.lattice(N_PER_AXIS, ORIGIN, SPACING, JITTER, SEED)
    n = len(parts)
    nt = cpu_threads()
    budget = max(30.0, min(150.0, 15.0 * args.steps))
    done, dt = time_oracle(parts, args.steps, args.warmup, budget, nt)
    value = n * SUBSTEPS * done / dt
    sample = (f"{done} of {args.steps} steps timed (1,000,000 particles x 2 substeps each) "
              f"after {args.warmup} warm-up steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / max(done, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE,
        "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": WORKLOAD, "particles": n, "grid": "128x128x128",
                   "substeps_per_step": SUBSTEPS, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture of `bench.py --quick` on this workload: its posvel-writing variant
# (profiles/k_g2p_p2g1_1M_128.md).
MEASURED_TRAFFIC_PER_LAUNCH = {"sorted_g2p_p2g_1": 93.59e6}
# ncu smsp__inst_executed.sum of one launch at the early dam-break state
# (profiles/k_g2p_p2g1_1M_128.md): the instruction-issue roofline.
MEASURED_WARP_INSTRUCTIONS_PER_LAUNCH = {"sorted_g2p_p2g_1": 70.22e6}


def algorithmic_bytes(kernel: str, n: int, cells: int) -> float | None:
    """Unique bytes a launch must read or write (each input read once, each
    output written once, an atomic counted as one write per cell and
    component); `cells` = cells holding any particle contribution."""
    if kernel == "sorted_g2p_p2g_1":
        # g2p: x in (12), x,v,C out (60); posvel (24) on the last of 2 substeps;
        # grid: raw cell in (16, updateGrid fused), next grid out (16)
        return n * (12 + 60 + 24 / SUBSTEPS) + cells * (16 + 16)
    if kernel == "sorted_p2g_2":
        # x, C in (48); mass in (4), momentum read-modify-write (12 + 12)
        return n * 48 + cells * 28
    return None


# The whole substep's algorithmic bytes as the reference's six dispatches
# define them (each stage reads its inputs once and writes its outputs once,
# an atomic result counted as one write per cell): per particle p2g_1 reads
# x, v, C (60 B), p2g_2 x, C (48), g2p x (12) and writes x, v, C (60),
# copyPosition writes pos, v (24); per grid cell (all gridCount cells, which
# clearGrid and updateGrid visit) clear 16, p2g_1 16, p2g_2 mass 4 and
# momentum read + write 24, updateGrid 16 + 12, g2p 12.
PATH_BYTES_PER_PARTICLE = 60 + 48 + 12 + 60 + 24
PATH_BYTES_PER_CELL = 16 + 16 + 4 + 24 + 16 + 12 + 12


def path_roofline(n: int, grid_cells: int, particle_substeps_per_s: float, peak: dict) -> dict:
    """The whole substep against HBM: its algorithmic bytes per substep
    times substeps per second, over the measured copy bandwidth."""
    per_substep = PATH_BYTES_PER_PARTICLE * n + PATH_BYTES_PER_CELL * grid_cells
    achieved = per_substep * (particle_substeps_per_s / n) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peak["hbm_gbs"], "peak_source": peak["source"],
            "bytes_per_substep": per_substep,
            "definition": f"({PATH_BYTES_PER_PARTICLE} B x particles + {PATH_BYTES_PER_CELL} B x "
                          "gridCount cells) per substep x substeps/s (value / particles)"}


BATCH_SCENES, BATCH_SUBSTEPS, BATCH_SEED = 256, 100, 20240601
BATCH_WORKLOAD = ("256 independent scenes, particles uniform in [4000, 64000], cubic grids of "
                  "side 32/48/64, lattice blocks at uniform origins, random gravity direction "
                  "x0.3, stiffness uniform [2, 4]; 100 substeps per rollout")


def measure_batched(pkg, torch, stream, repeats: int = 3, autotune: bool = True) -> dict:
    """Scene-substeps/s of one batch (one launch per stage for all scenes,
    CUDA graph) against looping single-scene simulators over the same scenes."""
    import numpy as np
    descs, recs = pkg.batch_scenes(BATCH_SCENES, seed=BATCH_SEED)
    S, K = len(descs), BATCH_SUBSTEPS
    batch = pkg.MLSMPMBatch(descs, recs, graph=True)
    if autotune:
        batch.autotune(4)
    tuned = batch.tuning()
    batch.step(K, stream)  # captures the graph and warms up
    stream.synchronize()
    l0 = batch.launchCount()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(repeats)]
    for a, b in evs:
        a.record(stream)
        batch.step(K, stream)
        b.record(stream)
    torch.cuda.synchronize()
    batch_ms = min(a.elapsed_time(b) for a, b in evs)
    batch_launches = (batch.launchCount() - l0) // repeats
    # the same rollout from the scenes' initial state (the blocks start above
    # rest density and spread, so the first substeps cost the most), and the
    # K substeps after it
    first_ms = next_ms = None
    for _ in range(2):
        batch.upload(recs)
        a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        a.record(stream)
        batch.step(K, stream)
        b.record(stream)
        batch.step(K, stream)
        c.record(stream)
        torch.cuda.synchronize()
        first_ms = a.elapsed_time(b) if first_ms is None else min(first_ms, a.elapsed_time(b))
        next_ms = b.elapsed_time(c) if next_ms is None else min(next_ms, b.elapsed_time(c))

    offs = np.concatenate([[0], np.cumsum([d.num_particles for d in descs])])
    sims = []
    for s, d in enumerate(descs):
        prm = pkg._lib.Params(d.stiffness, d.rest_density, d.dynamic_viscosity, d.dt,
                              d.fixed_point_multiplier)
        side = int(d.init_box[0])
        sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=d.num_particles,
                                  maxGrid=(side, side, side), params=prm)
        sim.setGravity(list(d.gravity))
        sim.upload(recs[offs[s]:offs[s + 1]], list(d.init_box))
        sims.append(sim)

    def loop_ms(graph: bool) -> float:
        for sim in sims:
            sim.setGraph(graph)
            sim.execute(stream, substeps=K)  # warm-up (and capture)
        stream.synchronize()
        best = None
        for _ in range(repeats):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for sim in sims:
                sim.execute(stream, substeps=K)
            b.record(stream)
            torch.cuda.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        return best

    plain_ms = loop_ms(False)
    graph_ms = loop_ms(True)

    def loop_initial_ms(graph: bool) -> float:
        # the same 100 substeps from the scenes' initial state (uploads
        # outside the timed region), best of 2
        best = None
        for _ in range(2):
            for s, sim in enumerate(sims):
                sim.setGraph(graph)
                sim.upload(recs[offs[s]:offs[s + 1]], list(descs[s].init_box))
            stream.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for sim in sims:
                sim.execute(stream, substeps=K)
            b.record(stream)
            torch.cuda.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        return best

    plain_first_ms = loop_initial_ms(False)
    graph_first_ms = loop_initial_ms(True)
    for sim in sims:
        sim.close()
    batch.close()
    # parity: the first four scenes as a fresh batch vs fresh single-scene
    # simulators, one rollout each
    fresh = pkg.MLSMPMBatch(descs[:4], recs[:offs[4]], graph=True)
    fresh.step(K, stream)
    stream.synchronize()
    got = fresh.downloadParticles()
    fresh.close()
    exact = True
    for s in range(4):
        d = descs[s]
        prm = pkg._lib.Params(d.stiffness, d.rest_density, d.dynamic_viscosity, d.dt,
                              d.fixed_point_multiplier)
        side = int(d.init_box[0])
        sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=d.num_particles,
                                  maxGrid=(side, side, side), params=prm)
        sim.setGravity(list(d.gravity))
        sim.upload(recs[offs[s]:offs[s + 1]], list(d.init_box))
        sim.execute(stream, substeps=K)
        exact &= bool(np.array_equal(got[offs[s]:offs[s + 1]].view(np.uint32),
                                     sim.downloadParticles().view(np.uint32)))
        sim.close()
    total = int(offs[-1])
    return {
        "workload": BATCH_WORKLOAD, "scenes": S, "particles": total, "substeps": K,
        "seed": BATCH_SEED,
        "scene_substeps_per_s": S * K / (batch_ms / 1e3),
        "particle_substeps_per_s": total * K / (batch_ms / 1e3),
        "ms_per_rollout": batch_ms,
        "gpu_launches_per_rollout": batch_launches,
        "loop_plain_scene_substeps_per_s": S * K / (plain_ms / 1e3),
        "loop_graph_scene_substeps_per_s": S * K / (graph_ms / 1e3),
        "speedup_vs_loop_plain": plain_ms / batch_ms,
        "speedup_vs_loop_graph": graph_ms / batch_ms,
        "bit_exact_vs_single_scene": bool(exact),
        "batch_autotune": tuned,
        "from_initial_state": {"ms_per_rollout": first_ms,
                               "scene_substeps_per_s": S * K / (first_ms / 1e3),
                               "particle_substeps_per_s": total * K / (first_ms / 1e3),
                               "fraction_of_warmed_rate": batch_ms / first_ms,
                               "next_ms_per_rollout": next_ms,
                               "fraction_of_next_rollout_rate": next_ms / first_ms,
                               "loop_plain_ms": plain_first_ms,
                               "loop_graph_ms": graph_first_ms,
                               "speedup_vs_loop_plain": plain_first_ms / first_ms,
                               "speedup_vs_loop_graph": graph_first_ms / first_ms},
        "timing": f"CUDA events around each {K}-substep rollout, best of {repeats}, after a "
                  f"{K}-substep warm-up (batch and loop over the same substeps); "
                  "loop = MLSMPMSimulator.execute(substeps=100) per scene, back to back "
                  "(default task size and lane table; the batch's are autotuned on its initial "
                  "state); from_initial_state: the first 100 substeps after an upload, best of 2 "
                  "(next_ms_per_rollout: substeps 100-200 after the upload)",
    }


ADJ_WORKLOAD = ("32,768 particles (32^3 jittered lattice, spacing 0.5, origin 8) in a 48^3 grid, "
                "velocities N(0, 0.1), 200 substeps, checkpoint every 20, centroid loss to "
                "(30, 10, 30), gradients w.r.t. initial state, stiffness and viscosity")


def measure_adjoint(pkg, torch, repeats: int = 3) -> dict:
    """Forward (with checkpoints) and backward times of the differentiable
    configuration, for both tapes, against the plain solver's forward."""
    import numpy as np
    recs = pkg.scene_lattice(32, 8.0, 0.5, 0.05, 3)
    rng = np.random.default_rng(1)
    recs[:, 4:7] = rng.normal(0.0, 0.1, (len(recs), 3)).astype(np.float32)
    box, T = [48.0, 48.0, 48.0], 200
    out = {"workload": ADJ_WORKLOAD, "substeps": T}
    # the plain solver over the same substeps from the same initial state
    # (upload included, as in the checkpointed forward), graph captured first
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(recs), maxGrid=(48, 48, 48))
    sim.upload(recs, box)
    sim.setGraph(True)
    sim.autotune(8)
    sim.upload(recs, box)
    sim.execute(substeps=T)
    sim.synchronize()
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        sim.upload(recs, box)
        sim.execute(substeps=T)
        sim.synchronize()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    out["plain_forward_ms"] = 1e3 * best
    sim.close()
    for name, tape, every in (("fixed", "fixed", 20), ("fp64", "fp64", 20),
                              ("fixed_full_tape", "fixed", 1)):
        adj = pkg.MLSMPMAdjoint([pkg.scene_desc(len(recs), box)], T, every, tape=tape)
        fwd = bwd = None
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            adj.forward(recs, T)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            _, seed = pkg.centroid_loss(adj.state(T), [30.0, 10.0, 30.0])
            t2 = time.perf_counter()
            adj.backward({T: seed})
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            fwd = t1 - t0 if fwd is None else min(fwd, t1 - t0)
            bwd = t3 - t2 if bwd is None else min(bwd, t3 - t2)
        adj.close()
        out[name] = {"checkpoint_every": every, "forward_ms": 1e3 * fwd, "backward_ms": 1e3 * bwd,
                     "fwd_plus_adj_over_own_forward": (fwd + bwd) / fwd,
                     "fwd_plus_adj_over_plain_forward": (fwd + bwd) / best}
    # the inverse problem's scale: 64 scenes, 1.5M particles, 100 substeps
    descs, recs64, _ = pkg.inverse.inverse_scenes(64, seed=BATCH_SEED)
    b = pkg.MLSMPMBatch(descs, recs64)
    b.step(100)
    plain64 = None
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.upload(recs64)
        b.step(100)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        plain64 = dt if plain64 is None else min(plain64, dt)
    b.close()
    seed = np.zeros((len(recs64), 20), np.float32)
    seed[:, 0:3] = 1e-6
    # checkpoints every 20 substeps (the backward recomputes 4 of the 5
    # segments), and the full tape (every substep's state and grid kept:
    # ~24 GB at this size; no recompute)
    for name, every in (("batch_64_scenes", 20), ("batch_64_scenes_full_tape", 1)):
        adj = pkg.MLSMPMAdjoint(descs, 100, every, tape="fixed")
        fwd = bwd = None
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            adj.forward(recs64, 100)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            adj.backward({100: seed})
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            fwd = t1 - t0 if fwd is None else min(fwd, t1 - t0)
            bwd = t2 - t1 if bwd is None else min(bwd, t2 - t1)
        adj.close()
        out[name] = {
            "particles": int(len(recs64)), "substeps": 100, "tape": "fixed",
            "checkpoint_every": every,
            "plain_batched_forward_ms": 1e3 * plain64,
            "forward_ms": 1e3 * fwd, "backward_ms": 1e3 * bwd,
            "fwd_plus_adj_over_own_forward": (fwd + bwd) / fwd,
            "fwd_plus_adj_over_plain_forward": (fwd + bwd) / plain64,
            "note": "forward_ms and plain_batched_forward_ms include uploading the initial state "
                    "from host memory"}
    out["timing"] = ("host wall clock around synchronised calls, best of "
                     f"{repeats}; plain forward = upload of the same initial state + "
                     "MLSMPMSimulator.execute(substeps=200) (CUDA graph, autotuned task size and "
                     "lane-table threshold), "
                     "batch: upload + MLSMPMBatch.step(100)")
    return out


def measure_inverse(pkg) -> dict:
    """The batched inverse problem: 64 scenes, 16k-32k particles, 48^3
    grids, hidden stiffness / viscosity, 100-substep rollouts, 50 Adam
    iterations of batched forward + adjoint."""
    import numpy as np
    # full tape (every substep's state and grid kept, ~24 GB): no recompute
    r = pkg.inverse.run_inverse_problem(64, seed=BATCH_SEED, substeps=100, iters=50,
                                        checkpoint_every=1)
    rel = r["rel_err"]
    h = r["history"]
    return {"scenes": r["scenes"], "particles": r["particles"], "substeps": 100,
            "iterations": 50, "tape": "fixed", "checkpoint_every": 1,
            "observed_substeps": [20, 40, 60, 80, 100],
            "seconds": r["seconds"], "ms_per_iteration": 1e3 * r["seconds"] / 50,
            "stiffness_rel_err_median": float(np.median(rel[:, 0])),
            "stiffness_rel_err_max": float(rel[:, 0].max()),
            "viscosity_rel_err_median": float(np.median(rel[:, 1])),
            "viscosity_rel_err_max": float(rel[:, 1].max()),
            "loss_first": float(h[0]["loss"].mean()), "loss_last": float(h[-1]["loss"].mean()),
            "loss": "per scene, mean squared distance to the observed positions summed over the "
                    "observed substeps; loss and seeds computed on the device "
                    "(MLSMPMAdjoint.observationLoss / backwardObserved)",
            "timing": "host wall clock around the 50 iterations (scene constants, forward with "
                      "the full tape, loss, backward, Adam step)"}


def measure_render(pkg, torch, frames: int = 10) -> dict:
    """Headless renderer (depth/thickness splats, 8 bilateral + 2 gaussian
    passes, shading): ms per frame for the reference's default scene
    (70,000 particles in 40x30x60, 60 frames in, camera distance 70) at
    896x504 (a 1280x720 canvas at main.ts's 0.7 pixel ratio), and for the
    1M-particle lattice at 1344x756."""
    import math
    out = {}
    fov = 45 * math.pi / 180
    cases = [("default_scene_70k_896x504", 70000, [40.0, 30.0, 60.0], 896, 504, 70.0, 60),
             ("lattice_1M_1344x756", None, BOX, 1344, 756, 160.0, 5)]
    for name, n_req, box, W, H, dist, warm in cases:
        if n_req is None:
            parts = make_scene(pkg)
            sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=len(parts),
                                      maxGrid=(128, 128, 128))
            sim.upload(parts, box)
            target = [29.0, 20.0, 29.0]
        else:
            sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=200000)
            sim.reset(n_req, box)
            target = [box[0] / 2, box[1] / 4, box[2] / 2]
        for _ in range(warm):
            sim.execute()
        r = pkg.FluidRenderer(W, H)
        u = pkg.camera_uniforms(W, H, dist, target, fov, 1.2)
        stream = torch.cuda.current_stream()
        for _ in range(3):
            r.execute(sim, sim.numParticles, u, stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(frames):
            r.execute(sim, sim.numParticles, u, stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / frames
        depth = r.download("depth")
        out[name] = {"particles": sim.numParticles, "width": W, "height": H,
                     "ms_per_frame": ms, "frames_per_s": 1e3 / ms,
                     "fluid_pixel_fraction": float((depth > 0).mean())}
        r.close()
        sim.close()
    out["timing"] = f"CUDA events around {frames} frames after 3 warm-up frames"
    return out


def measure_sph(pkg, torch, frames: int = 50) -> dict:
    """SPH solver: particle-substeps/s at the reference's largest UI setting
    (40,000 particles, half box 1.4 x 2.0 x 1.4, main.ts:130-131) and at
    400,000 particles (half box 1.9 x 2.0 x 1.9), after 20 frames."""
    out = {}
    for name, n, half in (("ui_max_40k", 40000, [1.4, 2.0, 1.4]),
                          ("400k", 400000, [1.9, 2.0, 1.9])):
        sim = pkg.SPHSimulator(None, None, 0.08, maxParticles=n)
        sim.reset(n, half)
        stream = torch.cuda.current_stream()
        for _ in range(20):
            sim.execute(stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(frames):
            sim.execute(stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / frames
        out[name] = {"particles": sim.numParticles, "ms_per_frame": ms,
                     "particle_substeps_per_s": sim.numParticles * 2 / (ms / 1e3)}
        sim.close()
    out["timing"] = f"CUDA events around {frames} frames (2 substeps each) after 20"
    return out


C0_WORKLOAD = ("jittered lattice dam-break: 64,000 particles (40^3, spacing 0.5, jitter +-0.05, "
               "filling [3,23)^3), 64^3 grid, 2 substeps/step")


def measure_c0(pkg, torch, stream, steps: int = 50, warmup: int = 5,
               autotune: bool = True) -> dict:
    """The 64,000-particle / 64^3 configuration (the reference's scale:
    its UI tops out at 200,000 particles on a 64^3 grid): device-resident
    particle-substeps/s over `steps` steps after `warmup`, per-step CUDA
    events (inputs far below L2 size, so no flush), and the configuration's
    whole 100-frame run from the initial state.  Autotuned like the 1M
    workload (block size, task size, z-pair and lane-table thresholds) unless
    autotune is False."""
    parts = pkg.scene_lattice(40, 3.0, SPACING, JITTER, SEED)
    box = [64.0, 64.0, 64.0]
    n = len(parts)
    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=n, maxGrid=(64, 64, 64))
    sim.upload(parts, box)
    for _ in range(warmup):
        sim.execute(stream)
    stream.synchronize()
    default_tuning = sim.tuning()
    if autotune:
        sim.autotune(8)  # as the 1M workload: on the state after the warm-up, which it keeps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for a, b in ev:
        a.record(stream)
        sim.execute(stream)
        b.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    sim.upload(parts, box)
    stream.synchronize()
    fa, fb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fa.record(stream)
    for _ in range(100):
        sim.execute(stream)
    fb.record(stream)
    torch.cuda.synchronize()
    full_ms = fa.elapsed_time(fb)
    sim_tuning = sim.tuning()
    sim.close()
    return {"workload": C0_WORKLOAD, "particles": n, "steps": steps, "warmup": warmup,
            "tuning": sim_tuning, "default_tuning": default_tuning,
            "ms_per_step": ms / steps,
            "particle_substeps_per_s": n * SUBSTEPS * steps / (ms / 1e3),
            "full_100_frame_run": {"ms": full_ms,
                                   "particle_substeps_per_s": n * SUBSTEPS * 100 / (full_ms / 1e3)},
            "timing": "CUDA events per step on the launch stream (CUDA graph), summed; "
                      "full run: one event pair around 100 execute() calls from the upload"}


def measure_expanding(pkg, torch, substeps: int = 40) -> dict:
    """The inverse problem's 64 scenes (1.52M particles) stepped from their
    initial state without CUDA graphs (one launch per kernel, each timed with
    CUDA events): the blocks expand over the rollout, bricks hold fewer
    particles and later substeps cost more.  Reports the p2g_2 kernel and the
    whole substep at substeps 2 and `substeps`."""
    descs, recs, _ = pkg.inverse.inverse_scenes(64, seed=BATCH_SEED)
    b = pkg.MLSMPMBatch(descs, recs, graph=False)
    b.autotune(4)  # on the initial state, which it restores
    tuned = b.tuning()
    per = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(substeps):
        b.setProfiling(True)  # resets the counters
        b.step(1)
        st = b.kernelStats()
        per.append((st.get("sorted_p2g_2", (0, 0, 0.0))[2], sum(v[2] for v in st.values())))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    b.setProfiling(False)
    out = {"particles": int(b.numParticles), "substeps": substeps,
           "wall_ms_profiled": 1e3 * dt, "health_ok": bool(b.checkHealth()["ok"]),
           "p2g2_ms_substep_2": per[1][0], f"p2g2_ms_substep_{substeps}": per[-1][0],
           "p2g2_ratio": per[-1][0] / per[1][0],
           "substep_ms_substep_2": per[1][1], f"substep_ms_substep_{substeps}": per[-1][1],
           "substep_ratio": per[-1][1] / per[1][1], "autotune": tuned,
           "timing": "CUDA events around each kernel of the substep (no CUDA graph)"}
    b.close()
    return out


def measure_batch_windows(pkg, torch) -> dict:
    """Per-kernel device ms per substep of the 256-scene batch in four
    windows of its rollout from the initial state (no CUDA graph, CUDA events
    around each launch): substeps 0-10 (dense blocks), 55-65 (spread, most
    bricks), 150-160 and 290-300 (settling).  The tuning is fixed at the
    choice the autotuner makes for this batch on its initial state (every z
    pair merged, 128-thread blocks, tasks of up to 1024 particles, lane table
    from 32), so that the kernel launches are the same in every run."""
    descs, recs = pkg.batch_scenes(BATCH_SCENES, seed=BATCH_SEED)
    b = pkg.MLSMPMBatch(descs, recs, graph=False)
    b.binPairing = 1 << 30
    b.taskThreads = 128
    b.setTaskSize(1024)
    b.laneTableMin = 32
    out = {"scenes": len(descs), "particles": int(b.numParticles), "tuning": b.tuning(),
           "timing": "CUDA events around each launch, ms per substep (no CUDA graph)"}
    done = 0
    for lo, hi in ((0, 10), (55, 65), (150, 160), (290, 300)):
        if done < lo:
            b.step(lo - done)
        torch.cuda.synchronize()
        b.setProfiling(True)  # resets the counters
        b.step(hi - lo)
        torch.cuda.synchronize()
        st = b.kernelStats()
        b.setProfiling(False)
        done = hi
        row = {k: v[2] / (hi - lo) for k, v in st.items() if v[1]}
        row["total"] = sum(v[2] for v in st.values()) / (hi - lo)
        out[f"substeps_{lo}_{hi}"] = row
    b.close()
    return out


def measure_adjoint_batch(pkg, torch, substeps: int = 40, every: int = 10) -> dict:
    """One checkpointed forward and backward of the inverse problem's 64
    scenes (1.52M particles) on the fixed-point tape (for kernel profiles)."""
    import numpy as np
    descs, recs, _ = pkg.inverse.inverse_scenes(64, seed=BATCH_SEED)
    adj = pkg.MLSMPMAdjoint(descs, substeps, every, tape="fixed")
    seed = np.zeros((len(recs), 20), np.float32)
    seed[:, 0:3] = 1e-6
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    adj.forward(recs, substeps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g, _ = adj.backward({substeps: seed})
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    adj.close()
    return {"particles": int(len(recs)), "substeps": substeps, "checkpoint_every": every,
            "forward_ms": 1e3 * (t1 - t0), "backward_ms": 1e3 * (t2 - t1),
            "grad_finite": bool(np.isfinite(g).all())}


def run_only(which: str, autotune: bool = True) -> None:
    import torch
    import __graft_entry__ as entry
    entry.build()
    pkg = entry.load_package()
    if which == "batched":
        out = measure_batched(pkg, torch, torch.cuda.Stream(), autotune=autotune)
    elif which == "adjoint":
        out = measure_adjoint(pkg, torch)
    elif which == "render":
        out = measure_render(pkg, torch)
    elif which == "sph":
        out = measure_sph(pkg, torch)
    elif which == "expanding":
        out = measure_expanding(pkg, torch)
    elif which == "adjoint_batch":
        out = measure_adjoint_batch(pkg, torch)
    elif which == "batch_windows":
        out = measure_batch_windows(pkg, torch)
    else:
        out = measure_inverse(pkg)
    print(json.dumps({"only": which, which: out}), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__ as entry
    entry.build()
    pkg = entry.load_package()
    parts = make_scene(pkg)
    n = len(parts)

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        return reduce_max(x, dist, "cuda")

    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    sim = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=n, maxGrid=(128, 128, 128))
    sim.upload(parts, BOX)
    for _ in range(args.warmup):
        sim.execute(stream)
    stream.synchronize()
    # task size and lane-table threshold tuned on the state the timed steps
    # start from (the autotuner restores it), then the same start again so
    # the graphs of the chosen configuration are captured before timing
    if args.no_autotune:
        tuned = {**sim.tuning(), "autotune": "off (engine defaults)"}
    else:
        sim.autotune(AUTOTUNE_SUBSTEPS)
        tuned = {**sim.tuning(),
                 "autotune": f"{AUTOTUNE_SUBSTEPS} substeps after the warm-up steps, over "
                             "z-pair thresholds {0, 256, 512, all} x task-kernel block sizes "
                             "{128, 256, 512} x task sizes {128 ... 1024} x lane-table "
                             "thresholds {32, 128, 512, off}"}
        sim.upload(parts, BOX)
        for _ in range(args.warmup):
            sim.execute(stream)
        stream.synchronize()

    # --- timed region: device-resident throughput ----------------------
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    launches0 = sim.launchCount()
    wall0 = time.perf_counter()
    for i in range(K):
        flush_l2()
        ev[i][0].record(stream)
        sim.execute(stream)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    launches = sim.launchCount() - launches0
    clocks = sampler.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    dev_ms = max_over_ranks(dev_ms)
    value = replica_throughput(world, n, K, dev_ms)

    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                              "steps": K, "warmup": args.warmup, "ms_per_step": dev_ms / K,
                              "quick": True, "gpu_launches": launches}), flush=True)
        sim.close()
        if dist is not None:
            dist.destroy_process_group()
        return

    # Every later pass restarts from the same state as the timed region (the
    # dam-break slows down as the block spreads): upload, the same warm-up.
    def restart():
        sim.upload(parts, BOX)
        for _ in range(args.warmup):
            sim.execute(stream)
        stream.synchronize()

    # --- per-kernel timing pass (roofline) ------------------------------
    restart()
    sim.setProfiling(True)
    for i in range(K):
        flush_l2()
        sim.execute(stream)
    stream.synchronize()
    stats = sim.kernelStats()
    sim.setProfiling(False)
    grid = sim.downloadGrid()
    cells = int(np.count_nonzero(grid.any(axis=1)))
    top = max(stats.items(), key=lambda kv: kv[1][2])
    top_name, (top_launches, top_timed, top_ms) = top
    peaks = measured_peaks()
    step_kernel_ms = sum(v[2] for v in stats.values())
    roof = None
    abytes = algorithmic_bytes(top_name, n, cells)
    if abytes is not None and top_timed:
        avg_s = top_ms / top_timed / 1e3
        achieved = abytes / avg_s / 1e9
        roof = {"bound": "hbm", "kernel": top_name, "achieved": achieved,
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": MEASURED_TRAFFIC_PER_LAUNCH.get(top_name),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                  "profiles/k_g2p_p2g1_1M_128.md",
                "algorithmic_bytes_per_launch": abytes,
                "mean_launch_us": avg_s * 1e6, "cells_touched": cells,
                "kernel_share": top_ms / step_kernel_ms if step_kernel_ms else None}
    # The kernel is bound by instruction issue and latency, not DRAM: its
    # warp-instructions per launch over the same mean duration, against 4
    # issues per SM per cycle at the sampled SM clock.
    issue = None
    instr = MEASURED_WARP_INSTRUCTIONS_PER_LAUNCH.get(top_name)
    if roof is not None and instr and clocks.get("sm_mhz"):
        nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        peak_issue = 4.0 * nsm * clocks["sm_mhz"] * 1e6
        got = instr / (roof["mean_launch_us"] * 1e-6)
        issue = {"kernel": top_name, "achieved": got / 1e12, "peak": peak_issue / 1e12,
                 "unit": "T warp-instructions/s", "frac": got / peak_issue,
                 "warp_instructions_per_launch": instr,
                 "source": "ncu smsp__inst_executed.sum of one early-state launch, "
                           "profiles/k_g2p_p2g1_1M_128.md; peak = 4 x SMs x median SM clock"}
    kernels = {k: {"launches": v[0], "mean_us": 1e3 * v[2] / v[1] if v[1] else None,
                   "share": v[2] / step_kernel_ms if step_kernel_ms else None}
               for k, v in stats.items()}

    # --- the whole 200-frame run of the 1M configuration -------------------
    # (from the initial state; the block spreads and later frames are slower
    # than the timed window above, so this is the run's average)
    restart_frames = 200
    sim.upload(parts, BOX)
    stream.synchronize()
    flush_l2()
    fa, fb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fa.record(stream)
    for _ in range(restart_frames):
        sim.execute(stream)
    fb.record(stream)
    torch.cuda.synchronize()
    full_ms = max_over_ranks(fa.elapsed_time(fb))
    full_run = {"frames": restart_frames, "ms": full_ms,
                "value": replica_throughput(world, n, restart_frames, full_ms),
                "timing": "one event pair around 200 execute() calls from the uploaded "
                          "initial state, CUDA graph, no L2 flush between frames"}

    # --- e2e through the public API with host buffers --------------------
    pinned = torch.empty((n, 8), dtype=torch.float32, pin_memory=True)
    host_out = pinned.numpy()
    box_host = list(BOX)
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(K)]
    restart()
    barrier()
    torch.cuda.synchronize()
    for i in range(K):
        flush_l2()
        ev2[i][0].record(stream)
        sim.changeBoxSize(box_host)
        sim.execute(stream)
        sim.downloadPosvel(stream, out=host_out)
        ev2[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_serial_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev2))
    e2e_serial = replica_throughput(world, n, K, e2e_serial_ms)
    assert np.isfinite(host_out[:, 0:3]).all(), "posvel read back non-finite positions"

    # the same frame loop pipelined as a renderer would run it: each step's
    # posvel is snapshotted and copied to one of two pinned host buffers on
    # the library's copy stream while the next step computes; one pair of
    # events spans all K steps and the last copy.  No L2 flush between steps:
    # a step streams ~300 MB (both particle buffers, the grids, posvel)
    # through the 129 MB L2.
    hosts = [torch.empty((n, 8), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    e_start = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    restart()
    flush_l2()
    barrier()
    torch.cuda.synchronize()
    e_start.record(stream)
    for i in range(K):
        sim.changeBoxSize(box_host)
        sim.execute(stream)
        sim.downloadPosvelAsync(stream, out=hosts[i % 2])
    sim.waitPosvel(stream)
    e_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = max_over_ranks(e_start.elapsed_time(e_end))
    e2e_value = replica_throughput(world, n, K, e2e_ms)
    assert np.isfinite(hosts[(K - 1) % 2][:, 0:3]).all(), "posvel read back non-finite positions"
    sim.close()

    c0 = measure_c0(pkg, torch, stream, autotune=not args.no_autotune)
    batched = None if args.skip_batched else measure_batched(pkg, torch, stream,
                                                             autotune=not args.no_autotune)
    adjoint = None if args.skip_adjoint else measure_adjoint(pkg, torch)
    inverse = None if args.skip_adjoint else measure_inverse(pkg)
    expanding = measure_expanding(pkg, torch)
    render = None if args.skip_batched else measure_render(pkg, torch)
    sph = None if args.skip_batched else measure_sph(pkg, torch)

    # --- bit-exactness self-check: sorted engine vs dispatch engine -------
    outs = []
    for engine in ("sorted", "dispatch"):
        s2 = pkg.MLSMPMSimulator(None, None, 1.2, maxParticles=n, maxGrid=(128, 128, 128))
        s2.engine = engine
        s2.upload(parts, BOX)
        for _ in range(3):
            s2.execute(stream)
        stream.synchronize()
        outs.append((s2.downloadGrid(), s2.downloadParticles()))
        s2.close()
    grid_exact = bool(np.array_equal(outs[0][0], outs[1][0]))
    parts_exact = bool(np.array_equal(outs[0][1].view(np.uint32), outs[1][1].view(np.uint32)))

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    cpu = None
    vs_oracle = None
    if world == 1 and not args.no_cpu_baseline:
        cpu, vs_oracle = cpu_baseline_and_parity(pkg, parts, stream, args.no_parity)
        cpu["detail"] = cpu_baseline_detail(pkg)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": dev_ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
        "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": WORKLOAD, "particles": n, "grid": "128x128x128",
                   "substeps_per_step": SUBSTEPS, "engine": "sorted", **tuned,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "flushed between timed steps (256 MiB write, outside the events)",
                   "timing": "CUDA events per step on the launch stream, summed"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 12,
                "d2h_bytes_per_step": 32 * n,
                "api": ("changeBoxSize(host) + execute() + downloadPosvelAsync() into two "
                        "alternating pinned host buffers (the copy of step i overlaps step i+1); "
                        "one event pair around all steps and the last copy"),
                "l2": "not flushed between steps: each step streams ~300 MB through the 129 MB L2",
                "serialized_value": e2e_serial,
                "serialized_api": ("changeBoxSize(host) + execute() + downloadPosvel() into pinned "
                                   "host memory, per-step events, L2 flushed outside them")},
        "roofline": roof,
        "path_roofline": path_roofline(n, 128 ** 3, value, peaks),
        "cpu_baseline": cpu,
        "clocks": clocks,
        "issue_roofline": issue,
        "full_200_frame_run": full_run,
        "c0_64k_64": c0,
        "gpu_launches": launches,
        "wall_s_timed_region": wall,
        "kernels": kernels,
        "batched": batched,
        "expanding_batch": expanding,
        "adjoint": adjoint,
        "inverse_problem": inverse,
        "render": render,
        "sph": sph,
        "parity": {**(vs_oracle or {"vs_oracle": "not run"}),
                   "engines": {"grid_bit_exact_vs_dispatch_engine": grid_exact,
                               "particles_bit_exact_vs_dispatch_engine": parts_exact,
                               "steps": 3}},
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="leave out the CPU oracle (its timed sample and the 200-frame parity run)")
    ap.add_argument("--no-parity", action="store_true",
                    help="time the CPU baseline only; skip the 200-frame comparison with the oracle")
    ap.add_argument("--skip-batched", action="store_true",
                    help="leave out the batched-scenes measurement")
    ap.add_argument("--skip-adjoint", action="store_true",
                    help="leave out the adjoint and inverse-problem measurements")
    ap.add_argument("--only", choices=["batched", "adjoint", "inverse", "render", "sph",
                                       "expanding", "adjoint_batch", "batch_windows"],
                    help="run one side measurement alone and print its JSON (profiling)")
    ap.add_argument("--quick", action="store_true",
                    help="time the device-resident steps only (for profiler captures)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the engine's default block size, task size and lane-table "
                         "threshold (the configuration of the committed ncu captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.only:
        run_only(args.only, autotune=not args.no_autotune)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
