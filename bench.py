"""Benchmark: particle-steps/s of the PBF step at 1,048,576 particles, 4 iterations.

Workload (the reference's 1M configuration): seeded 128x128x64 dam-break
lattice, spacing 0.5h, box 12.8x6.4x6.4, h = 0.1, rho0 = 6378, 1 substep,
4 solver iterations, s_corr n = 4 dq = 0.2h, eps = 600, gravity -9.8, with
dt = 1/120 per step and the reference benchmark's s_corr k = 1e-4, XSPH
1e-5 and vorticity 1e-5 (the configured dt = 1/60, k = 0.1, XSPH 0.01 and
vorticity 1e-4 diverge in the reference's own update).  One step = one
step() call.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value     K steps replayed from HBM-resident state, CUDA events on the
          launching stream, synchronize on both sides; N ranks = N
          independent replicas (one process per GPU, no collective on the
          data path), value = all ranks' particle-steps / max rank time.
e2e       the same metric through the public API with host buffers: every step
          uploads positions+velocities from pinned host memory
          (pbf_set_particles), steps, and downloads positions+velocities to
          pinned host memory.
roofline  dominant kernel of the step, timed live with CUDA events captured
          in the frame graph, against the measured HBM copy bandwidth.
vs_baseline  value over the reference's own CUDA kernels on the same GPU,
          same workload and the same frames (the metric's comparison).
--impl reference  the CPU restatement of the reference step (the reference
          has no CPU implementation) on all host cores, over the same warm-up
          and timed steps when they fit PBF_REF_SECONDS, else a bounded sample.
"""

from __future__ import annotations

import argparse
import importlib
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M (4 iters)"
UNIT = "particle-steps/s"
WORKLOAD = ("dam_break_1m: 1,048,576 particles (128x128x64 lattice, spacing 0.5h, jitter "
            "+-0.01h seed 0) in a 12.8x6.4x6.4 box, h=0.1, rho0=6378, dt=1/120 per step, "
            "1 substep, 4 iterations, scorr k=1e-4 n=4 dq=0.2h, eps=600, xsph 1e-5, "
            "vorticity 1e-5, friction 0.03, 256 neighbour slots")
# Algorithmic bytes per particle-step: 492 + I*(128 + 8C) + 8C with I = 4
# iterations and C = cells/particle (minimal compulsory traffic: integrate,
# hash, counting sort, reorder, lambda, delta-p + apply, final rebuild, the
# one-time gather and the four velocity stages).
def b_alg(iters: int, cells_per_particle: float) -> float:
    return 492.0 + iters * (128.0 + 8.0 * cells_per_particle) + 8.0 * cells_per_particle


# Algorithmic bytes per particle of each stage (same accounting; neighbour
# data staged on chip, lists counted as zero).
STAGE_BYTES = {
    "predict": 64.0 + 20.0,          # R x, v; W x*, v_in; + hash of the first rebuild
    "sort": 8.0,                      # R key, W permutation
    "gather_ranges": 46.0,            # R perm, R/W x*, R/W composed permutation, first[]
    "search_lambda": 24.0,            # R x*, W lambda, W count
    "delta_apply_collide": 56.0,      # R x*, R lambda, W x* + next hash
    "search_final": 20.0 + 48.0,     # walk + XSPH pass (R x*, v; W count, v)
    "finalize": 68.0,
    "xsph": 48.0,
    "vorticity": 48.0,
    "confine_resolve": 64.0,
}


# ncu captures of the dominant kernel (k_search<1>: walk + lambda) on the
# 1M dam break, keyed by frame: the mean over the frame's four launches of
# DRAM bytes read + written (dram__bytes_read.sum + dram__bytes_write.sum)
# and warp instructions (smsp__inst_executed.sum), from
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,smsp__inst_executed.sum,
#       gpu__time_duration.sum --clock-control none --kernel-name-base demangled
#       -k 'regex:k_search<.bool.1' -s <4 (F - 1)> -c 4
#       python fluid-simulator_gb300/profile_report.py --child --scene dam_break_1m
#       --warmup <F - 1>
# A timed window is matched with the capture nearest its middle frame; the
# line names that frame.
CAPTURES = {
    "search_lambda": {
        16: {"dram_bytes": 60.676864e6 + 94.141632e6, "inst": 163705114.0},
        106: {"dram_bytes": 111.414400e6 + 199.216960e6, "inst": 245673552.0},
        150: {"dram_bytes": 95.744576e6 + 158.054208e6, "inst": 207600024.0},
    },
}
SMS, ISSUE_PER_SM_CLK = 152, 4


def capture_for(kernel, scene, mid_frame):
    """The capture of `kernel` nearest frame `mid_frame` of the 1M dam break."""
    caps = CAPTURES.get(kernel) if scene == "dam_break_1m" else None
    if not caps:
        return None, None
    frame = min(caps, key=lambda f: abs(f - mid_frame))
    return frame, caps[frame]


def issue_roofline(kernel, ms_per_launch, clocks, scene, mid_frame):
    """Warp instructions per second of the dominant kernel against the SMs'
    issue peak (4 per SM per clock at the SM clock sampled while timing),
    with the instruction count of the capture nearest the timed window."""
    frame, cap = capture_for(kernel, scene, mid_frame)
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not cap or not mhz:
        return None
    achieved = cap["inst"] / (ms_per_launch / 1000.0) / 1e9
    peak = SMS * ISSUE_PER_SM_CLK * mhz * 1e6 / 1e9
    return {"bound": "issue", "kernel": kernel, "achieved": achieved, "peak": peak,
            "unit": "G warp-instructions/s", "frac": achieved / peak,
            "inst_per_launch": cap["inst"], "captured_at_frame": frame,
            "window_mid_frame": mid_frame,
            "source": "smsp__inst_executed.sum, mean of the frame's four launches in one ncu capture (--clock-control none)"}


def load_pkg():
    name = "fluid_simulator_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "fluid-simulator_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "pbf_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        load = [v for v in sm if smax and v > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def setup_dist(world, local):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cuda_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


def pinned_like(a: np.ndarray):
    """A pinned host copy of `a` (torch pin_memory), as a numpy view."""
    try:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t, t.numpy()
    except Exception:
        return None, np.ascontiguousarray(a).copy()


def cpu_baseline(scene, seconds_budget: float = 20.0, threads: int = 0, warmup: int = 1,
                 steps: int = 0):
    """FP32 restatement of the reference step (oracle, OpenMP) on the host cores.

    `warmup` untimed steps, then `steps` timed steps (the GPU arm's window);
    when those would take longer than `seconds_budget` (estimated from the
    first warm-up step), or when steps == 0, as many steps as fit the budget.
    The line reports the steps actually timed."""
    from oracle import oracle as O
    pos, vel, mn, mx, prm, _ = scene
    threads = threads or os.cpu_count() or 1
    o = O.OracleSolver(32, threads=threads)
    o.initialize(len(pos), mn, mx, prm.as_dict())
    o.set_particles(pos, vel)
    t0 = time.perf_counter()
    st = o.step()  # first warm-up step (first touch of the lists)
    first = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError("oracle step failed: %d" % st)
    for _ in range(max(warmup, 1) - 1):
        st = o.step()
        if st != 0:
            raise RuntimeError("oracle step failed: %d" % st)
    fit = max(1, int(seconds_budget / max(first, 1e-3)))
    timed = min(steps, fit) if steps > 0 else fit
    t0 = time.perf_counter()
    for _ in range(timed):
        st = o.step()
        if st != 0:
            raise RuntimeError("oracle step failed: %d" % st)
    dt = time.perf_counter() - t0
    whole = steps > 0 and timed == steps
    return {"value": len(pos) * timed / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "steps": timed, "warmup": max(warmup, 1),
            "sample": "steps %d..%d of the full %d-particle workload (%s; FP32 C++/OpenMP "
                      "restatement on %d threads, %.1f s)"
                      % (max(warmup, 1), max(warmup, 1) + timed, len(pos),
                         "the same window as the GPU arm" if whole else
                         "a bounded sample of %d steps" % timed, threads, dt)}


def density_of(positions, scene):
    """FP64 density error of a final state (oracle.density_stats): the same
    measure for this library's and the reference's positions."""
    from oracle import oracle as O
    _, _, mn, mx, prm, _ = scene
    return O.density_stats(positions, mn, mx, prm.smoothingRadius, prm.particleMass,
                           prm.restDensity)


def reference_cuda(scene, steps: int, warmup: int, max_neighbors: int = 256):
    """The reference's own kernels (compiled from its sources, Release, sm_103a)
    driven with PBFSolver's host sequence, timed like its benchmark: steady
    clock around each step() (benchmark/pbf_benchmark.cu:121-137).  Steps
    warmup .. warmup + steps of the run, the window this library is timed on;
    the density error of the final state is measured as for this library."""
    from oracle import oracle as O
    from oracle import build_ref
    if not build_ref.available():
        return {"unavailable": "reference kernels not built (oracle/_ref needs the reference "
                               "sources at build time)"}
    pos, vel, mn, mx, prm, col = scene
    r = O.RefCudaSolver()
    r.initialize(len(pos), mn, mx, prm.as_dict(), max_neighbors)
    sp = [(*c, rr) for c, rr in col.get("spheres", [])]
    bx = [(*c, *e) for c, e in col.get("boxes", [])]
    r.set_colliders(np.asarray(sp, np.float32).reshape(-1, 4),
                    np.asarray(bx, np.float32).reshape(-1, 6), np.zeros((0, 6), np.float32))
    r.set_particles(pos, vel)
    st = r.run(warmup)
    if st != 0:
        return {"unavailable": "reference step failed with status %d" % st}
    ms = r.time_steps(steps)
    final = r.positions()
    r.close()
    return {"value": len(pos) * steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / steps,
            "steps": steps, "warmup": warmup, "max_neighbors": max_neighbors,
            "density_error": density_of(final, scene),
            "method": "reference kernels compiled from its sources (-O3 -DNDEBUG, sm_103a), "
                      "PBFSolver host sequence and synchronisation, steady_clock around each "
                      "step()"}


def configured_parameters(pkg, scene, steps: int = 100):
    """The 1M lattice with the configuration's literal step parameters (one
    step of dt = 1/60, s_corr k = 0.1, XSPH c = 0.01, vorticity 1e-4): how
    far the reference's kernels and this library get before a step fails
    (neighbour overflow) and the fastest particle when they stop."""
    import dataclasses
    from oracle import oracle as O
    from oracle import build_ref
    pos, vel, mn, mx, prm, _ = scene
    cfg = dataclasses.replace(prm, dt=1.0 / 60.0, scorrK=0.1, xsphViscosity=0.01,
                              vorticityStrength=1e-4)
    out = {"params": {"dt": cfg.dt, "scorrK": cfg.scorrK, "xsphViscosity": cfg.xsphViscosity,
                      "vorticityStrength": cfg.vorticityStrength}, "max_steps": steps}

    def speed(v):
        return float(np.sqrt((v[:, :3].astype(np.float64) ** 2).sum(1).max()))

    if build_ref.available():
        r = O.RefCudaSolver()
        r.initialize(len(pos), mn, mx, cfg.as_dict())
        r.set_colliders(np.zeros((0, 4), np.float32), np.zeros((0, 6), np.float32),
                        np.zeros((0, 6), np.float32))
        r.set_particles(pos, vel)
        done, st, vmax = 0, 0, 0.0
        while done < steps:
            st = r.step()
            if st != 0:
                break
            done += 1
            if done in (1, 2, 5, 10, 20, 50, 100):
                vmax = speed(r.velocities())
        out["reference_cuda"] = {
            "steps_completed": done,
            "status": {0: "ok", 1: "error", 2: "overflow_error (neighbour capacity 256)",
                       3: "not converged"}.get(st, str(st)),
            "max_speed_before_stop": vmax}
        r.close()
    s = pkg.PBFSolver()
    s.initialize(len(pos), mn, mx, cfg)
    s.set_particles(pos, vel)
    done, err, vmax = 0, None, 0.0
    while done < steps:
        try:
            s.step()
        except pkg.PBFError as e:
            err = type(e).__name__ + ": " + str(e)[:120]
            break
        done += 1
        if done in (1, 2, 5, 10, 20, 50, 100):
            vmax = speed(s.copy_velocities_to_host())
    s.close()
    out["this_library"] = {"steps_completed": done, "status": err or "ok",
                           "max_speed_before_stop": vmax}
    return out


def reference_scene(pkg, scenes, frames: int = 60, reps: int = 5, warmup: int = 10):
    """The reference's own benchmark (benchmark/pbf_benchmark.cu:158-212):
    262,144 particles, 2 substeps x 4 iterations, box + sphere; `warmup`
    frames, then `reps` runs of `frames` frames, each from the initial state;
    the run with the median average is reported as particle-frames/s and
    particle-substeps/s.  The reference's kernels run the same scene on the
    same GPU the same way."""
    from oracle import oracle as O
    from oracle import build_ref
    pos, vel, mn, mx, prm, col = scenes.reference_benchmark()
    n = len(pos)
    sub = prm.substeps

    def summary(run_ms):
        med = sorted(run_ms)[len(run_ms) // 2]
        return {"ms_per_frame": med / frames, "runs_ms": run_ms,
                "particle_frames_per_s": n * frames / (med / 1000.0),
                "particle_substeps_per_s": n * frames * sub / (med / 1000.0)}

    s = pkg.PBFSolver()
    s.initialize(n, mn, mx, prm)
    s.set_spheres(col["spheres"])
    s.set_boxes(col["boxes"])
    s.set_particles(pos, vel)
    s.run(warmup)
    ours = []
    for _ in range(reps):
        s.set_particles(pos, vel)
        ours.append(s.time_frames(frames))
    s.close()
    out = {"particles": n, "substeps": sub, "iterations": prm.solverIterations,
           "frames": frames, "repetitions": reps, "warmup_frames": warmup,
           "ours": summary(ours)}
    out["ours_cpp_shim"] = shim_driver()
    if not build_ref.available():
        out["reference_cuda"] = {"unavailable": "reference kernels not built"}
        return out
    r = O.RefCudaSolver()
    r.initialize(n, mn, mx, prm.as_dict())
    sp = [(*c, rr) for c, rr in col["spheres"]]
    bx = [(*c, *e) for c, e in col["boxes"]]
    r.set_colliders(np.asarray(sp, np.float32).reshape(-1, 4),
                    np.asarray(bx, np.float32).reshape(-1, 6), np.zeros((0, 6), np.float32))
    r.set_particles(pos, vel)
    st = r.run(warmup)
    ref = []
    for _ in range(reps if st == 0 else 0):
        r.set_particles(pos, vel)
        ref.append(r.time_steps(frames))
    r.close()
    if st != 0:
        out["reference_cuda"] = {"unavailable": "reference step failed with status %d" % st}
        return out
    out["reference_cuda"] = summary(ref)
    out["speedup"] = (out["ours"]["particle_frames_per_s"]
                      / out["reference_cuda"]["particle_frames_per_s"])
    if "particle_frames_per_s" in out["ours_cpp_shim"]:
        out["speedup_cpp_shim"] = (out["ours_cpp_shim"]["particle_frames_per_s"]
                                   / out["reference_cuda"]["particle_frames_per_s"])
    return out


def shim_driver():
    """The same scene and protocol through the C++ shim, timed like the
    reference's driver: steady_clock around every synchronous
    PBFSolver::step() (fluid-simulator_gb300/cpp/reference_scene_bench.cpp)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_pbf103_build_b", os.path.join(ROOT, "fluid-simulator_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    try:
        exe = b.build_shim_bench()
        r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    except (RuntimeError, OSError, subprocess.TimeoutExpired) as e:
        return {"unavailable": str(e).splitlines()[0][:200]}
    if r.returncode != 0:
        return {"unavailable": "driver exited %d: %s" % (r.returncode, r.stderr.strip()[:200])}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    d["method"] = ("C++ driver on include/pbf103/pbf_solver.hpp: steady_clock around each "
                   "synchronous step(), median of 5 runs of 60 frames")
    return d


def batched(pkg, scenes, steps: int, warmup: int, per_scene_steps: int):
    """256 independent scenes (particle counts log-uniform in [2,048, 65,536])
    stepped by one batched solver -- one launch per stage for all scenes --
    against the same scenes stepped by one single-scene solver each."""
    import torch
    sc, prm, pos, vel, per = scenes.batched_scenes()
    n = len(pos)
    b = pkg.PBFSolver()
    b.initialize_batch(sc, prm)
    b.set_particles(pos, vel)
    b.run(warmup)
    tuned = b.autotune(2)
    b.run(1)
    with Clocks(0) as clk:
        ms = b.time_frames(steps)
    kernels = b.kernels_per_frame()
    density = b.density_error()
    b.close()
    value = n * steps / (ms / 1000.0)

    solvers = []
    for p, v, lo, hi, q in per:
        a = pkg.PBFSolver()
        a.initialize(len(p), lo, hi, q)
        a.set_particles(p, v)
        solvers.append(a)
    shared = torch.cuda.Stream()

    def run_all(k, one_stream):
        for a in solvers:
            a.set_stream(shared.cuda_stream if one_stream else None)
        cuda_sync()
        t0 = time.perf_counter()
        for _ in range(k):
            for a in solvers:
                a.run_async(1)
        for a in solvers:
            a.synchronize()
        return time.perf_counter() - t0

    # Each baseline takes its better walk setting: the size rule (scenes below
    # 32,768 particles split their walks over 8 or 4 lanes, best for one scene
    # at a time) or 1 lane per particle (best when many solvers share the GPU).
    timed = {}
    for lanes in (0, 1):
        for a in solvers:
            a.set_walk_lanes(lanes)
        run_all(warmup, True)   # instantiates every scene's frame graph
        run_all(warmup, False)
        timed[lanes] = (run_all(per_scene_steps, True), run_all(per_scene_steps, False))
    t_one, lanes_one = min((timed[k][0], k) for k in timed)
    t_many, lanes_many = min((timed[k][1], k) for k in timed)
    for a in solvers:
        a.close()
    lanes_name = {0: "walk lanes by scene size", 1: "one walk lane per particle"}
    one = n * per_scene_steps / t_one
    many = n * per_scene_steps / t_many
    return {
        "scenes": len(sc), "particles": n, "steps": steps, "warmup": warmup,
        "value": value, "unit": UNIT, "ms_per_step": ms / steps, "kernels_per_step": kernels,
        "gpu_launches": kernels * steps, "clocks": clk.summary(), "block_sizes": tuned,
        "density_error": {"mean": density[0], "max": density[1]},
        "per_scene_launches": {
            "value": one, "ms_per_step": 1000.0 * t_one / per_scene_steps,
            "steps": per_scene_steps,
            "method": "one single-scene solver per scene, each frame a graph launch, all on "
                      "one stream, host wall clock around the launches and the final sync; "
                      "the faster of two walk settings: " + lanes_name[lanes_one]},
        "per_scene_launches_concurrent": {
            "value": many, "ms_per_step": 1000.0 * t_many / per_scene_steps,
            "method": "same, each solver on its own stream; the faster of two walk settings: "
                      + lanes_name[lanes_many]},
        "gain": value / one,
        "gain_vs_concurrent": value / many,
        "workload": "256 dam-break scenes, counts log-uniform in [2048, 65536] (seed 7), "
                    "rho0 x U(0.9, 1.1), XSPH c ~ U(0.005, 0.05) applied as c m / rho0, "
                    "4 iterations, dt 1/120",
    }


def adjoint_bench(pkg, scenes, steps: int, every: int, ndirs: int, fd_steps: int = 5):
    """Differentiable rollout: 65,536 particles (64x64x16 lattice, the 1M
    dam break's parameters, vorticity confinement included), `steps`
    steps with checkpoints every `every`; loss = mean squared distance of the
    final positions to the initial lattice shifted +0.3 in x with
    N(0, 0.01h) noise; gradients w.r.t. v0, rest density and XSPH c.

    Two accuracy checks.  Over `steps` steps the collapsing dam is chaotic
    (its FP64 derivative grows by orders of magnitude and stops matching FP64
    central differences), so the full horizon is checked against FP64
    tangents linearised about the GPU's own trajectory (the same derivative
    on the same states).  FP64 central differences of the FP64 restatement
    check a `fd_steps`-step rollout, where the function is smooth."""
    from oracle import oracle as O
    nx, ny, nz = 64, 64, 16
    S = scenes.SPACING
    box = (2 * nx * S, 1.5 * ny * S, 2 * nz * S)
    pos, vel, mn, mx, prm, _ = scenes.dam_break(nx, ny, nz, box)
    n = len(pos)
    rng = np.random.default_rng(5)
    target = pos[:, :3].astype(np.float64) + np.array([0.3, 0.0, 0.0])
    target += rng.normal(0.0, 0.01 * scenes.H, target.shape)

    def grads(a, T):
        x, _ = a.forward(pos, vel, T)
        d = x[:, :3].astype(np.float64) - target
        gx = np.zeros((n, 4), np.float32)
        gx[:, :3] = (2.0 / n) * d
        gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
        return d, gv0[:, :3].astype(np.float64), gr, gc

    a = pkg.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=every)
    a.forward(pos, vel, steps)  # warm-up
    cuda_sync()
    t0 = time.perf_counter()
    x, v = a.forward(pos, vel, steps)
    cuda_sync()
    t_fwd = time.perf_counter() - t0
    d = x[:, :3].astype(np.float64) - target
    gx = np.zeros((n, 4), np.float32)
    gx[:, :3] = (2.0 / n) * d
    t0 = time.perf_counter()
    gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
    cuda_sync()
    t_bwd = time.perf_counter() - t0
    gv0 = gv0[:, :3].astype(np.float64)

    # Full horizon: FP64 tangents linearised about the GPU trajectory.
    states = np.zeros((steps, 2, n, 4), np.float32)
    xs, vs = pos, vel
    for t in range(steps):
        states[t, 0], states[t, 1] = xs, vs
        xs, vs = a.forward(xs, vs, 1)
    dirs = rng.standard_normal((ndirs, n, 3))
    k = ndirs + 2
    tv = np.zeros((k, n, 3))
    tv[:ndirs] = dirs
    trho = np.zeros(k)
    tc = np.zeros(k)
    trho[ndirs] = 1.0
    tc[ndirs + 1] = 1.0
    p = prm.as_dict()
    _, _, txo, _ = O.diff_rollout(pos, vel, p, mn, mx, steps, tv0=tv, trho=trho, tc=tc,
                                  states=states)
    jvp = np.array([(d * (2.0 / n) * txo[q]).sum() for q in range(k)])
    adj = np.array([(gv0 * dirs[q]).sum() for q in range(ndirs)] + [gr, gc])
    lin_err = np.abs(adj - jvp) / np.abs(jvp)

    # Short horizon: FP64 central differences.
    dF, gvF, grF, gcF = grads(a, fd_steps)
    a.close()

    def loss64(v0=vel, **phys):
        xx, _ = O.diff_rollout(pos, v0, p, mn, mx, fd_steps, **phys)
        return float(((xx - target) ** 2).sum() / n)

    # Step 2^-24: the rollout is piecewise smooth (container clamps), and
    # steps of 2^-20 and above cross kinks often enough to move central
    # differences by up to 1e-2 from the FP64 forward-mode derivative.
    e = 2.0 ** -24
    gnorm = float(np.linalg.norm(gvF))
    fd_dirs = list(dirs) + [gvF / gnorm]  # random directions, then the gradient's own
    fd_adj, fd_val = [], []
    for dq in fd_dirs:
        vp, vm = vel.copy(), vel.copy()
        vp[:, :3] += (e * dq).astype(np.float32)
        vm[:, :3] -= (e * dq).astype(np.float32)
        dvf = (vp[:, :3].astype(np.float64) - vm[:, :3].astype(np.float64)) / (2 * e)
        fd_val.append((loss64(v0=vp) - loss64(v0=vm)) / (2 * e))
        fd_adj.append(float((gvF * dvf).sum()))
    fd_adj, fd_val = np.array(fd_adj), np.array(fd_val)
    fd_err = (np.abs(fd_adj - fd_val) / np.abs(fd_val)).tolist()
    # A random direction's derivative is a sum of 3n terms of random sign and
    # cancels; over Gaussian directions r, E[(e.r)^2] = |e|^2, so this ratio
    # estimates the relative error of the whole v0 gradient.
    fd_grad_err = float(np.sqrt(((fd_adj[:ndirs] - fd_val[:ndirs]) ** 2).sum()
                                / (fd_val[:ndirs] ** 2).sum()))
    lin_grad_err = float(np.sqrt(((adj[:ndirs] - jvp[:ndirs]) ** 2).sum()
                                 / (jvp[:ndirs] ** 2).sum()))

    # Parameter steps in double (the restatement takes them beside the float32
    # parameters): with vorticity confinement the loss is strongly curved
    # where |eta| is small, and float32-sized steps (one ulp of rho0 is 5e-4)
    # miss the derivative by 10 % and more; these relative steps converge.
    def fd_param(kw, value, rel):
        h = rel * value
        return (loss64(**{kw: value + h}) - loss64(**{kw: value - h})) / (2 * h)

    fr = fd_param("rest_density", float(p["restDensity"]), 1e-8)
    fc = fd_param("xsph", float(p["xsphViscosity"]), 1e-5)

    s = pkg.PBFSolver()
    s.initialize(n, mn, mx, prm)
    s.set_particles(pos, vel)
    s.run(3)
    ms_solver = s.time_frames(steps)
    s.close()
    return {
        "particles": n, "steps": steps, "checkpoint_every": every,
        "forward_ms": 1000.0 * t_fwd, "backward_ms": 1000.0 * t_bwd,
        "adjoint_over_forward": t_bwd / t_fwd,
        "solver_forward_ms": ms_solver,
        "adjoint_over_solver_forward": 1000.0 * t_bwd / ms_solver,
        "loss": float((d * d).sum() / n),
        "check_full_horizon": {
            "reference": "FP64 forward-mode tangents (oracle/pbf_diff_oracle.cpp) linearised "
                         "about the GPU trajectory, %d v0 directions + rest density + XSPH c"
                         % ndirs,
            "rel_err": lin_err.tolist(), "max_rel_err": float(lin_err.max()),
            "v0_gradient_rel_err": lin_grad_err,
            "adjoint": adj.tolist(), "fp64": jvp.tolist()},
        "check_finite_differences": {
            "steps": fd_steps,
            "reference": "FP64 central differences of the FP64 restatement, step 2^-24 along "
                         "the same v0 directions and along the adjoint's v0 gradient; relative "
                         "steps 1e-8 in rest density and 1e-5 in c (in double)",
            "v0_rel_err": fd_err[:ndirs], "v0_max_rel_err": max(fd_err[:ndirs]),
            "v0_along_gradient_rel_err": fd_err[ndirs],
            "v0_gradient_rel_err": fd_grad_err,
            "rest_density": {"adjoint": grF, "fd": fr, "rel_err": abs(grF - fr) / abs(fr)},
            "xsph": {"adjoint": gcF, "fd": fc, "rel_err": abs(gcF - fc) / abs(fc)}},
        "workload": "64x64x16 dam-break lattice (spacing 0.5h) in a 6.4x4.8x1.6 box, "
                    "parameters as the 1M dam break (XSPH and vorticity confinement on)",
    }


def adjoint_reference_scene(pkg, scenes, frames: int = 10, every: int = 5):
    """Timing of the adjoint on the reference's own benchmark scene (262,144
    particles, 2 substeps x 4 iterations, box + sphere, XSPH and vorticity
    on): `frames` steps forward and back against the solver's own forward.
    Its accuracy is checked on smaller scenes by the test suite."""
    pos, vel, mn, mx, prm, col = scenes.reference_benchmark()
    n = len(pos)
    a = pkg.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=every)
    a.set_spheres(col["spheres"])
    a.set_boxes(col["boxes"])
    x, v = a.forward(pos, vel, frames)  # warm-up (graphs)
    gx = np.zeros((n, 4), np.float32)
    gx[:, :3] = (2.0 / n) * (x[:, :3] - pos[:, :3])
    a.backward(gx, np.zeros_like(gx))
    cuda_sync()
    t0 = time.perf_counter()
    a.forward(pos, vel, frames)
    cuda_sync()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    a.backward(gx, np.zeros_like(gx))
    cuda_sync()
    t_bwd = time.perf_counter() - t0
    a.close()
    s = pkg.PBFSolver()
    s.initialize(n, mn, mx, prm)
    s.set_spheres(col["spheres"])
    s.set_boxes(col["boxes"])
    s.set_particles(pos, vel)
    s.run(2)
    s.set_particles(pos, vel)
    ms_solver = s.time_frames(frames)
    s.close()
    return {"particles": n, "frames": frames, "substeps": prm.substeps,
            "checkpoint_every": every, "forward_ms": 1000.0 * t_fwd,
            "backward_ms": 1000.0 * t_bwd, "solver_forward_ms": ms_solver,
            "adjoint_over_solver_forward": 1000.0 * t_bwd / ms_solver,
            "workload": "the reference benchmark scene: box + sphere colliders, 2 substeps, "
                        "XSPH and vorticity confinement on"}


def run_reference(args):
    """The reference arm: the reference ships no CPU implementation of the
    step, so its CPU restatement (oracle/pbf_oracle.cpp, FP32, OpenMP on all
    host cores) runs the GPU arm's workload and window: `--warmup` untimed
    steps, then `--steps` timed steps, bounded to PBF_REF_SECONDS (default
    240) of timed CPU work."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    pkg = load_pkg()
    scenes = importlib.import_module("fluid_simulator_gb300.scenes")
    scene = scenes.dam_break_1m()
    budget = float(os.environ.get("PBF_REF_SECONDS", "240"))
    cb = cpu_baseline(scene, seconds_budget=budget, warmup=args.warmup, steps=args.steps)
    n = len(scene[0])
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": world, "steps": cb["steps"], "warmup": cb["warmup"],
        "ms_per_step": 1000.0 * n / cb["value"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded 128x128x64 dam-break lattice",
        "config": {"workload": WORKLOAD, "particles": n, "iterations": 4,
                   "implementation": "CPU restatement of the reference step (the reference "
                                     "ships CUDA only)"},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    del pkg
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scene", default="dam_break_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-cuda", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default 256-thread blocks")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-configured", action="store_true",
                    help="skip the run with the configuration's literal step parameters")
    ap.add_argument("--no-reference-scene", action="store_true",
                    help="skip the reference's own 262,144-particle benchmark scene")
    ap.add_argument("--adjoint-steps", type=int, default=60)
    ap.add_argument("--adjoint-directions", type=int, default=8)
    ap.add_argument("--batched-steps", type=int, default=120)
    ap.add_argument("--per-scene-steps", type=int, default=20)
    ap.add_argument("--list-capacity", type=int, default=None,
                    help="compact neighbour lists of this many entries in all "
                         "(pbf_initialize_compact) instead of max-neighbors slots per particle")
    ap.add_argument("--max-neighbors", type=int, default=256,
                    help="neighbour list capacity (the reference fixes 256)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.warmup < 3:
        args.warmup = 3

    rank, world, local = dist_env()
    dist = setup_dist(world, local)
    pkg = load_pkg()
    scenes = importlib.import_module("fluid_simulator_gb300.scenes")
    scene = scenes.SCENES[args.scene]()
    pos, vel, mn, mx, prm, col = scene
    n = len(pos)

    s = pkg.PBFSolver(local)
    s.initialize(n, mn, mx, prm, args.max_neighbors, list_capacity=args.list_capacity)
    for k, fn in (("spheres", s.set_spheres), ("boxes", s.set_boxes), ("planes", s.set_planes)):
        if col.get(k):
            fn(col[k])
    s.set_particles(pos, vel)
    s.run(args.warmup)
    tuned = s.autotune(2) if not args.no_autotune else s.block_sizes()
    s.run(1)  # re-instantiates the frame graphs after tuning
    first_timed = args.warmup + 1  # frames before the timed window
    kernels = s.kernels_per_frame()

    # ---- device-timed value -------------------------------------------------
    cuda_sync()
    barrier(dist)
    with Clocks(local) as clk:
        ms = s.time_frames(args.steps)
    clocks = clk.summary()
    cuda_sync()
    barrier(dist)
    ms_max = allreduce_max(dist, ms)
    value = n * args.steps * world / (ms_max / 1000.0)
    final_positions = s.copy_positions_to_host() if rank == 0 and world == 1 else None

    # ---- dominant kernel, timed live in the frame graph ---------------------
    prof = {}
    for _ in range(3):
        for k, (t, c) in s.profile_frame().items():
            a = prof.setdefault(k, [0.0, 0])
            a[0] += t
            a[1] += c
    stages = {k: {"ms_per_launch": v[0] / v[1], "launches_per_frame": v[1] / 3.0,
                  "share": 0.0} for k, v in prof.items()}
    total = sum(v[0] for v in prof.values())
    for k, v in prof.items():
        stages[k]["share"] = v[0] / total if total else 0.0
    dom = max(stages, key=lambda k: prof[k][0])
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    dom_bytes = STAGE_BYTES.get(dom, 0.0) * n
    achieved = dom_bytes / (stages[dom]["ms_per_launch"] / 1000.0) / 1e9
    cells = 1
    for a, b_ in zip(mn, mx):
        cells *= int(np.ceil((np.float64(np.float32(b_)) - np.float64(np.float32(a))) /
                             np.float64(np.float32(prm.smoothingRadius))))
    balg = b_alg(prm.solverIterations, cells / n)
    step_achieved = balg * n * (args.steps / (ms / 1000.0)) / 1e9

    # ---- end to end through the public API with pinned host buffers ---------
    keep = []

    def pinned(a):
        t, view = pinned_like(a)
        keep.append(t)
        return view

    # Start from the state the timed region ended in (same phase of the flow).
    in_p = pinned(s.copy_positions_to_host())
    in_v = pinned(s.copy_velocities_to_host())
    out_p, out_v = pinned(np.zeros_like(pos)), pinned(np.zeros_like(vel))
    s.set_particles(in_p, in_v)
    s.step()
    cuda_sync()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        s.set_particles(in_p, in_v)
        s.step()
        s.copy_positions_to_host(out=out_p)
        s.copy_velocities_to_host(out=out_v)
        in_p, out_p = out_p, in_p
        in_v, out_v = out_v, in_v
    cuda_sync()
    e2e_s = allreduce_max(dist, time.perf_counter() - t0)
    e2e_value = n * args.e2e_steps * world / e2e_s

    density = s.density_error()
    walk_lanes = s.walk_lanes()
    # Free this solver's device memory before the reference's kernels run
    # (both hold full neighbour lists; the 8M scene at 4,096 slots needs the
    # room), and before the other legs.
    s.close()
    mid_frame = first_timed + args.steps // 2
    cap_frame, cap = capture_for(dom, args.scene, mid_frame)

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded 128x128x64 dam-break lattice (no dataset)",
            "config": {"workload": WORKLOAD if args.scene == "dam_break_1m" else args.scene,
                       "particles": n, "iterations": prm.solverIterations,
                       "max_neighbors": args.max_neighbors,
                       "neighbor_lists": ("compact, %d entries" % args.list_capacity
                                          if args.list_capacity else "slot-major"),
                       "substeps": prm.substeps, "parallelism": "replicas" if world > 1 else
                       "single GPU", "l2": "step working set ~250 MB > 129 MB L2 (no flush)",
                       "timing": "CUDA events around %d graph-replayed steps on the solver "
                                 "stream" % args.steps,
                       "block_sizes": tuned, "walk_lanes": walk_lanes},
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(2 * 16 * n), "d2h_bytes_per_step": int(2 * 16 * n),
                    "steps": args.e2e_steps,
                    "path": "pbf_set_particles(pinned host) + pbf_step + "
                            "pbf_copy_positions/velocities(pinned host) per step"},
            "gpu_launches": kernels * args.steps,
            "kernels_per_step": kernels,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": cap["dram_bytes"] if cap else None,
                         "traffic_captured_at_frame": cap_frame,
                         "window_frames": [first_timed, first_timed + args.steps],
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": dom_bytes,
                         "ms_per_launch": stages[dom]["ms_per_launch"]},
            "issue_roofline": issue_roofline(dom, stages[dom]["ms_per_launch"], clocks,
                                             args.scene, mid_frame),
            "step_roofline": {"bytes_per_particle_step": balg, "achieved": step_achieved,
                              "peak": hbm, "unit": "GB/s", "frac": step_achieved / hbm},
            "stages": stages,
            "density_error": {"mean": density[0], "max": density[1],
                              "lists": "this library's own lists after the e2e steps"},
        }
        if final_positions is not None:
            line["density_error_fp64"] = dict(
                density_of(final_positions, scene),
                state="frame %d (end of the timed window), FP64 over all pairs within h"
                      % (first_timed + args.steps))
        if world == 1 and not args.no_reference_cuda:
            line["reference_cuda"] = reference_cuda(scene, args.steps, first_timed,
                                                    args.max_neighbors)
            if "value" in line["reference_cuda"]:
                ratio = value / line["reference_cuda"]["value"]
                line["speedup_vs_reference_cuda"] = ratio
                # The metric is quoted against the reference's CUDA solver: the
                # same workload and window on the same GPU, measured here.
                line["vs_baseline"] = ratio
                line["vs_baseline_basis"] = (
                    "value / the reference's own CUDA kernels' particle-steps/s, same "
                    "workload, same GPU, same frames %d..%d"
                    % (first_timed, first_timed + args.steps))
        if world == 1 and not args.no_configured:
            line["configured_parameters"] = configured_parameters(pkg, scene)
        if world == 1 and not args.no_reference_scene:
            line["reference_scene"] = reference_scene(pkg, scenes)
        if world == 1 and not args.no_batched:
            line["batched"] = batched(pkg, scenes, args.batched_steps, args.warmup,
                                      args.per_scene_steps)
        if world == 1 and not args.no_adjoint:
            line["adjoint"] = adjoint_bench(pkg, scenes, args.adjoint_steps, 10,
                                            args.adjoint_directions)
            line["adjoint_reference_scene"] = adjoint_reference_scene(pkg, scenes)
        if not args.no_cpu_baseline and world == 1:
            budget = float(os.environ.get("PBF_CPU_SECONDS", "20"))
            line["cpu_baseline"] = cpu_baseline(scene, seconds_budget=budget,
                                                warmup=first_timed, steps=args.steps)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
