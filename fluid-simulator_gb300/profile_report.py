"""Per-kernel profile of one PBF frame with Nsight Compute.

The counterpart of the reference's ``benchmark/profile.py`` (nsys + ncu), with
no disassembly step.  A timeline section first: with Nsight Systems on the
PATH, ``nsys profile --trace=cuda,nvtx`` of the same workload and its NVTX
range and kernel summaries (the library marks pbf_step, pbf_run,
pbf_run_async, pbf_time_frames and the adjoint's forward and backward with
NVTX ranges); without it, the frame's stages timed by CUDA events recorded
inside the frame graph (pbf_profile_frame), in pipeline order.  Then two
kinds of ncu runs, both with ``--clock-control none``:

1. a launch list of one whole frame (``gpu__time_duration.sum`` only, a
   single replay pass): launches, device time and share per kernel;
2. for each of the ``--top`` kernels by time, its first launch in the frame
   captured alone (``--launch-skip`` to it, ``--launch-count 1``) with DRAM
   bytes, L2 hit rate, issue and occupancy counters: achieved HBM GB/s =
   DRAM bytes / duration.

Each ncu run first runs the same workload without ncu and stops if it fails.
Usage (on a machine with a GPU and ncu):

    python fluid-simulator_gb300/profile_report.py --scene dam_break_1m --warmup 2 \\
        --out report.md

Times under ncu are serialised and cold-cache: compare shares, not absolutes.
"""

from __future__ import annotations

import argparse
import csv
import importlib
import importlib.util
import io
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
METRICS = [
    "gpu__time_duration.sum",
    "dram__bytes_read.sum",
    "dram__bytes_write.sum",
    "lts__t_sector_hit_rate.pct",
    "smsp__issue_active.avg.pct_of_peak_sustained_active",
    "sm__warps_active.avg.pct_of_peak_sustained_active",
    "launch__registers_per_thread",
]


def load_pkg():
    name = "fluid_simulator_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def child(scene: str, warmup: int, frames: int):
    """The profiled workload: set_particles, `warmup` frames, `frames` frames."""
    pkg = load_pkg()
    scenes = importlib.import_module("fluid_simulator_gb300.scenes")
    pos, vel, mn, mx, prm, col = scenes.SCENES[scene]()
    s = pkg.PBFSolver()
    s.initialize(len(pos), mn, mx, prm)
    for k, fn in (("spheres", s.set_spheres), ("boxes", s.set_boxes), ("planes", s.set_planes)):
        if col.get(k):
            fn(col[k])
    s.set_particles(pos, vel)
    s.run(warmup)
    s.run(frames)
    print("kernels_per_frame %d" % s.kernels_per_frame(), flush=True)


def child_stages(scene: str, warmup: int):
    """Stage times of one frame from CUDA events inside the frame graph,
    printed one stage per line in pipeline order: name, ms, launches."""
    pkg = load_pkg()
    scenes = importlib.import_module("fluid_simulator_gb300.scenes")
    pos, vel, mn, mx, prm, col = scenes.SCENES[scene]()
    s = pkg.PBFSolver()
    s.initialize(len(pos), mn, mx, prm)
    for k, fn in (("spheres", s.set_spheres), ("boxes", s.set_boxes), ("planes", s.set_planes)):
        if col.get(k):
            fn(col[k])
    s.set_particles(pos, vel)
    s.run(warmup)
    s.profile_frame()  # records the profiled graph
    for name, (ms, launches) in s.profile_frame().items():
        print("stage %s %.6f %d" % (name, ms, launches), flush=True)


def timeline(args, me, shown, tmp):
    """Report lines of the timeline section (see the module docstring)."""
    import shutil
    nsys = shutil.which(args.nsys)
    if nsys:
        rep = os.path.join(tmp, "timeline")
        cmd = [nsys, "profile", "--trace=cuda,nvtx", "--sample=none", "--cpuctxsw=none",
               "--force-overwrite=true", "-o", rep] + me
        run(cmd)
        lines = ["## Timeline (Nsight Systems)", "", "    " + shown(cmd), ""]
        for report in ("nvtx_sum", "cuda_gpu_kern_sum"):
            base = os.path.join(tmp, "stats")
            run([nsys, "stats", "--report", report, "--format", "csv", "--force-export=true",
                 "--output", base, rep + ".nsys-rep"])
            path = [os.path.join(tmp, f) for f in os.listdir(tmp)
                    if f.startswith("stats") and report in f and f.endswith(".csv")]
            if not path:
                continue
            rows = list(csv.reader(open(path[0])))
            if not rows:
                continue
            lines += ["### " + report, "", "| " + " | ".join(rows[0]) + " |",
                      "|" + "---|" * len(rows[0])]
            lines += ["| " + " | ".join(r) + " |" for r in rows[1:40]]
            lines.append("")
        return lines
    if args.adjoint:
        return ["## Timeline", "", "Nsight Systems (%s) is not installed here; the adjoint "
                "has no stage timeline." % args.nsys, ""]
    cmd = [sys.executable, os.path.abspath(__file__), "--child", "--stages", "--scene",
           args.scene, "--warmup", str(args.warmup)]
    out = run(cmd)
    lines = ["## Timeline (CUDA events inside the frame graph)", "",
             "Nsight Systems (%s) is not installed here.  One frame's stages, timed by CUDA "
             "events recorded between them in the profiled frame graph, in pipeline order "
             "(warm caches, graph launch):" % args.nsys, "", "    " + shown(cmd), "",
             "| stage | launches | ms | starts at ms (stages in order) | share |",
             "|---|---|---|---|---|"]
    stages = [l.split()[1:] for l in out.splitlines() if l.startswith("stage ")]
    total = sum(float(t) for _, t, _ in stages) or 1.0
    at = 0.0
    for name, t, n in stages:
        lines.append("| %s | %s | %.4f | %.4f | %.1f%% |" % (name, n, float(t), at,
                                                           100.0 * float(t) / total))
        at += float(t)
    lines.append("")
    return lines


def child_adjoint(steps: int):
    """The profiled adjoint workload: 65,536 particles (64x64x16 dam-break
    lattice, the 1M dam break's parameters: XSPH and vorticity confinement
    on), a `steps`-step forward with one checkpoint segment (recorded by the
    forward), then the backward's adjoint passes."""
    import numpy as np
    pkg = load_pkg()
    scenes = importlib.import_module("fluid_simulator_gb300.scenes")
    nx, ny, nz = 64, 64, 16
    S = scenes.SPACING
    pos, vel, mn, mx, prm, _ = scenes.dam_break(nx, ny, nz, (2 * nx * S, 1.5 * ny * S, 2 * nz * S))
    n = len(pos)
    a = pkg.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=steps)
    x, _ = a.forward(pos, vel, steps)
    gx = np.zeros((n, 4), np.float32)
    gx[:, :3] = (2.0 / n) * (x[:, :3] - pos[:, :3] - np.array([0.3, 0.0, 0.0], np.float32))
    a.backward(gx, np.zeros_like(gx))
    a.close()
    print("kernels_per_frame 0", flush=True)


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        sys.stderr.write(r.stdout[-4000:] + r.stderr[-4000:])
        raise SystemExit("command failed (%d): %s" % (r.returncode, " ".join(cmd)))
    return r.stdout


def ncu_rows(path):
    text = open(path).read()
    start = text.find('"ID"')
    rows = list(csv.DictReader(io.StringIO(text[start:])))
    return [r for r in rows if r.get("Kernel Name")]


SCALE = {"ns": 1e-9, "nsecond": 1e-9, "us": 1e-6, "usecond": 1e-6, "ms": 1e-3, "msecond": 1e-3,
         "s": 1.0, "second": 1.0, "byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9,
         "KB": 1e3, "MB": 1e6, "GB": 1e9}


def value(r):
    """Metric value in base units (seconds, bytes) where the unit is a scale."""
    v = float(r["Metric Value"].replace(",", ""))
    return v * SCALE.get(r.get("Metric Unit", ""), 1.0)


def short(name: str) -> str:
    name = name.split("(")[0]
    for pre in ("void ", "(anonymous namespace)::", "pbf::", "adj::"):
        name = name.replace(pre, "")
    return name.replace("unnamed>::", "").strip()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="dam_break_1m")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--top", type=int, default=4)
    ap.add_argument("--ncu", default="ncu")
    ap.add_argument("--nsys", default="nsys")
    ap.add_argument("--stages", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--out", default=None)
    ap.add_argument("--adjoint", action="store_true",
                    help="profile the adjoint (forward + backward of --adjoint-steps steps at "
                         "65,536 particles) instead of a solver frame")
    ap.add_argument("--adjoint-steps", type=int, default=10)
    ap.add_argument("--child", action="store_true")
    args = ap.parse_args()
    if args.child:
        if args.adjoint:
            child_adjoint(args.adjoint_steps)
        elif args.stages:
            child_stages(args.scene, args.warmup)
        else:
            child(args.scene, args.warmup, 1)
        return 0

    me = [sys.executable, os.path.abspath(__file__), "--child", "--scene", args.scene,
          "--warmup", str(args.warmup)]
    if args.adjoint:
        me = [sys.executable, os.path.abspath(__file__), "--child", "--adjoint",
              "--adjoint-steps", str(args.adjoint_steps)]
    root = os.path.dirname(HERE)

    def shown(cmd):
        """The command as a user would type it from the repository root."""
        out = []
        for c in cmd:
            if c == sys.executable:
                c = "python"
            elif os.path.isabs(c) and c.startswith(root + os.sep):
                c = os.path.relpath(c, root)
            elif os.path.isabs(c) and c.startswith(tempfile.gettempdir()):
                c = "<tmp>/" + os.path.basename(c)
            out.append(c)
        return " ".join(out)

    out = run(me)  # plain run first: it must succeed before ncu sees it
    kpf = int(out.split("kernels_per_frame")[1].split()[0])
    tmp_tl = tempfile.mkdtemp(prefix="pbf_tl_")
    tl_lines = timeline(args, me, shown, tmp_tl)
    # Solver: skip set_particles (two kernels) and the warm-up frames, list
    # one frame.  Adjoint: list every launch of the forward and backward.
    before = 0 if args.adjoint else 2 + args.warmup * kpf
    tmp = tempfile.mkdtemp(prefix="pbf_prof_")
    lst = os.path.join(tmp, "launches.csv")
    window = [] if args.adjoint else ["--launch-count", str(kpf)]
    cmd1 = [args.ncu, "--metrics", "gpu__time_duration.sum", "--clock-control", "none",
            "--launch-skip", str(before)] + window + ["--csv", "--log-file", lst] + me
    run(cmd1)
    agg = {}
    rows = [r for r in ncu_rows(lst) if r["Metric Name"] == "gpu__time_duration.sum"]
    for pos, r in enumerate(rows):
        k = short(r["Kernel Name"])
        sec = value(r)
        a = agg.setdefault(k, [0, 0.0, pos])  # count, time, first launch in the frame
        a[0] += 1
        a[1] += sec
    total = sum(a[1] for a in agg.values())
    order = sorted(agg.items(), key=lambda kv: -kv[1][1])

    detail = {}
    cmds = [shown(cmd1)]
    for k, (cnt, _, first) in order[: args.top]:
        # Exactly one launch: the kernel's first launch of the profiled frame.
        path = os.path.join(tmp, "k_%d.csv" % len(detail))
        cmd = [args.ncu, "--metrics", ",".join(METRICS), "--clock-control", "none",
               "--launch-skip", str(before + first), "--launch-count", "1", "--csv",
               "--log-file", path] + me
        run(me)
        run(cmd)
        cmds.append(shown(cmd))
        vals = {}
        for r in ncu_rows(path):
            if short(r["Kernel Name"]) != k:
                continue
            vals[r["Metric Name"]] = value(r)
        detail[k] = vals

    if args.adjoint:
        title = ("# Kernel profile: adjoint, 65,536 particles, %d-step forward + backward"
                 % args.adjoint_steps)
        gen = ("    python fluid-simulator_gb300/profile_report.py --adjoint --adjoint-steps %d "
               "--top %d" % (args.adjoint_steps, args.top))
        unit = "launches"
    else:
        title = "# Kernel profile: %s, one frame after %d warm-up frames" % (args.scene,
                                                                            args.warmup)
        gen = ("    python fluid-simulator_gb300/profile_report.py --scene %s --warmup %d --top %d"
               % (args.scene, args.warmup, args.top))
        unit = "launches / frame"
    lines = [title, "", "Generated by:", "", gen, "",
             "which runs (each after the same workload exited 0 without ncu):", ""]
    lines += ["    " + c for c in cmds]
    lines += [""] + tl_lines
    lines += ["## Launch list (ncu)", "", "| kernel | %s | device us | share |" % unit,
              "|---|---|---|---|"]
    for k, (cnt, sec, _) in order:
        lines.append("| %s | %d | %.1f | %.1f%% |" % (k, cnt, sec * 1e6, 100.0 * sec / total))
    lines += ["", "Top kernels, one launch each:", "",
              "| kernel | us | DRAM read MB | DRAM write MB | HBM GB/s | L2 hit % | issue % | "
              "warps % | regs |", "|---|---|---|---|---|---|---|---|---|"]
    for k, v in detail.items():
        if "gpu__time_duration.sum" not in v:
            continue
        sec = v["gpu__time_duration.sum"]
        rd = v.get("dram__bytes_read.sum", 0.0)
        wr = v.get("dram__bytes_write.sum", 0.0)
        lines.append("| %s | %.1f | %.1f | %.1f | %.0f | %.1f | %.1f | %.1f | %d |" % (
            k, sec * 1e6, rd / 1e6, wr / 1e6, (rd + wr) / sec / 1e9 if sec else 0.0,
            v.get("lts__t_sector_hit_rate.pct", 0.0),
            v.get("smsp__issue_active.avg.pct_of_peak_sustained_active", 0.0),
            v.get("sm__warps_active.avg.pct_of_peak_sustained_active", 0.0),
            int(v.get("launch__registers_per_thread", 0))))
    text = "\n".join(lines) + "\n"
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
