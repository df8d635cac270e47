"""Benchmark: tet-substeps/s of the small-step XPBD substep on one GB300.

Workload: the 128x64x32-cube throughput mesh (1,572,864 Neo-Hookean tets,
276,705 nodes, 0.1 m cubes jittered by N(0, (0.005 m)^2) with a fixed seed,
bottom face fixed, gravity -z, incompressible, dt = 1/60 s with 20 substeps).
One bench step = one frame = 20 substeps of the whole mesh; --steps 50 is the
configuration's 50 frames. Inputs are synthetic (seeded), the mesh has the
shape the configuration names.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl xfem|reference]

--impl xfem (default): the GPU solver through libxfem.so's C ABI.
  value  = tet-substeps/s with the state resident in HBM (device-timed with
           CUDA events on the solver's stream, L2 flushed between frames);
  e2e    = the same metric through the public API with pinned host buffers:
           every step uploads positions and velocities, steps one frame and
           reads the positions back (host-timed, copies included);
  roofline, cpu_baseline (the oracle port of the reference in its own
  shuffled order, 1 thread, on a bounded sample), clocks, gpu_launches, and
  "batched": 512 bodies in one launch per frame against one launch per body,
  "damped": the same mesh with the reference web UI's default damping against
  undamped, "models": the same mesh at nu = 0.45 with Mixed, YeohSkin, Pixar,
  one volume pass and ContinuousMixed (one-ring mode) against MixedSel, "setup": wall time of a handle's
  set-up (GPU set-up path and host set-up, 1.5M-tet mesh; 512-body batch),
  "hexes": hex mode on the same grid as 262,144 linear hexahedra (MixedSel,
  YeohSkinFast, Mixed, CubeNeo) with the oracle port's single-thread hex substep as
  its CPU baseline, "t10": quadratic-tet mode on the same mesh's 1,572,864 tets
  read as T10s (MixedSel, YeohSkinFast) with the oracle port's single-thread
  T10 substep as its CPU baseline, "h27": quadratic-hex mode on a 96x48x24 block of
  the grid read as 110,592 H27s (MixedSel, YeohSkinFast, Mixed) with the oracle
  port's single-thread H27 substep as its CPU baseline (each element line with
  its MixedSel element bandwidth against the measured HBM peak),
  "adjoint": cost of the reverse-mode gradient (recording forward + backward)
  against the plain forward, on the 32x8x8 beam (200 substeps, 20 tips,
  checkpoints every 20 substeps) and on the 1.5M-tet mesh (one frame),
  "drop": the drop configuration (64x16x16 cubes of Yeoh C10/C20/C30 =
  3e4/1e3/1e2 Pa dropped from 0.5 m onto a frictional ground), all 300 frames
  of 30 substeps, with its CPU baseline; and "summary", the side legs'
  headline figures in one compact object at the end of the line.
--impl reference: the reference's CPU algorithm (the oracle port, run in the
  GPU's colour order with all host threads) on the same mesh; each step is
  one frame (20 substeps), as in the GPU arm.

Multi-GPU (torchrun): replicas only — every rank steps its own copy of the
mesh, no collective on the data path; value sums the ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "xpbd-fem_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "tet-substeps/s (1.5M tets FP32)"
UNIT = "tet-substeps/s"
# Per-unit algorithmic bytes of the reference layout: 80 B tet record (4 u32 indices + Qi, QQ,
# QR, volume) + 76 B per vertex per substep (X, V, O read/write 24 B each,
# w 4 B) x V/T.
REC_BYTES, VERT_BYTES = 80.0, 76.0
# DRAM bytes (read + write) per tet-substep of each launch form's kernel, from
# the ncu capture of the same command (one launch, --set full), per launch of
# 20 substeps x 1,572,864 tets: k_persistent 2.143 GB, k_bricks 2.583 GB (two
# bricks per SM, 192-thread blocks, the layout the autotuner picks there).
NCU_DRAM_BYTES_PER_TET_SUBSTEP = {"k_persistent": 68.12, "k_bricks": 82.12}
# Launch forms (xfem_options.sync_mode) and the kernel each one times.
SYNC_NAMES = {1: "persistent", 2: "cuda-graph", 3: "dataflow", 4: "bricks"}
SYNC_KERNELS = {1: "k_persistent", 3: "k_dataflow", 4: "k_bricks"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("XFEM_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline_native(w, budget_s=12.0):
    """The oracle port of the reference, in the reference's own MINSTD order
    (XPBDFEM/Geo.cpp:759-777), single thread, on the first substeps of the
    same mesh; sized to about budget_s seconds."""
    import oracle
    tets, _ = oracle.parse_tets(w["idx"])
    ep, wi, _ = oracle.init_rest(w["nodes"], tets, w["density"])
    order = oracle.minstd_order(tets.shape[0])
    sdt = w["dt"] / w["substeps"]
    p = oracle.params_from_settings(w["settings"], sdt)
    X = w["nodes"].reshape(-1, 3).astype(np.float64)
    V = np.zeros_like(X)
    t0 = time.perf_counter()
    X, V, wi, _ = oracle.substeps(X, V, wi, tets, ep, order, 1, p, lock_mask=w["lock"])
    t1 = time.perf_counter() - t0
    n = max(1, min(30, int(budget_s / max(t1, 1e-3)) - 1))
    t0 = time.perf_counter()
    oracle.substeps(X, V, wi, tets, ep, order, n, p, lock_mask=w["lock"])
    t = time.perf_counter() - t0
    nt = tets.shape[0]
    return {"value": nt * n / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} substeps of the full {nt}-tet mesh after 1 untimed, reference shuffled order, 1 thread"}


def run_reference(args, world, rank):
    """--impl reference: the oracle port with all host threads, colour order."""
    if rank != 0:
        return
    import oracle
    from xfem import workloads as W
    w = W.throughput()
    tets, _ = oracle.parse_tets(w["idx"])
    ep, wi, _ = oracle.init_rest(w["nodes"], tets, w["density"])
    sch = oracle.schedule(w["nodes"], tets, mode=1, morton=1)
    sdt = w["dt"] / w["substeps"]
    p = oracle.params_from_settings(w["settings"], sdt)
    X = w["nodes"].reshape(-1, 3).astype(np.float64)
    V = np.zeros_like(X)
    threads = os.cpu_count() or 1
    per_step = w["substeps"]  # one step = one frame, as in the GPU arm
    nt = tets.shape[0]

    def step(X, V, wi):
        X2, V2, w2, _ = oracle.substeps(X, V, wi, tets, ep, sch["tet_order"], per_step, p, lock_mask=w["lock"],
                                        threads=threads, colour_begin=sch["colour_tet_begin"])
        return X2, V2, w2

    for _ in range(args.warmup):
        X, V, wi = step(X, V, wi)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        X, V, wi = step(X, V, wi)
    t = time.perf_counter() - t0
    value = nt * per_step * args.steps / t
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": w["name"], "tets": nt, "vertices": int(X.shape[0]),
                       "substeps_per_step": per_step, "dt": w["dt"], "order": "colour order (same schedule as the GPU)",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"one frame ({per_step} substeps) of the full mesh per step, {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_xfem(args, world, rank, local):
    import torch

    import xfem
    from xfem import workloads as W
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = W.throughput()
    nt, nv = w["idx"].size // 5, w["nodes"].size // 3
    sdt = w["dt"] / w["substeps"]
    S = w["substeps"]
    stream = torch.cuda.Stream(device=dev)
    body = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], device=local,
                     stream=C_void_p(stream.cuda_stream), sync_mode=args.sync_mode, block_size=args.block,
                     bricks=args.bricks)
    body.set_lock_mask(w["lock"])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    for _ in range(args.warmup):
        body.step_frames(1, S, sdt)
    body.synchronize()
    info = body.info()
    # device-timed region: one event pair per frame on the solver's stream,
    # the L2 flush between frames stays outside the pairs
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev[k][0].record(stream)
            body.step_frames(1, S, sdt)
            with torch.cuda.stream(stream):
                ev[k][1].record(stream)
        body.synchronize()
        torch.cuda.synchronize()
    barrier(world)
    ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(ms) / 1e3
    total_s = reduce_max(total_s, world)
    tet_sub = nt * S * args.steps
    value = world * tet_sub / total_s
    # end to end through the public API with pinned host buffers
    px = np.frombuffer((ctypes_buffer(xfem, 3 * nv)), np.float32)
    pv = np.frombuffer((ctypes_buffer(xfem, 3 * nv)), np.float32)
    po = np.frombuffer((ctypes_buffer(xfem, 3 * nv)), np.float32)  # the read-back, pinned too
    px[:] = w["nodes"]
    pv[:] = 0.0
    e2e_steps = max(3, min(args.steps, 20))
    body.set_positions(px)
    body.set_velocities(pv)
    body.step_frames(1, S, sdt)
    e2e_t = 0.0
    for k in range(e2e_steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        body.synchronize()
        t0 = time.perf_counter()
        body.set_state(px, pv)
        body.step_frames(1, S, sdt)
        out = body.positions(out=po)
        e2e_t += time.perf_counter() - t0
        px[:] = out.reshape(-1)
    e2e_t = reduce_max(e2e_t, world)
    e2e = world * nt * S * e2e_steps / e2e_t
    if rank != 0:
        return
    hbm, peak_kind = peaks()
    bpu = REC_BYTES + VERT_BYTES * nv / nt
    per_launch_ms = statistics.mean(ms)
    launches_per_frame = 1 if info["sync_mode"] != 2 else S * info["colours"] + 1
    achieved = bpu * nt * S / (per_launch_ms / 1e3) / 1e9
    kernel = SYNC_KERNELS.get(info["sync_mode"], "k_colour (whole frame)")
    dram = NCU_DRAM_BYTES_PER_TET_SUBSTEP.get(kernel)
    traffic = None if dram is None else dram * nt * S
    cpu = cpu_baseline_native(w) if not args.no_cpu else None
    batched = None if args.no_batched else run_batched(stream)
    adjoint = None if args.no_adjoint else run_adjoint(stream)
    damped = None if args.no_damped else run_damped(stream)
    models = None if args.no_models else run_models(stream)
    setup = None if args.no_setup else run_setup(stream)
    hexes = None if args.no_hexes else run_hexes(stream, cpu=not args.no_cpu)
    t10 = None if args.no_t10 else run_t10(stream, cpu=not args.no_cpu)
    h27 = None if args.no_h27 else run_h27(stream, cpu=not args.no_cpu)
    drop = None if args.no_drop else run_drop(stream, cpu=not args.no_cpu)
    for kind, rec in (("hexes", hexes), ("t10", t10), ("h27", h27)):
        if rec is not None:
            rec["roofline"] = element_roofline(kind, rec)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": w["name"], "tets": nt, "vertices": nv, "substeps_per_step": S,
                   "dt": w["dt"], "parallelism": f"replicas{world}", "l2": "flushed between steps (256 MB write)",
                   "colours": info["colours"], "clusters": info["clusters"], "sync_mode":
                   SYNC_NAMES[info["sync_mode"]], "block": info["block_size"],
                   "blocks": info["blocks"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_kind": peak_kind, "bytes_per_tet_substep": bpu,
                     "kernel": kernel,
                     "launch_ms": per_launch_ms},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * 12 * nv, "d2h_bytes_per_step": 12 * nv,
                "steps": e2e_steps},
        "gpu_launches": launches_per_frame * args.steps,
        "batched": batched,
        "adjoint": adjoint,
        "damped": damped,
        "models": models,
        "setup": setup,
        "hexes": hexes,
        "t10": t10,
        "h27": h27,
        "drop": drop,
        "clocks": clk.summary(),
    }
    line["summary"] = summary(line)
    print(json.dumps(line), flush=True)


def summary(line):
    """The side legs' headline figures in one compact object, printed last
    on the line so that a reader keeping only the end of the output has them."""
    def g(*keys):
        v = line
        for k in keys:
            if not isinstance(v, dict) or v.get(k) is None:
                return None
            v = v[k]
        return round(v, 4) if isinstance(v, float) else v
    return {"value": g("value"), "frac": g("roofline", "frac"), "e2e": g("e2e", "value"),
            "batched_speedup": g("batched", "speedup"), "batched_value": g("batched", "value"),
            "adjoint_beam_cost": g("adjoint", "beam", "record_plus_backward_over_forward"),
            "adjoint_large_cost": g("adjoint", "large", "record_plus_backward_over_forward"),
            "damped_cost": g("damped", "cost"), "hexes_frac": g("hexes", "roofline", "frac"),
            "t10_frac": g("t10", "roofline", "frac"), "h27_frac": g("h27", "roofline", "frac"),
            "drop_value": g("drop", "value"), "drop_ms_per_frame": g("drop", "ms_per_frame"),
            "drop_frac": g("drop", "roofline", "frac"), "setup_s": g("setup", "throughput")}


def run_drop(stream, cpu=True, cpu_budget_s=6.0):
    """The drop configuration: 64x16x16 cubes (98,304 tets) of Yeoh with C10 =
    3e4, C20 = 1e3, C30 = 1e2 Pa, incompressible, dropped from 0.5 m with a
    seeded random rotation onto a frictional ground (mu = 0.4), 30 substeps
    per frame of 1/60 s: all 300 frames device-timed one event pair per frame
    (the L2 flushed between frames, outside the pairs), the body landing and
    bouncing on the way; its element bandwidth against the measured HBM peak;
    and the oracle port of the reference, one thread in the reference's
    shuffled order, on a bounded sample of substeps of the same mesh."""
    import torch

    import oracle
    import xfem
    from xfem import workloads as W
    w = W.drop_yeoh()
    nt, nv = w["idx"].size // 5, w["nodes"].size // 3
    S, frames = w["substeps"], w["frames"]
    sdt = w["dt"] / S
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    body = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], stream=C_void_p(stream.cuda_stream))
    x0, v0 = body.positions(), body.velocities()
    for _ in range(3):
        body.step_frames(1, S, sdt)
    body.set_positions(x0)
    body.set_velocities(v0)
    body.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    for k in range(frames):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[k][0].record(stream)
        body.step_frames(1, S, sdt)
        with torch.cuda.stream(stream):
            ev[k][1].record(stream)
    body.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    x = body.positions()
    info = body.info()
    body.close()
    per_frame = sum(ms) / frames
    hbm, peak_kind = peaks()
    bpu = REC_BYTES + VERT_BYTES * nv / nt
    achieved = bpu * nt * S / (per_frame / 1e3) / 1e9
    out = {"workload": w["name"], "frames": frames, "substeps_per_frame": S, "ms_per_frame": per_frame,
           "value": nt * S / (per_frame / 1e3), "unit": UNIT,
           "sync_mode": SYNC_NAMES.get(info["sync_mode"]),
           "block": info["block_size"], "final_min_z": float(x[:, 2].min()),
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "peak_kind": peak_kind, "bytes_per_tet_substep": bpu}}
    if cpu:
        tets, _ = oracle.parse_tets(w["idx"])
        ep, wi, _ = oracle.init_rest(w["nodes"], tets, w["density"])
        order = oracle.minstd_order(tets.shape[0])
        p = oracle.params_from_settings(w["settings"], sdt)
        X = w["nodes"].reshape(-1, 3).astype(np.float64)
        V = np.zeros_like(X)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < cpu_budget_s or n == 0:
            X, V, wi, _ = oracle.substeps(X, V, wi, tets, ep, order, 1, p)
            n += 1
        out["cpu_baseline"] = {"value": nt * n / (time.perf_counter() - t0), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{n} substeps of the same mesh, reference shuffled order, 1 thread"}
    return out


def run_batched(stream, frames=5, plain_frames=2):
    """512 independent bodies (a, b, c ~ U{2..24} cubes, coin-flip Neo-Hookean /
    Yeoh, log-uniform E, each on its own ground): one handle and one launch per
    frame, against the same bodies as 512 handles stepped one launch per body
    on the same stream. Device-timed with CUDA events; 20 substeps per frame."""
    import torch

    import xfem
    from xfem import workloads as W
    w = W.batched()
    sdt = w["dt"] / w["substeps"]
    sp = C_void_p(stream.cuda_stream)
    batch = xfem.Body(meshes=w["meshes"], settings=w["settings"], stream=sp)
    nt = batch.info()["tets"]
    for _ in range(3):
        batch.step_frames(1, 20, sdt)
    batch.synchronize()

    def timed(fn, n):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
        for _ in range(n):
            fn()
        with torch.cuda.stream(stream):
            b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3 / n

    tb = timed(lambda: batch.step_frames(1, 20, sdt), frames)
    info = batch.info()
    batch.close()
    singles = [xfem.Body(nodes, idx, d, s_, sync_mode=1, block_size=128, stream=sp)
               for (nodes, idx, d), s_ in zip(w["meshes"], w["settings"])]

    def plain():
        for b in singles:
            b.step_frames(1, 20, sdt)

    plain()
    tp = timed(plain, plain_frames)
    for b in singles:
        b.close()
    return {"workload": w["name"], "bodies": len(w["meshes"]), "tets": nt, "substeps_per_frame": 20,
            "value": nt * 20 / tb, "unit": UNIT, "ms_per_frame": 1e3 * tb,
            "plain_one_body_per_launch": nt * 20 / tp, "plain_ms_per_frame": 1e3 * tp, "speedup": tp / tb,
            "sync_mode": SYNC_NAMES.get(info["sync_mode"]),
            "launches_per_frame": 1 if info["sync_mode"] != 2 else 20 * info["colours"] + 1}


def run_adjoint(stream, reps=5, cases=("beam", "large"), large_substeps=None):
    """Cost of the gradient: the recording forward (xfem_adjoint_forward) and
    the reverse pass (xfem_adjoint_backward, host cotangent in, dL/dmu, dL/dX0,
    dL/dV0 out) against the plain forward (xfem_step_frames) of the same
    substeps, each device-timed with CUDA events on the solver's stream around
    the synchronising C ABI calls (host copies included), median of `reps`."""
    import torch

    import xfem
    from xfem import workloads as W
    sp = C_void_p(stream.cuda_stream)

    def ev_time(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
        fn()
        with torch.cuda.stream(stream):
            b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    def measure(nodes, idx, s, lock, mu, tips, nsub, dt, ckpt):
        body = xfem.Body(nodes, idx, 1000.0, s, stream=sp)
        body.set_lock_mask(lock)
        body.set_tet_mu(mu)
        x0, v0 = body.positions(), body.velocities()
        G = np.full((nsub, len(tips), 3), 1e-3, np.float32)

        def reset():
            body.set_positions(x0)
            body.set_velocities(v0)
            body.synchronize()

        out = {"forward_ms": [], "record_ms": [], "backward_ms": [], "backward_ckpt_ms": []}
        reset()
        body.step_frames(1, nsub, dt)  # tunes the plain launch
        for _ in range(reps):
            reset()
            out["forward_ms"].append(ev_time(lambda: (body.step_frames(1, nsub, dt), body.synchronize())))
            reset()
            out["record_ms"].append(ev_time(lambda: body.adjoint_forward(nsub, dt, tips, 0)))
            out["backward_ms"].append(ev_time(lambda: body.adjoint_backward(G)))
            if ckpt:
                reset()
                body.adjoint_forward(nsub, dt, tips, ckpt)
                out["backward_ckpt_ms"].append(ev_time(lambda: body.adjoint_backward(G)))
        body.close()
        r = {k: statistics.median(v) for k, v in out.items() if v}
        r["backward_over_forward"] = r["backward_ms"] / r["forward_ms"]
        r["record_plus_backward_over_forward"] = (r["record_ms"] + r["backward_ms"]) / r["forward_ms"]
        return r

    res = {"timing": f"CUDA events around the synchronising C ABI calls, median of {reps}"}
    if "beam" in cases:
        d = W.adjoint_beam()
        beam = measure(d["nodes"], d["idx"], d["settings"], d["lock"], d["mu"], d["tips"], d["substeps"], d["dt"], 20)
        beam.update({"workload": d["name"], "substeps": d["substeps"], "tips": int(d["tips"].size),
                     "checkpoint_every": 20})
        res["beam"] = beam
    if "large" in cases:
        t = W.throughput()
        nt = t["idx"].size // 5
        mu = np.full(nt, 1.0 / t["settings"]["compliance"], np.float32)
        S = large_substeps or t["substeps"]
        big = measure(t["nodes"], t["idx"], t["settings"], t["lock"], mu, np.arange(20, dtype=np.uint32), S,
                      t["dt"] / t["substeps"], 0)
        big.update({"workload": t["name"], "substeps": S, "tips": 20})
        res["large"] = big
    return res


def run_damped(stream, frames=5):
    """The throughput mesh with the damping the reference's web UI starts with
    (wasm/ui.js:76-78, 88: Rayleigh PostAmortized, damping 0.005, pbdDamping
    0.03, drag 0.002; the element spacing 0.1 m stands in for the demo's
    kSpacing), against the same mesh undamped: device-timed frames of 20
    substeps, L2 flushed between frames."""
    import torch

    import xfem
    from xfem import workloads as W
    w = W.throughput()
    S = w["substeps"]
    sdt = w["dt"] / S
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    vc, avc = xfem.pbd_damping_coefficients(0.03, sdt, 0.1)
    damp = dict(w["settings"], damping=0.005, pbd_damping=0.03, time_corrected_drag=xfem.time_corrected_drag(0.002, sdt),
                volume_and_time_corrected_pbd_damping=vc, amortized_volume_and_time_corrected_pbd_damping=avc,
                flags=w["settings"]["flags"] | (3 << 20))
    out = {key: time_frames(stream, w, s_, flush, frames)
           for key, s_ in (("undamped", w["settings"]), ("damped", damp))}
    return {"workload": w["name"] + ", damping as the reference's web UI starts (PostAmortized 0.005, PBD 0.03, "
                                   "drag 0.002)", "unit": UNIT, **out,
            "cost": out["damped"]["ms_per_frame"] / out["undamped"]["ms_per_frame"]}


def time_frames(stream, w, settings, flush, frames):
    """Median device time of one frame (w's substeps) of a body of workload w
    with the given settings, L2 flushed before each frame."""
    import torch

    import xfem
    S = w["substeps"]
    sdt = w["dt"] / S
    body = xfem.Body(w["nodes"], w["idx"], w["density"], settings, stream=C_void_p(stream.cuda_stream))
    # a T10 body has more vertices than the mesh (its edge nodes): its lock
    # mask comes from its own rest positions by the same rule
    from xfem import workloads as W
    body.set_lock_mask(w["lock"] if w["lock"] is not None else W.lock_mask_axis(body.positions(), 2))
    for _ in range(3):
        body.step_frames(1, S, sdt)
    ms = []
    for _ in range(frames):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            a.record(stream)
        body.step_frames(1, S, sdt)
        with torch.cuda.stream(stream):
            b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    info = body.info()
    body.close()
    nt = w["idx"].size // 5
    return {"ms_per_frame": statistics.median(ms), "value": nt * S / (statistics.median(ms) / 1e3),
            "sync_mode": SYNC_NAMES.get(info["sync_mode"]),
            "block": info["block_size"]}


def run_setup(stream):
    """Wall time of a handle's set-up (rest state, schedule, device layout,
    uploads; xfem_create / xfem_batch_create) for the throughput mesh with the
    GPU set-up path and with the host set-up, and for the 512-body batch.
    The reference's GeoLinear3d::Init of the same mesh takes about 2 s."""
    import xfem
    from xfem import workloads as W
    sp = C_void_p(stream.cuda_stream)
    w = W.throughput()
    out = {"unit": "s"}
    for key, host in (("throughput", False), ("throughput_host_setup", True)):
        t = time.perf_counter()
        b = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], stream=sp, host_setup=host)
        out[key] = time.perf_counter() - t
        b.close()
    wb = W.batched()
    t = time.perf_counter()
    b = xfem.Body(meshes=wb["meshes"], settings=wb["settings"], stream=sp)
    out["batched_512"] = time.perf_counter() - t
    b.close()
    out["workload"] = w["name"] + "; " + wb["name"] + " (%d tets)" % sum(m[1].size // 5 for m in wb["meshes"])
    return out


def run_models(stream, frames=5):
    """The throughput mesh at nu = 0.45 (the Pixar models need nu < 0.5) with
    the other energy models, with volume passes and with the continuous-
    pressure model ContinuousMixed (one-ring mode), against MixedSel (the hot
    kernel): device-timed frames of 20 substeps, L2 flushed between frames."""
    import torch

    import xfem
    from xfem import workloads as W
    w = W.throughput()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    base = dict(w["settings"], poissons_ratio=0.45, compliance=W.nh_compliance(5e5, 0.45))
    solve = (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT
    cases = (("mixed_sel", base), ("mixed", dict(base, flags=(xfem.ENERGY_MIXED << xfem.ENERGY_BIT) | solve)),
             ("yeoh_skin", dict(base, flags=(xfem.ENERGY_YEOH_SKIN << xfem.ENERGY_BIT) | solve)),
             ("pixar", dict(base, flags=(xfem.ENERGY_PIXAR << xfem.ENERGY_BIT) | solve)),
             ("mixed_sel_volume_1", dict(base, volume_passes=1)),
             ("continuous_mixed", dict(base, flags=(xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT) | solve)))
    out = {key: time_frames(stream, w, s_, flush, frames) for key, s_ in cases}
    return {"workload": w["name"].replace("Neo-Hookean", "nu = 0.45"), "unit": UNIT, **out,
            "cost": {k: out[k]["ms_per_frame"] / out["mixed_sel"]["ms_per_frame"] for k, _ in cases[1:]}}


def run_hexes(stream, frames=5, cpu_budget_s=6.0, cpu=True):
    """Hex mode: the throughput grid as 262,144 linear hexahedra (the same
    jittered nodes; each hex is the 6 tets of the tet mesh's cube) with
    MixedSel, YeohSkinFast, Mixed (2x2x2 quadrature) and CubeNeo (its short
    path at nu = 0.5), device-timed frames
    of 20 substeps with L2 flushed between frames; and the oracle port of the
    reference's hex substep on one host thread on the same mesh (a bounded
    sample of substeps) as the CPU baseline."""
    import torch

    import oracle
    import xfem
    from xfem import workloads as W
    w = W.throughput_hex()
    nh = w["idx"].size // 9
    S = w["substeps"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    solve = (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT
    cases = (("mixed_sel", w["settings"]),
             ("yeoh_skin_fast", dict(w["settings"], flags=(xfem.ENERGY_YEOH_SKIN_FAST << xfem.ENERGY_BIT) | solve,
                                     compliance=3.2e-4)),
             ("mixed", dict(w["settings"], flags=(xfem.ENERGY_MIXED << xfem.ENERGY_BIT) | solve)),
             ("cube_neo", dict(w["settings"], flags=(xfem.ENERGY_CUBE_NEO << xfem.ENERGY_BIT) | solve)))
    out = {}
    for key, s_ in cases:
        r = time_frames(stream, w, s_, flush, frames)
        r["value"] = nh * S / (r["ms_per_frame"] / 1e3)
        r.pop("sync_mode")
        r.pop("block")
        out[key] = r
    if not cpu:
        return {"workload": w["name"], "unit": "hex-substeps/s", **out}
    # CPU: the oracle's float restatement, one thread, the reference's
    # algorithm in the GPU's hex order
    hexes, _ = oracle.parse_hexes(w["idx"])
    ep, wi, fl = oracle.hex_init_rest(w["nodes"], hexes, w["density"])
    order = oracle.hex_schedule(w["nodes"], hexes)["hex_order"]
    p = oracle.params_from_settings(w["settings"], w["dt"] / S, lock=False)
    X = w["nodes"].astype(np.float64).reshape(-1, 3)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget_s or n == 0:
        X, V, wi, _ = oracle.hex_substeps(X, np.zeros_like(X), wi, hexes, ep, order, 1, p)
        n += 1
    cpu = nh * n / (time.perf_counter() - t0)
    return {"workload": w["name"], "unit": "hex-substeps/s", **out,
            "cpu_baseline": {"value": cpu, "unit": "hex-substeps/s", "cores": 1, "kind": "port",
                             "sample": "%d substeps of the same mesh (MixedSel)" % n},
            "vs_tet_mesh_of_the_same_grid": "each hex covers the 6 tets of one cube of the throughput mesh"}


def run_t10(stream, frames=5, cpu_budget_s=6.0, cpu=True):
    """Quadratic-tet mode: the throughput mesh's 1,572,864 tets read as T10s
    (GeoQuadratic3d: a node on each of the 1.9 M edges, 10-node elements on
    the 4-point rule) with MixedSel and YeohSkinFast, device-timed frames of
    20 substeps with L2 flushed between frames; and the oracle port of the
    reference's T10 substep on one host thread on the same mesh (a bounded
    sample of substeps) as the CPU baseline."""
    import torch

    import oracle
    import xfem
    from xfem import workloads as W
    w = dict(W.throughput(), lock=None)
    nt = w["idx"].size // 5
    S = w["substeps"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    solve = (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | xfem.ELEMENT_T10
    cases = (("mixed_sel", dict(w["settings"], flags=w["settings"]["flags"] | xfem.ELEMENT_T10)),
             ("yeoh_skin_fast", dict(w["settings"], flags=(xfem.ENERGY_YEOH_SKIN_FAST << xfem.ENERGY_BIT) | solve,
                                     compliance=3.2e-4)))
    out = {}
    for key, s_ in cases:
        r = time_frames(stream, w, s_, flush, frames)
        r["value"] = nt * S / (r["ms_per_frame"] / 1e3)
        r.pop("sync_mode")
        r.pop("block")
        out[key] = r
    if not cpu:
        return {"workload": w["name"] + " as T10s", "unit": "T10-substeps/s", **out}
    # CPU: the oracle's float restatement, one thread, the reference's
    # algorithm in the GPU's T10 order
    q = oracle.Quadratic(w["nodes"], w["idx"], w["density"])
    order = q.schedule()["tet_order"]
    p = oracle.params_from_settings(w["settings"], w["dt"] / S, lock=False)
    X, wi = q.X0.copy(), q.w.copy()
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget_s or n == 0:
        X, V, wi, _ = q.substeps(X, np.zeros_like(X), wi, order, 1, p)
        n += 1
    cpu = nt * n / (time.perf_counter() - t0)
    return {"workload": w["name"] + " as T10s", "unit": "T10-substeps/s", "vertices": int(q.X0.shape[0]), **out,
            "cpu_baseline": {"value": cpu, "unit": "T10-substeps/s", "cores": 1, "kind": "port",
                             "sample": "%d substeps of the same mesh (MixedSel)" % n}}


def run_h27(stream, frames=5, cpu_budget_s=6.0, cpu=True):
    """Quadratic-hex mode: a 96x48x24 block of the throughput grid (same
    spacing and jitter) read as 110,592 H27s (GeoQuadratic3d: nodes on the
    edges, faces and centres, 27-node elements on the 2x2x2 and 3x3x3 rules;
    one warp per element) with MixedSel, YeohSkinFast and Mixed, device-timed
    frames of 20 substeps with L2 flushed between frames; and the oracle port
    of the reference's H27 substep on one host thread on the same mesh (a
    bounded sample of substeps) as the CPU baseline."""
    import torch

    import oracle
    import xfem
    from xfem import workloads as W
    w = dict(W.throughput_hex(W=96, H=48, D=24), lock=None)
    nh = w["idx"].size // 9
    S = w["substeps"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=stream.device)
    solve = (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | xfem.ELEMENT_H27
    cases = (("mixed_sel", dict(w["settings"], flags=w["settings"]["flags"] | xfem.ELEMENT_H27)),
             ("yeoh_skin_fast", dict(w["settings"], flags=(xfem.ENERGY_YEOH_SKIN_FAST << xfem.ENERGY_BIT) | solve,
                                     compliance=3.2e-4)),
             ("mixed", dict(w["settings"], flags=(xfem.ENERGY_MIXED << xfem.ENERGY_BIT) | solve)))
    out = {}
    for key, s_ in cases:
        r = time_frames(stream, w, s_, flush, frames)
        r["value"] = nh * S / (r["ms_per_frame"] / 1e3)
        r.pop("sync_mode")
        r.pop("block")
        out[key] = r
    if not cpu:
        return {"workload": w["name"] + " as H27s", "unit": "H27-substeps/s", **out}
    q = oracle.QuadraticHex(w["nodes"], w["idx"], w["density"])
    order = q.schedule()["hex_order"]
    p = oracle.params_from_settings(w["settings"], w["dt"] / S, lock=False)
    X, wi = q.X0.copy(), q.w.copy()
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget_s or n == 0:
        X, V, wi, _ = q.substeps(X, np.zeros_like(X), wi, order, 1, p)
        n += 1
    cpu = nh * n / (time.perf_counter() - t0)
    return {"workload": w["name"] + " as H27s", "unit": "H27-substeps/s", "vertices": int(q.X0.shape[0]), **out,
            "cpu_baseline": {"value": cpu, "unit": "H27-substeps/s", "cores": 1, "kind": "port",
                             "sample": "%d substeps of the same mesh (MixedSel)" % n}}


# Element bytes a MixedSel element-substep moves (vertex state read and
# written, 32 B each way per vertex; the record fields the solve reads; the
# vertex ids): hex 8 x 64 + 192, T10 10 x 64 + 224 + 48, H27 27 x 64 + 1,728
# (the 2x2x2 rule's Ji and weights, QQ, QR, volume) + 108. Vertices are shared
# between elements, so DRAM sees less than this when they stay in L2.
ELEMENT_BYTES = {"hexes": 8 * 64 + 192, "t10": 10 * 64 + 224 + 48, "h27": 27 * 64 + 1728 + 108}


def element_roofline(kind, line):
    """The element kernel's element bandwidth on the MixedSel case against
    the measured HBM copy bandwidth."""
    hbm, peak_kind = peaks()
    achieved = ELEMENT_BYTES[kind] * line["mixed_sel"]["value"] / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "peak_kind": peak_kind, "bytes_per_element_substep": ELEMENT_BYTES[kind],
            "note": "element bytes, not DRAM traffic: shared vertices hit in L2"}


def C_void_p(v):
    import ctypes
    return ctypes.c_void_p(v)


def ctypes_buffer(xfem, nfloats):
    import ctypes
    p = xfem.lib().xfem_alloc_host(4 * nfloats)
    if not p:
        raise MemoryError("pinned allocation failed")
    return (ctypes.c_float * nfloats).from_address(p)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xfem", choices=["xfem", "reference"])
    ap.add_argument("--sync-mode", type=int, default=0)
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--bricks", type=int, default=0, help="bricks of the brick launch form (0: one per SM)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-damped", action="store_true")
    ap.add_argument("--no-models", action="store_true")
    ap.add_argument("--no-setup", action="store_true")
    ap.add_argument("--no-hexes", action="store_true")
    ap.add_argument("--no-t10", action="store_true")
    ap.add_argument("--no-h27", action="store_true")
    ap.add_argument("--no-drop", action="store_true")
    ap.add_argument("--adjoint-only", choices=["beam", "large", "both"], default=None,
                    help="time only the adjoint (no main metric line)")
    ap.add_argument("--adjoint-substeps", type=int, default=None, help="substeps of the large adjoint case")
    ap.add_argument("--adjoint-reps", type=int, default=5)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.adjoint_only:
        import torch
        stream = torch.cuda.Stream()
        cases = ("beam", "large") if args.adjoint_only == "both" else (args.adjoint_only,)
        print(json.dumps({"adjoint": run_adjoint(stream, args.adjoint_reps, cases, args.adjoint_substeps)}), flush=True)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_xfem(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
