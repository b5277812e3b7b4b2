"""Benchmark of the estimate-and-mark pass (vertices/s).

One step = one pass of gradient-at-IP -> SPR recovery -> SPR size field ->
metric edge lengths -> split/collapse mark bitmaps over a 160^3 jittered
box (24.6M tets, 4.17M vertices; Gaussian bumps + ramp, adapt ratio 0.008),
inputs resident in HBM.  The default form is the plain FP32 path (FP32 fits
and sweeps, FP64 for ill-conditioned patches and near-threshold edges); its
size-field error and mark agreement against the FP64 path (which equals the
oracle to 1e-10) are measured outside the timed region and reported.  `value` is whole-job vertices/s; `e2e` runs the
same pass through the public host API (sprg_estimate_and_mark) with pinned
host buffers, copies included.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|fp32]
  python bench.py --impl reference ...   # the reference's CPU path (compiled from
                                         # source where its tree is present; else
                                         # the oracle port) on the host cores

Multi-GPU: one process per GPU (torchrun), each an independent replica of
the workload (the pass needs no exchange); value = total vertices / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SPR estimate+mark vertices/sec at 24.6M tets: learned vs plain, at stated size-field error"
UNIT = "vertices/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="fp32", choices=["fp64", "fp32", "learned"],
                   help="form of the headline line: plain FP32 (exact marks), FP64, or learned")
    p.add_argument("--workload", default="jbox", choices=["jbox", "batched", "aniso2d", "order"],
                   help="jbox: 160^3 jittered box (the headline); batched: 4096 uneven boxes; "
                        "aniso2d: 4096^2 anisotropic square")
    p.add_argument("--no-compare", action="store_true", help="skip the learned / FP64 comparison blocks")
    p.add_argument("--n", type=int, default=160, help="box cells per side (160 -> 24.6M tets)")
    p.add_argument("--adapt-ratio", type=float, default=0.008,
                   help="getSPRSizeField adapt ratio (0.008 gives a balanced split/collapse mix at 160^3)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-accuracy", action="store_true", help="skip the FP64 comparison of the FP32 result")
    p.add_argument("--tiling", default=None,
                   help="fix the FP32 recovery's launch shape instead of autotuning it: "
                        "LANES:TILE_VERTS:BLOCKS_PER_SM, LANES four comma-separated lane modes (0 sliced, 1, 2, 4)")
    return p.parse_args()


def parse_tiling(text):
    """--tiling LANES:TILE_VERTS:BLOCKS_PER_SM -> ([four lane modes], tile_verts, blocks_per_sm)."""
    parts = text.split(":")
    if len(parts) != 3:
        raise ValueError("--tiling wants LANES:TILE_VERTS:BLOCKS_PER_SM")
    lanes = [int(x) for x in parts[0].split(",")]
    if len(lanes) != 4 or any(l not in (0, 1, 2, 4) for l in lanes):
        raise ValueError("--tiling wants four lane modes out of 0 (sliced), 1, 2, 4")
    tile_verts, blocks = int(parts[1]), int(parts[2])
    if tile_verts <= 0 or blocks <= 0:
        raise ValueError("--tiling wants a positive tile size and block count")
    return lanes, tile_verts, blocks


def workload_desc(n, precision, adapt_ratio=0.008):
    V, T, E = (n + 1) ** 3, 6 * n ** 3, 3 * n * (n + 1) ** 2 + 3 * n ** 2 * (n + 1) + n ** 3
    return {"workload": f"{n}^3 jittered unit box, {T} tets, {V} vertices, {E} edges; u = 4 Gaussian bumps "
                        f"+ linear ramp (seed 4); interior jitter +-0.2h (seed 4); getSPRSizeField adapt_ratio {adapt_ratio}; "
                        f"split/collapse bitmaps", "precision": precision, "n_verts": V, "n_elems": T, "n_edges": E,
            "l2": "inputs larger than L2 (working set > 129 MB)"}


def build_workload(n):
    from core_gb300 import workload
    m = workload.box(n, jitter=0.2, seed=4)
    u = workload.bump_field(m.coords, seed=4)
    return m, u


# ---------------------------------------------------------------------------
# algorithmic bytes per launch (one touch of each array the kernel needs)
# ---------------------------------------------------------------------------
def pass_bytes(V, T, E):
    """Algorithmic bytes of one whole pass: FP32 values and int32 indices, each
    array touched once per dependency phase (recover 32V+32T, error 28V+20T,
    element size + average 20V+44T, measure + mark 16V+8.25E)."""
    return 96 * V + 96 * T + 8.25 * E


def algorithmic_bytes(kernel, V, T, E, vb=8):
    ib = 4
    table = {
        "grad_ip_f64": 4 * ib * T + 3 * vb * V + vb * V + 3 * vb * T,
        "recover_f64": ib * (V + 1) + 4 * ib * T + 4 * ib * T + 3 * vb * V + 3 * vb * T + 3 * vb * V,
        "error_f64": 4 * ib * T + 3 * vb * V + 3 * vb * T + 3 * vb * V + vb * T,
        "esize_f64": 4 * ib * T + 3 * vb * V + vb * T + vb * T,
        "average_f64": ib * (V + 1) + 4 * ib * T + vb * T + vb * V,
        "measure_f64": 2 * ib * E + 3 * vb * V + vb * V + vb * E,
        "mark_bits": vb * E + E // 4,
        # FP32 path: 32-byte vertex records (coordinates + field pair), 16-byte
        # packed element gradients and recovered values, per-mesh geometry
        "prep_f32": 8 * V + 32 * V + 32 * V,
        "tet_f32": 4 * ib * T + 32 * V + 16 * T,
        "recover_f32": ib * (V + 1) + 4 * ib * T + 4 * 4 * T + 16 * T + 16 * V,
        "error_f32": 4 * ib * T + 16 * T + 8 * T + 16 * V + 8 * T,
        "average_f32": ib * (V + 1) + 4 * ib * T + 8 * T + 8 * V,
        "measure_f32": 2 * ib * E + 4 * E + 8 * V + E // 4,
        # learned form: 16-byte vertex records in, 32-byte records out of the
        # network kernel, FP32 element errors
        "prep_l": 8 * V + 16 * V + 16 * V,
        "mlp_l": ib * (V + 1) + 2 * ib * E + 16 * V + 32 * V,
        "error_l": 4 * ib * T + 32 * V + 8 * T + 4 * T,
        "average_l": ib * (V + 1) + 4 * ib * T + 4 * T + 4 * V,
        "measure_l": 2 * ib * E + 4 * E + 4 * V + E // 4,
    }
    return table.get(kernel)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
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
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        return summarize_clocks(self.lines)


def summarize_clocks(lines):
    """Clock record of the timed region from nvidia-smi CSV rows (the
    ClockSampler.FIELDS columns, no header or units): median SM clock, the
    maximum SM clock and every throttle reason seen active in any row."""
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        parts = [x.strip() for x in ln.split(",")]
        if len(parts) < 9:
            continue
        try:
            sm.append(float(parts[1]))
            smax.append(float(parts[2]))
        except ValueError:
            continue
        for nm, val in zip(names, parts[5:9]):
            if val.lower() == "active":
                reasons.add(nm)
    return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU arms
# ---------------------------------------------------------------------------
def cpu_sample(n, seed=4):
    """The CPU baselines' sample: the n^3 box of the benchmark's family, built
    by the oracle's own MDS box builder (no product code is loaded), interior
    jitter +-0.2h and the 4-bump + ramp field with the benchmark's seed,
    restated with numpy (the same numbers core_gb300.workload gives)."""
    import oracle
    o = oracle.OracleMesh.box(n, n, n)
    x = o.coords.copy()
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.uniform(-0.2 / n, 0.2 / n, size=x.shape)
    d[np.any((x == 0.0) | (x == 1.0), axis=1)] = 0.0
    x = x + d
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, size=(4, 3))
    w = rng.uniform(0.05, 0.2, size=4)
    u = x @ np.array([0.3, -0.2, 0.1])
    for k in range(4):
        u = u + np.exp(-((x - c[k]) ** 2).sum(axis=1) / (2 * w[k] ** 2))
    o.set_coords(x)
    return o, x, u


def cpu_port_run(budget_s, threads, n=48, ratio=0.008):
    """Times the oracle port of the reference path (C, the reference's
    operation order, pinned bitwise to it) on `threads` host threads on a
    bounded sample of the benchmark's workload family.  Returns (vertices/s,
    desc)."""
    import oracle
    used = oracle.set_threads(threads)
    ratio = ratio * n / 160.0
    o, _, u = cpu_sample(n)
    o.estimate_and_mark(u, ratio)  # warm
    t0 = time.perf_counter()
    passes = 0
    while True:
        rc = o.estimate_and_mark(u, ratio)[0]
        assert rc == 0
        passes += 1
        el = time.perf_counter() - t0
        if el >= budget_s or passes >= 1000:
            break
    V = (n + 1) ** 3
    return V * passes / el, {"cores": used, "kind": "port",
                             "sample": f"{passes} passes of the {n}^3 jittered box ({V} vertices, {6 * n ** 3} tets, "
                                       f"adapt ratio {ratio:g}) in {el:.1f} s on {used} threads (oracle port, "
                                       "OpenMP; pinned bitwise to the reference by tests/test_reference_pin.py)"}


def cpu_reference_run(budget_s, n=24, ratio=0.008):
    """Times the reference's own path, compiled from its sources
    (oracle/_ref/libspr_ref.so): getGradIPField -> getSPRSizeField ->
    ma::configure -> markEdgesToCollapse -> markEdgesToSplit on an
    apf::makeMdsBox mesh with the sample's coordinates and field, on one host
    core (the path is serial).  Returns (vertices/s, desc) or None where the
    library is absent (hosts without the reference tree)."""
    from oracle import reference
    if not reference.available():
        return None
    ratio = ratio * n / 160.0
    _, x, u = cpu_sample(n)
    r = reference.RefMesh.box(n, n, n)
    r.set_coords(x)
    passes, el, ph = 0, 0.0, np.zeros(4)
    while el < budget_s and passes < 100:
        *_, sec = r.estimate_and_mark(u, ratio)
        ph += sec
        el += float(sec.sum())
        passes += 1
    V = (n + 1) ** 3
    return V * passes / el, {"cores": 1, "kind": "reference",
                             "sample": f"{passes} passes of the {n}^3 jittered box ({V} vertices, {6 * n ** 3} tets, "
                                       f"adapt ratio {ratio:g}) in {el:.1f} s on 1 core (the reference, serial; "
                                       f"phases gradient {ph[0] / passes:.3f} s, size field {ph[1] / passes:.3f} s, "
                                       f"configure {ph[2] / passes:.3f} s, marks {ph[3] / passes:.3f} s per pass; "
                                       f"{os.cpu_count()} host cores)"}


def cpu_baseline_run(budget_s, ratio):
    """The reference itself where it was built on this host, else the port on
    every host thread."""
    got = cpu_reference_run(budget_s, ratio=ratio)
    if got is None:
        got = cpu_port_run(budget_s, os.cpu_count() or 1, ratio=ratio)
    return got


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = []
    desc = None
    budget = max(1.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    for i in range(args.warmup + args.steps):
        v, desc = cpu_baseline_run(budget, args.adapt_ratio)
        if i >= args.warmup:
            steps.append(v)
    value = float(np.mean(steps))
    note = ("the reference's own path, compiled from its sources (oracle/Makefile refall), on one core"
            if desc["kind"] == "reference" else
            "the reference's source tree is not on this host, so its path cannot be compiled here; the oracle port "
            "(C, the reference's operation order and FP64 arithmetic, pinned bitwise to the compiled reference's "
            "outputs by tests/test_reference_pin.py and tests/golden/ref_path.npz) is timed instead, on every host "
            "thread, on a bounded sample of the same workload family; no product library is loaded")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": dict(workload_desc(args.n, args.precision, args.adapt_ratio),
                          form="plain " + args.precision.upper(),
                          sample="bounded CPU sample of the workload family (see cpu_baseline.sample)"),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": desc["cores"], "kind": desc["kind"],
                            "sample": desc["sample"]},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": note}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def host_placement():
    """Where the host side of the end-to-end calls runs: the CPUs this
    process may use and the host's NUMA nodes."""
    out = {"cpus_allowed": len(os.sched_getaffinity(0)), "host_cpus": os.cpu_count()}
    try:
        out["numa_nodes"] = sorted(int(d[4:]) for d in os.listdir("/sys/devices/system/node") if d.startswith("node"))
    except OSError:
        pass
    return out


def job_throughput(ms_local, units_per_rank, steps, world, device=None):
    """Whole-job throughput of `world` independent replicas: the slowest
    rank's time (all-reduce MAX) for world x units x steps.  Returns
    (ms_max, units per second)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    ms_max = float(t.item())
    return ms_max, world * units_per_rank * steps / (ms_max / 1e3)


def time_form(m, u, precision, ratio, steps, dev, s64=None, f64=None):
    """Resident pass of one form on the same mesh: ms per pass (CUDA events
    on the launching stream, after warm-up) and, given the FP64 sizes and
    flags, the size error and mark agreement of its host-API result."""
    import torch
    import core_gb300 as cg
    E = m.n_edges
    nw = (E + 31) // 32
    with cg.Context(m, device=dev.index or 0, precision=precision) as c:
        st = torch.cuda.Stream(dev)
        c.set_stream(st.cuda_stream)
        d_u = torch.from_numpy(u).to(dev)
        bits = torch.zeros(2 * nw, dtype=torch.int32, device=dev)
        ps, pc = bits.data_ptr(), bits.data_ptr() + 4 * nw
        for _ in range(3):
            c.estimate_and_mark_resident(d_u.data_ptr(), ratio, ps, pc)
        torch.cuda.synchronize(dev)
        launches = int(c.last_launch_count)
        run = lambda: c.estimate_and_mark_resident(d_u.data_ptr(), ratio, ps, pc)
        try:  # replayed from a CUDA graph, as the headline form
            c.graph_capture(d_u.data_ptr(), ratio, ps, pc)
            run = c.graph_replay
            run()
        except Exception:
            pass
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            run()
        e1.record(st)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        out = {"ms_per_step": ms, "value": m.n_verts / (ms / 1e3), "unit": UNIT, "gpu_launches_per_step": launches}
        if s64 is not None:
            c.set_stream(0)
            s, f, _, _, info = c.estimate_and_mark(u, ratio)
            fin = np.isfinite(s) & np.isfinite(s64)
            rel = np.abs(s[fin] - s64[fin]) / np.abs(s64[fin])
            out.update({"size_rel_err_median": float(np.median(rel)), "size_rel_err_p99": float(np.percentile(rel, 99)),
                        "size_rel_err_max": float(rel.max()), "mark_agreement": float(np.mean(f == f64)),
                        "marks_identical": bool(np.array_equal(f, f64))})
            if precision == "learned":
                out["fallback_vertices"] = int(info["n_learned_fallback"])
    return out


def gpu_arm(args):
    import torch
    import torch.distributed as dist
    import core_gb300 as cg
    from core_gb300.mesh import Mesh

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    t_build = time.perf_counter()
    m, u = build_workload(args.n)
    t_mesh = time.perf_counter() - t_build
    V, T, E = m.n_verts, m.n_elems, m.n_edges
    t0 = time.perf_counter()
    ctx = cg.Context(m, device=local, precision=args.precision)
    torch.cuda.synchronize(dev)
    t_flatten = time.perf_counter() - t0
    # an explicit stream: the library launches on it and the timing events are
    # recorded on it (the legacy default stream's handle is 0, which the
    # library reads as "use the context's own stream")
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    if args.tiling:
        ctx.set_tiling(*parse_tiling(args.tiling))
    d_u = torch.from_numpy(u).to(dev)
    nw = (E + 31) // 32
    bits = torch.zeros(2 * nw, dtype=torch.int32, device=dev)
    ps, pc = bits.data_ptr(), bits.data_ptr() + 4 * nw

    def step():
        ctx.estimate_and_mark_resident(d_u.data_ptr(), args.adapt_ratio, ps, pc)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    launches_per_step = ctx.last_launch_count
    # the timed steps replay the resident pass from a CUDA graph captured
    # after the warm-up (the same kernels and arguments, without the launch
    # gaps); direct launches if the capture is refused
    replay = step
    try:
        ctx.graph_capture(d_u.data_ptr(), args.adapt_ratio, ps, pc)
        replay = ctx.graph_replay
        for _ in range(2):
            replay()
    except Exception:
        replay = step
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        replay()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms_max, value = job_throughput(ms_total, V, args.steps, world, dev)
    # per-kernel times: CUDA events around every launch of as many direct
    # passes right after the timed replays (events cannot sit inside the
    # replayed graph)
    ctx.profile(True)
    ctx.profile_report(reset=True)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.steps):
        step()
    p1.record(stream)
    torch.cuda.synchronize(dev)
    ms_profiled = p0.elapsed_time(p1) / args.steps
    prof = ctx.profile_report(reset=True)
    ctx.profile(False)

    # the per-mesh work an adapt loop repays after every topology change:
    # the first pass on a new context (coordinate records, geometry, SPR
    # weights, listed patches' growth and QR, bins, autotuner) and the first
    # pass after sprg_update_mesh (one interior vertex moved by 1e-3 h)
    first = {}
    if rank == 0:
        def timed_first_pass(c):
            c.set_stream(stream.cuda_stream)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            c.estimate_and_mark_resident(d_u.data_ptr(), args.adapt_ratio, ps, pc)
            torch.cuda.synchronize(dev)
            return round((time.perf_counter() - t0) * 1e3, 2)
        t0 = time.perf_counter()
        c_new = cg.Context(m, device=local, precision=args.precision)
        torch.cuda.synchronize(dev)
        first["new_context_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        first["first_pass_ms"] = timed_first_pass(c_new)
        moved = Mesh(m.dim, m.coords.copy(), m.elem_verts, m.edge_verts, m.v2e_off, m.v2e, m.grid)
        iv = int(np.nonzero(~m.boundary_vertices())[0][0])
        moved.coords[iv] += 1e-3 / args.n
        t0 = time.perf_counter()
        delta = cg.mesh_delta(m, moved)  # host diff of the flattened arrays (a caller that knows its rows skips it)
        first["mesh_delta_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        t0 = time.perf_counter()
        c_new.update_mesh(moved, delta=delta)
        torch.cuda.synchronize(dev)
        first["update_mesh_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        first["first_pass_after_update_ms"] = timed_first_pass(c_new)
        first["second_pass_after_update_ms"] = timed_first_pass(c_new)
        c_new.close()

    # e2e through the host API: pinned u in, flags + size out, every step
    e2e = None
    if not args.no_e2e:
        u_pin = torch.from_numpy(u).pin_memory().numpy()
        ctx.set_stream(0)
        k = max(3, min(args.steps, 10))
        # one fresh (all clear) ma_flags array per step, pinned, prepared
        # before the timed region: each step uploads u and its flags, runs the
        # pass and reads the marked flags and the size field back
        flag_sets = [torch.zeros(E, dtype=torch.int32).pin_memory().numpy() for _ in range(k + 3)]
        size_pin = torch.zeros(V, dtype=torch.float64).pin_memory().numpy()
        # three warm-up calls: the entry point captures its pass into a CUDA
        # graph on the third call with the same inputs and replays it after
        for i in range(3):
            ctx.estimate_and_mark(u_pin, args.adapt_ratio, flag_sets[k + i], size_pin)
        t0 = time.perf_counter()
        for i in range(k):
            _, _, ns, nc, _ = ctx.estimate_and_mark(u_pin, args.adapt_ratio, flag_sets[i], size_pin)
        el = time.perf_counter() - t0
        # the same calls again with the entry point's stage timing on (events
        # at its stage boundaries), outside the timed loop
        ctx.e2e_timing(True)
        for i in range(k):
            flag_sets[i][:] = 0
            ctx.estimate_and_mark(u_pin, args.adapt_ratio, flag_sets[i], size_pin)
        e2e_phases = ctx.e2e_timing_report()
        ctx.e2e_timing(False)
        e2e = {"value": world * V * k / el, "unit": UNIT, "h2d_bytes_per_step": int(8 * V + 4 * E),
               "d2h_bytes_per_step": int(4 * E + 8 * V), "steps": k, "n_split": ns, "n_collapse": nc,
               "ms_per_call": el / k * 1e3, "phases": e2e_phases, "host": host_placement()}
        ctx.set_stream(stream.cuda_stream)

    # accuracy of the FP32 result against the FP64 path, outside the timed region
    acc = None
    compare = None
    if rank == 0 and not (args.no_accuracy and args.no_compare):
        with cg.Context(m, device=local, precision="fp64") as c64:
            s64, f64, *_ = c64.estimate_and_mark(u, args.adapt_ratio)
    if args.precision != "fp64" and not args.no_accuracy and rank == 0:
        ctx.set_stream(0)
        s32, f32, *_ = ctx.estimate_and_mark(u, args.adapt_ratio)
        fin = np.isfinite(s32) & np.isfinite(s64)
        rel = np.abs(s32[fin] - s64[fin]) / np.abs(s64[fin])
        acc = {"size_rel_err_max": float(rel.max()), "size_rel_err_p99": float(np.percentile(rel, 99)),
               "size_rel_err_median": float(np.median(rel)), "mark_agreement": float(np.mean(f32 == f64)),
               "marks_identical": bool(np.array_equal(f32, f64)),
               "against": "FP64 path (equal to the oracle within 1e-10 relative)"}
        ctx.set_stream(stream.cuda_stream)
    if rank == 0 and not args.no_compare:
        # the learned-vs-plain comparison of the metric, and the FP64 path
        compare = {}
        for form in ("fp32", "learned", "fp64"):
            if form == args.precision:
                continue
            compare[form] = time_form(m, u, form, args.adapt_ratio, args.steps if form != "fp64" else 3, dev, s64, f64)

    if rank != 0:
        ctx.close()
        if world > 1:
            dist.destroy_process_group()
        return

    # roofline of the dominant kernel
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    phases = {k: {"launches": n, "total_ms": ms, "avg_ms": ms / max(n, 1)} for k, (n, ms) in prof.items()}
    dom = max(prof.items(), key=lambda kv: kv[1][1])[0] if prof else None
    roof = None
    if dom:
        n_l, ms = prof[dom]
        avg = ms / n_l
        vb = 8 if args.precision == "fp64" else 4
        byts = algorithmic_bytes(dom, V, T, E, vb)
        traffic = None
        if dom == "mlp_l":
            # the network kernel is a contraction: tensor FLOPs per vertex
            # (K = 64 first layer for <= 16 neighbours: 64x64 + 64x64 + 16x64 MACs)
            flops = 2.0 * (64 * 64 + 64 * 64 + 16 * 64) * V
            tf = peaks.get("bf16_tflops") or 1900.0
            ach = flops / (avg / 1e3) / 1e12
            roof = {"bound": "tensor", "kernel": dom, "achieved": ach, "peak": tf, "unit": "TFLOP/s",
                    "frac": ach / tf, "traffic": None, "algorithmic_flops": flops, "avg_ms": avg,
                    "peak_source": "measured (MEASURED_PEAKS.json bf16_tflops)" if peaks.get("bf16_tflops")
                    else "fallback 1900 TFLOP/s"}
            byts = None
        tf = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tf):
            traffic = json.load(open(tf)).get(f"{dom}@{args.n}")
        if byts and dom != "mlp_l":
            ach = byts / (avg / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s",
                    "frac": ach / hbm, "traffic": traffic, "algorithmic_bytes": byts, "avg_ms": avg,
                    "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else
                    "fallback 6800 GB/s"}
    cpu = None
    if not args.no_cpu_baseline:
        try:
            v, desc = cpu_baseline_run(args.cpu_seconds, args.adapt_ratio)
            cpu = {"value": v, "unit": UNIT, "cores": desc["cores"], "kind": desc["kind"], "sample": desc["sample"]}
        except Exception as e:  # the baseline is reported, never the target
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"unavailable: {e}"}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": {"fp64": "f64", "fp32": "f32", "learned": "bf16/f32"}[args.precision],
           "data": "synthetic", "config": dict(workload_desc(args.n, args.precision, args.adapt_ratio),
                                                 form="plain " + args.precision.upper()), "roofline": roof,
           "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches_per_step * args.steps),
           "clocks": clk, "phases": phases, "timed_by": "CUDA graph replay" if replay != step else "direct launches",
           "ms_per_step_profiled_direct": ms_profiled, "accuracy": acc, "forms": compare,
           "pass_roofline": {"algorithmic_bytes": pass_bytes(V, T, E),
                             "achieved": pass_bytes(V, T, E) / (ms_max / args.steps / 1e3) / 1e9, "peak": hbm,
                             "unit": "GB/s",
                             "frac": pass_bytes(V, T, E) / (ms_max / args.steps / 1e3) / 1e9 / hbm},
           "setup_s": dict({"mesh_build": round(t_mesh, 3), "flatten_upload": round(t_flatten, 3)}, **first)}
    if args.precision == "fp32":
        tr = ctx.tuning_report()
        out["tuning"] = {k: tr[k] for k in ("bins", "lanes", "tile_verts", "blocks_per_sm") if k in tr}
    print(json.dumps(out), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def gpu_batched(args):
    """The batched workload: 4096 uneven boxes (n log-uniform in [4, 40],
    1-8 bumps each) in one context, FP32 with the FP64 guard, autotuned
    binned recovery, the pass replayed from a CUDA graph."""
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    m, u, voff, eoff, doff, ns = workload.batch_boxes(4096, seed=3)
    t_mesh = time.perf_counter() - t0
    V, T, E = m.n_verts, m.n_elems, m.n_edges
    nw = (E + 31) // 32
    with cg.Context(m, precision="fp32") as c:
        c.set_batch(voff, eoff, np.full(len(ns), 0.1))
        st = torch.cuda.Stream(dev)
        torch.cuda.set_stream(st)
        c.set_stream(st.cuda_stream)
        d_u = torch.from_numpy(u).to(dev)
        bits = torch.zeros(2 * nw, dtype=torch.int32, device=dev)
        ps, pc = bits.data_ptr(), bits.data_ptr() + 4 * nw
        c.graph_capture(d_u.data_ptr(), 1.0, ps, pc)
        for _ in range(args.warmup):
            c.graph_replay()
        clocks = ClockSampler(0)
        clocks.start()
        time.sleep(0.3)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            c.graph_replay()
        e1.record(st)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
        clk = clocks.stop()
        # per-kernel times from as many direct, event-bracketed passes
        c.profile(True)
        c.profile_report(reset=True)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(st)
        for _ in range(args.steps):
            c.estimate_and_mark_resident(d_u.data_ptr(), 1.0, ps, pc)
        p1.record(st)
        torch.cuda.synchronize(dev)
        ms_direct = p0.elapsed_time(p1) / args.steps
        prof = c.profile_report(reset=True)
        c.profile(False)
        tune = c.tuning_report()
        c.set_stream(0)
        _, flags, _, _, info = c.estimate_and_mark(u, 1.0)
    # marks of a sample of the meshes (every 32nd) against each mesh's own
    # FP64 pass (the FP64 path equals the reference's marks)
    from core_gb300.mesh import Mesh
    sample = list(range(0, len(ns), 32))
    differ = 0
    for k in sample:
        mk = Mesh(3, m.coords[voff[k]:voff[k + 1]], m.elem_verts[eoff[k]:eoff[k + 1]] - voff[k],
                  m.edge_verts[doff[k]:doff[k + 1]] - voff[k])
        with cg.Context(mk, precision="fp64") as c64:
            _, f64, *_ = c64.estimate_and_mark(u[voff[k]:voff[k + 1]], 0.1)
        differ += int(np.sum(f64 != flags[doff[k]:doff[k + 1]]))
    marks = {"meshes_checked": len(sample), "edges_checked": int(sum(doff[k + 1] - doff[k] for k in sample)),
             "differing_flag_words": differ, "against": "each mesh's own FP64 pass"}
    out = {"metric": METRIC, "value": V / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"4096 unit tet boxes, n per side log-uniform in [4, 40] (seed 3), 1-8 Gaussian "
                                  f"bumps each; {V} vertices, {T} tets, {E} edges; adapt ratio 0.1 per mesh",
                      "form": "plain FP32, batched, CUDA graph", "l2": "inputs larger than L2"},
           "tuning": tune, "guard_edges": int(info["n_guard_edges"]), "marks": marks,
           "listed_patches": int(info["n_expanded"] + info["n_fp64_refits"]), "clocks": clk,
           "timed_by": "CUDA graph replay", "ms_per_step_profiled_direct": ms_direct,
           "phases": {k: {"launches": n, "total_ms": t, "avg_ms": t / max(n, 1)} for k, (n, t) in prof.items()},
           "setup_s": {"mesh_build": round(t_mesh, 2)}}
    print(json.dumps(out), flush=True)


def gpu_aniso2d(args):
    """The 2D anisotropic workload: 4096^2 square (33.5M triangles), nodal
    Hessian by two SPR recoveries, metric, AnisoSizeField measure, marks and
    quality.  Two forms: FP64 throughout (the reference's arithmetic; patch
    QR in its operation order) and the mixed form (SPRG_FP32: recoveries from
    cached FP64 patch weights, FP64 metric, FP32 measure with the FP64 guard
    band, FP32 qualities).  The line is the --precision form (fp32 = mixed);
    `forms` holds both with the mark comparison."""
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    n = 4096
    m, u, (eps, hmin, hmax) = workload.aniso2d(n)
    V, T, E = m.n_verts, m.n_elems, m.n_edges
    nw = (E + 31) // 32

    def run_form(precision, m=m, u=u, eps=eps, hmin=hmin, hmax=hmax):
        T, E = m.n_elems, m.n_edges
        nw = (E + 31) // 32
        with cg.Context(m, precision=precision) as c:
            st = torch.cuda.Stream(dev)
            torch.cuda.set_stream(st)
            c.set_stream(st.cuda_stream)
            d_u = torch.from_numpy(u).to(dev)
            bits = torch.zeros(2 * nw, dtype=torch.int32, device=dev)
            q = torch.zeros(T, dtype=torch.float64, device=dev)
            run = lambda: c.aniso_estimate_and_mark_resident(d_u.data_ptr(), eps, hmin, hmax, bits.data_ptr(),
                                                              bits.data_ptr() + 4 * nw, q.data_ptr())
            for _ in range(max(1, args.warmup)):
                run()
            torch.cuda.synchronize(dev)
            c.profile(True)
            c.profile_report(True)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            steps = min(args.steps, 5)
            e0.record(st)
            for _ in range(steps):
                run()
            e1.record(st)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / steps
            prof = c.profile_report(True)
            guard = int(c.debug_read("agcount", np.int32, 1)[0]) if precision == "fp32" else 0
            launches = c.last_launch_count
            res = (bits.cpu().numpy().view(np.uint32).copy(), q.cpu().numpy())
        return ms, steps, prof, guard, launches, res

    forms = {}
    results = {}
    main_form = "fp32" if args.precision == "fp32" else "fp64"
    # --no-compare: the line's form alone (no FP64 comparison pass)
    for prec in (main_form,) if args.no_compare else ("fp64", "fp32"):
        ms, steps, prof, guard, launches, res = run_form(prec)
        results[prec] = res
        forms[prec] = {"ms_per_step": ms, "value": V / (ms / 1e3), "unit": UNIT, "steps": steps,
                       "gpu_launches_per_step": launches,
                       "phases": {k: {"launches": nl, "total_ms": t, "avg_ms": t / max(nl, 1)}
                                  for k, (nl, t) in prof.items()}}
        if prec == "fp32":
            forms[prec]["guard_edges"] = guard
    if "fp64" in results and "fp32" in results:
        b64, q64 = results["fp64"]
        b32, q32 = results["fp32"]
        rel = np.abs(q32 - q64) / np.maximum(np.abs(q64), 1e-300)
        forms["fp32"].update({"marks_identical": bool(np.array_equal(b32, b64)),
                              "quality_rel_err_max": float(rel.max()),
                              "quality_rel_err_median": float(np.median(rel))})
    if not args.no_compare:
        # the batched form: uneven squares with their own fields in one
        # context (a disjoint union; the anisotropic pass has no reduction
        # across vertices), both forms, marks compared
        mb, ub, voff, eoff, doff, ns = workload.batch_squares(256, seed=5, lo=32, hi=512)
        pb = workload.aniso2d_params(256)
        bat = {"meshes": int(len(ns)), "vertices": int(mb.n_verts), "triangles": int(mb.n_elems),
               "n_range": [int(ns.min()), int(ns.max())], "fields": "1-8 Gaussian bumps per mesh",
               "eps_hmin_hmax": list(pb)}
        bres = {}
        for prec in ("fp64", "fp32"):
            ms, steps, prof, guard, launches, res = run_form(prec, mb, ub, *pb)
            bres[prec] = res
            bat[prec] = {"ms_per_step": ms, "value": mb.n_verts / (ms / 1e3), "unit": UNIT,
                         "gpu_launches_per_step": launches}
            if prec == "fp32":
                bat[prec]["guard_edges"] = guard
        bat["marks_identical"] = bool(np.array_equal(bres["fp32"][0], bres["fp64"][0]))
        forms["batched"] = bat
    f = forms[main_form]
    out = {"metric": METRIC, "value": f["value"], "unit": UNIT, "n_gpus": 1, "steps": f["steps"],
           "warmup": args.warmup, "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64/f32" if main_form == "fp32" else "f64", "data": "synthetic",
           "config": {"workload": f"{n}^2 unit square, {T} triangles, {V} vertices, {E} edges, interior jitter "
                                  f"+-0.15h (seed 5); u = tanh((y-0.5)/1e-3) + 0.1 sin(8 pi x); Hessian by two SPR "
                                  f"recoveries, metric eps {eps:.3g}, h in [{hmin:.3g}, {hmax:.3g}]; AnisoSizeField "
                                  f"measure, marks, quality",
                      "form": "mixed (FP64 recovery and metric decisions, FP32 metric records, measure + FP64 "
                              "guard, FP32 quality)" if main_form == "fp32" else "FP64"},
           "gpu_launches": f["gpu_launches_per_step"] * f["steps"],
           "phases": f["phases"], "forms": forms}
    print(json.dumps(out), flush=True)


def gpu_order(args):
    """Locality renumbering: the plain FP32 pass on the jittered n^3 box in its
    own (makeMdsBox) numbering, with every entity kind's numbering randomly
    shuffled, and on the shuffled mesh after core_gb300.mesh.reorder
    (sprg_locality_order); marks of the shuffled and renumbered passes mapped
    back and compared with the ordered box's."""
    import torch
    import core_gb300 as cg
    from core_gb300.mesh import reorder
    n = args.n if args.n != 160 else 96
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    m, u = build_workload(n)
    rng = np.random.Generator(np.random.PCG64(9))
    ms, vs, ts, es = reorder(m, rng.permutation(m.n_verts).astype(np.int32),
                             rng.permutation(m.n_elems).astype(np.int32), rng.permutation(m.n_edges).astype(np.int32))
    us = np.empty_like(u)
    us[vs] = u
    t0 = time.perf_counter()
    mr, vr, tr, er = reorder(ms)
    t_order = time.perf_counter() - t0
    ur = np.empty_like(us)
    ur[vr] = us
    ratio = args.adapt_ratio * n / 160.0
    out, flags = {}, {}
    for name, mm, uu in (("ordered", m, u), ("shuffled", ms, us), ("renumbered", mr, ur)):
        out[name] = time_form(mm, uu, "fp32", ratio, args.steps, dev)
        with cg.Context(mm, precision="fp32") as c:
            flags[name] = c.estimate_and_mark(uu, ratio)[1]
    same = bool(np.array_equal(flags["renumbered"][er][es], flags["ordered"]) and
                np.array_equal(flags["shuffled"][es], flags["ordered"]))
    V = m.n_verts
    res = {"metric": METRIC, "value": out["renumbered"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": out["renumbered"]["ms_per_step"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{n}^3 jittered box ({V} vertices, {m.n_elems} tets), numbering shuffled, then "
                                  f"locality-renumbered (sprg_locality_order); plain FP32 pass, adapt ratio {ratio:g}",
                      "l2": "inputs larger than L2"},
           "forms": out, "marks_identical_after_mapping_back": same, "renumber_host_s": round(t_order, 3)}
    print(json.dumps(res), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "batched":
        gpu_batched(args)
    elif args.workload == "aniso2d":
        gpu_aniso2d(args)
    elif args.workload == "order":
        gpu_order(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
