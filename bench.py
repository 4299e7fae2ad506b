#!/usr/bin/env python3
"""Benchmark of the implicit soft-body step on GB300: vertex-steps/s of the batched solver.

Workload (default "batch"): 512 independent Kuhn-split tetrahedral blocks of a x b x c vertices,
a, b, c ~ U{4..40} (seeded), Young modulus log-uniform in [1e4, 1e6], Poisson ratio U[0.2, 0.45],
+-1% jitter, one random face pinned, h = 1/60, PCG relative tolerance 1e-5 with at most 200
iterations, FP32 blocks and vectors with FP64 dot products. One "step" is one implicit step of
every body of the batch (one persistent, graph-replayed launch).

Printed on one JSON line: whole-job vertex-steps/s (device-timed, inputs resident), the same
metric end to end through the C ABI with host buffers (e2e), p50/p99 step latency, the plain
one-body-at-a-time GPU path on a sample of the same bodies, the roofline of the batch kernel,
SM clocks sampled during the timed region and the CPU baseline (the oracle's C restatement of
the reference algorithm on this host's cores, on a bounded sample).

--impl reference times that CPU implementation alone on the same workload and prints its own
line. Under torchrun every rank steps its own batch (weak scaling); rank 0 prints.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "vertex-steps/s batched vs plain at resid 1e-5; p50/p99 step latency"
DT = 1.0 / 60.0
PCG_TOL = 1e-5
PCG_MAX = 200
# DRAM traffic / algorithmic bytes of the batch PCG launch, from the ncu capture of the
# 128-body case (profiles/k_batch_batch512.md)
PCG_TRAFFIC_RATIO = 1.072
# steps of the CPU-baseline run and of the parity check, from the bodies' initial state
PARITY_STEPS = 3


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="batch", choices=["batch", "tet64", "cloth128", "tet10", "serve"])
    p.add_argument("--bodies", type=int, default=512)
    p.add_argument("--split", action="store_true",
                   help="several GPUs: one body list split over the ranks by device footprint (strong scaling) "
                        "instead of a batch per rank (weak scaling)")
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "bf16"])
    p.add_argument("--no-extras", action="store_true", help="skip e2e, plain path and CPU baseline")
    p.add_argument("--path", default="plain", choices=["plain", "batch"],
                   help="single-body workloads: the per-op kernels (plain) or the persistent kernel with one body")
    # serving (--workload serve): Poisson arrivals over a pool of bodies
    p.add_argument("--serve-rate", type=float, default=2000.0, help="requests per second")
    p.add_argument("--serve-seconds", type=float, default=60.0, help="length of the arrival stream")
    p.add_argument("--no-serve", action="store_true", help="batch workload: skip the serving sub-run")
    p.add_argument("--serve-grace", type=float, default=5.0, help="seconds to keep serving after the stream")
    p.add_argument("--serve-pool", type=int, default=256, help="distinct bodies of the stream")
    p.add_argument("--serve-max-active", type=int, default=256, help="bodies per launch at most")
    p.add_argument("--serve-budget-gb", type=float, default=64.0, help="device memory for resident bodies")
    p.add_argument("--serve-plain-seconds", type=float, default=10.0, help="plain-path sample length")
    return p.parse_args()


# ------------------------------------------------------------------ distributed plumbing
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "ours" and torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg, device=None):
    if pg is None:
        return
    import torch

    if pg.get_backend() == "nccl":
        pg.barrier(device_ids=[device])
    else:
        pg.barrier()


def max_over_ranks(pg, value: float, device=None) -> float:
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=f"cuda:{device}" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, value: float, device=None) -> float:
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=f"cuda:{device}" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ workload
def split_workload(descs, world, rank):
    """This rank's share of one body list split over `world` GPUs by estimated device bytes
    (b3g_body_desc_estimate_bytes, b3g_partition_bodies: host only, the same split on every rank).
    Returns the indices of this rank's bodies and the estimated bytes of every rank."""
    from bounce_softbody_gb300 import b3g

    sizes = [b3g.estimate_bytes(d) for d in descs]
    owner = b3g.partition(sizes, world)
    mine = [k for k in range(len(descs)) if int(owner[k]) == rank]
    per_rank = [int(sum(s for s, o in zip(sizes, owner) if int(o) == r)) for r in range(world)]
    return mine, per_rank


def gather_rank_stats(pg, stats: dict, world: int):
    """Every rank's stats dict on every rank (host objects: gloo or NCCL)."""
    if pg is None:
        return [stats]
    out = [None] * world
    pg.all_gather_object(out, stats)
    return out


def workload(args, rank, world=1):
    from bounce_softbody_gb300 import meshes

    if args.workload == "batch" and args.split:
        # one list for the whole job, the same on every rank; each rank keeps its share
        descs = meshes.batch_bodies(args.bodies, seed=3)
        mine, per_rank = split_workload(descs, world, rank)
        descs = [descs[k] for k in mine]
        cfg = {"workload": f"batch of {args.bodies} Kuhn tet blocks a,b,c~U{{4..40}} split over {world} GPUs by "
                           f"device footprint", "bodies": args.bodies, "bodies_this_rank": len(descs),
               "estimated_bytes_per_rank": per_rank, "E": "log-uniform 1e4..1e6", "poisson": "U[0.2,0.45]",
               "h": "1/60", "pcg_tol": PCG_TOL, "pcg_max_iter": PCG_MAX}
    elif args.workload == "batch":
        descs = meshes.batch_bodies(args.bodies, seed=3 + 1000 * rank)
        cfg = {"workload": f"batch of {args.bodies} Kuhn tet blocks a,b,c~U{{4..40}}", "bodies": args.bodies,
               "E": "log-uniform 1e4..1e6", "poisson": "U[0.2,0.45]", "h": "1/60", "pcg_tol": PCG_TOL,
               "pcg_max_iter": PCG_MAX}
    elif args.workload == "tet64":
        descs = [meshes.tet_grid(64, 64, 64, seed=rank, E=1e6, nu=0.45, name="tet64")]
        cfg = {"workload": "64^3 Kuhn tet block E=1e6 nu=0.45", "bodies": 1, "h": "1/30", "pcg_tol": PCG_TOL,
               "pcg_max_iter": 2000}
    elif args.workload == "cloth128":
        descs = [meshes.config_cloth128()]
        cfg = {"workload": "128^2 cloth + sphere contact", "bodies": 1, "h": "1/60", "pcg_tol": PCG_TOL,
               "pcg_max_iter": PCG_MAX}
    else:
        descs = [meshes.config_tet10(seed=rank)]
        cfg = {"workload": "10^3 Kuhn tet block", "bodies": 1, "h": "1/60", "pcg_tol": PCG_TOL,
               "pcg_max_iter": PCG_MAX}
    return descs, cfg


def bf16_inner():
    """Inner BF16 iterations per outer iteration of the per-op BF16 mode (the library's default)."""
    return int(os.environ.get("B3G_BF16_INNER", "20"))


def step_dt(args):
    return 1.0 / 30.0 if args.workload == "tet64" else DT


def pcg_max(args):
    return 2000 if args.workload == "tet64" else PCG_MAX


# ------------------------------------------------------------------ algorithmic bytes
def spmv_bytes(info, vs=4, bs=36):
    """One SpMV over the body's blocks: values, column ids, row lengths, x read, y written."""
    n, nnzb = info["vertices"], info["nnzb"]
    return (bs + 4) * nnzb + n + 3 * vs * n + 3 * vs * n


def iteration_bytes(info, vs=4, bs=36):
    """One PCG iteration: SpMV of s + (d, q read; d written: the direction d = s + beta d and
    q = A s + beta q in the SpMV sweep) + update (x, r, d, q, Minv read; x, r, s written)."""
    n = info["vertices"]
    return spmv_bytes(info, vs, bs) + 8 * 3 * vs * n + 3 * 3 * vs * n


def final_bytes(info):
    """Final update of one step: solution read (16 B), state x, v, translation, external force
    read and x, v, external force, translation written (12 B each)."""
    return info["vertices"] * (16 + 4 * 12 + 4 * 12)


def assembly_bytes(info):
    """Element phase and row assembly of one step (first touch of every array, FP32; the
    precomputed contribution lists are not counted)."""
    n, nt, nnzb = info["vertices"], info["tets"], info["nnzb"]
    tets = nt * (16 + 36 + 16 + 16 + 16 + 64 + 48)     # ids, invE, material, q r/w, records, rhs parts
    gathers = n * (12 * 4)                             # x, v, translation, fext
    # blocks written and column ids; each tetrahedron's four records (16 B) and four
    # right-hand-side parts (12 B) read by its vertices' rows; vertex terms and the six vectors
    rows = 40 * nnzb + nt * 4 * 16 + nt * 4 * 12 + n * (4 + 4 + 1 + 12) + n * 12 * 7
    return tets + gathers + rows


# ------------------------------------------------------------------ clocks
class Clocks:
    def __init__(self, device: int):
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU implementation (oracle port)
def stratified(n_items, sizes, every):
    """Indices of every `every`-th item in size order (largest first)."""
    order = sorted(range(n_items), key=lambda k: -sizes[k])
    return order[::every] if n_items > every else order


def run_cpu(descs, steps, dt, max_sub, threads, bits=32):
    """The oracle's C restatement of the reference step on `threads` host threads, from each body's
    initial state. Returns (vertex-steps/s, seconds, iterations, positions, velocities)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    xs, vs, iters, sec = oracle.simulate_batch(descs, steps, dt=dt, max_sub=max_sub, sub_tol=PCG_TOL, bits=bits,
                                               threads=threads)
    return sum(d.n for d in descs) * steps / sec, sec, iters, xs, vs


def rel_errors(x, v, xr, vr, x0):
    """Position error relative to the oracle's displacement, velocity error relative to its norm."""
    xr, vr = np.asarray(xr, np.float64), np.asarray(vr, np.float64)
    ex = float(np.linalg.norm(np.asarray(x, np.float64) - xr) / max(np.linalg.norm(xr - x0), 1e-30))
    ev = float(np.linalg.norm(np.asarray(v, np.float64) - vr) / max(np.linalg.norm(vr), 1e-30))
    return ex, ev


def reference_arm(args, world, rank, pg):
    descs, cfg = workload(args, rank)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    sample = descs  # the whole workload: every body, one step from its initial state per timed step
    dt, mx = step_dt(args), pcg_max(args)
    for _ in range(args.warmup):
        run_cpu(sample, 1, dt, mx, threads)
    times = []
    for _ in range(args.steps):
        _, sec, _, _, _ = run_cpu(sample, 1, dt, mx, threads)
        times.append(sec)
    total = sum(times)
    vs = sum(d.n for d in sample) * args.steps / total
    desc = (f"oracle C restatement (FP32, Jacobi PCG, tol 1e-5) of all {len(descs)} bodies "
            f"({sum(d.n for d in sample)} vertices), 1 step from the initial state per timed step, {threads} threads")
    line = {"metric": METRIC, "value": vs, "unit": "vertex-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes)",
            "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": vs, "unit": "vertex-steps/s", "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": vs, "unit": "vertex-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "p50_step_ms": 1e3 * statistics.median(times), "p99_step_ms": 1e3 * float(np.percentile(times, 99))}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
def ours(args, world, rank, local, pg):
    import torch

    from bounce_softbody_gb300 import b3g

    descs, cfg = workload(args, rank, world)
    dt, mx = step_dt(args), pcg_max(args)
    prec = {"fp32": b3g.PRECISION_FP32, "fp64": b3g.PRECISION_FP64, "bf16": b3g.PRECISION_BF16}[args.precision]
    scfg = b3g.solver_config(max_pcg_iterations=mx, pcg_tolerance=PCG_TOL, precision=prec)
    ctx = b3g.Context(local)
    t0 = time.time()
    bodies = [b3g.Body(ctx, d) for d in descs]
    setup_s = time.time() - t0
    infos = [b.info() for b in bodies]
    nverts = sum(i["vertices"] for i in infos)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)

    single = args.workload != "batch"
    per_op = single and args.path == "plain"

    def step_once():
        if per_op:
            # one body: the per-op kernels of the single-body path (grid-wide SpMV / reductions)
            bodies[0].step(dt, scfg, stats=False)
        else:
            b3g.step_batch(ctx, bodies, dt, 1, scfg, stats=False)

    for _ in range(max(args.warmup, 3)):
        step_once()
    ctx.synchronize()

    # The per-launch timings and the end-to-end leg below restart from the state the timed steps
    # start from: the bodies swing as they step, and a tetrahedron's rotation extraction takes more
    # iterations as its rotation changes faster, so later steps cost more than earlier ones.
    def checkpoint():
        return [(b.state(), b.rotations() if i["tets"] else None) for b, i in zip(bodies, infos)]

    def restore(cp):
        for b, ((x, v), q) in zip(bodies, cp):
            b.set_state(x, v)
            if q is not None:
                b.set_rotations(q)
        ctx.synchronize()

    start_state = checkpoint() if not per_op else None
    before = [b.stats()["total_pcg_iterations"] for b in bodies]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier(pg, local)
    torch.cuda.synchronize(local)
    clocks = Clocks(local)
    ev[0].record(stream)
    for k in range(args.steps):
        step_once()
        ev[k + 1].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize(local)
    clk = clocks.stop()
    barrier(pg, local)
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[args.steps])
    after = [b.stats()["total_pcg_iterations"] for b in bodies]
    iters = [a - b for a, b in zip(after, before)]
    t_max = max_over_ranks(pg, total_ms / 1e3, local)
    value = sum_over_ranks(pg, nverts * args.steps, local) / t_max
    rank_stats = gather_rank_stats(pg, {"rank": rank, "bodies": len(bodies), "vertices": nverts,
                                        "ms_per_step": total_ms / args.steps}, world)

    # rooflines. Whole step: every kernel of the timed region. Persistent path: the PCG launch
    # (the dominant kernel, 78 % of a step) and the assembly launch, each timed live with CUDA
    # events around its own launch on the context's stream (b3g_batch_set_launch_timing) over
    # extra steps run after the timed region.
    bs, vsz = {"fp32": (36, 4), "fp64": (72, 8), "bf16": (18, 4)}[args.precision]
    alg_asm = sum(args.steps * assembly_bytes(i) for i in infos)
    if per_op and args.precision == "bf16":
        # the per-op BF16 mode counts outer iterations of its flexible CG: each is BF16_INNER inner
        # iterations with the bf16 blocks, one FP32 product with its update, and z.q_prev
        m = bf16_inner()
        alg_pcg = sum(it * (m * iteration_bytes(i, 4, 18) + iteration_bytes(i, 4, 36) + 32 * i["vertices"])
                      + args.steps * final_bytes(i) for i, it in zip(infos, iters))
    else:
        alg_pcg = sum(it * iteration_bytes(i, vsz, bs) + args.steps * final_bytes(i) for i, it in zip(infos, iters))
    alg = alg_asm + alg_pcg
    achieved = alg / (total_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    step_roof = {"achieved": achieved, "frac": achieved / peak, "algorithmic_bytes_per_step": alg / args.steps}
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "", "peak_source": f"{peak_kind} hbm_gbs",
            "algorithmic_bytes_per_step": alg / args.steps,
            "pcg_iterations_per_step_mean": float(np.mean(iters)) / args.steps if iters else 0.0}
    if not per_op:
        tsteps = max(3, min(args.steps, 5))
        restore(start_state)
        b3g.batch_set_launch_timing(ctx, True)
        b3g.batch_launch_times(ctx, reset=True)
        before_t = [b.stats()["total_pcg_iterations"] for b in bodies]
        b3g.step_batch(ctx, bodies, dt, tsteps, scfg, stats=False)
        lt = b3g.batch_launch_times(ctx, reset=True)
        b3g.batch_set_launch_timing(ctx, False)
        its_t = [b.stats()["total_pcg_iterations"] - x for b, x in zip(bodies, before_t)]
        pcg_b = sum(it * iteration_bytes(i, vsz, bs) + tsteps * final_bytes(i) for i, it in zip(infos, its_t)) / tsteps
        asm_b = sum(assembly_bytes(i) for i in infos)
        pcg_ms, asm_ms = lt["pcg_ms"] / lt["steps"], lt["assembly_ms"] / lt["steps"]
        ach = pcg_b / (pcg_ms / 1e3) / 1e9
        roof.update({"achieved": ach, "frac": ach / peak, "kernel": "k_batch PCG launch (PCG + final update)",
                     "algorithmic_bytes_per_launch": pcg_b, "launch_ms": pcg_ms, "launches_timed": lt["steps"]})
        # DRAM traffic of the PCG launch: ncu on the 128-body case measured 39.55 GB for
        # 36.90 GB of algorithmic bytes with 256-thread CTAs (PCG_TRAFFIC_RATIO; 1.093 with
        # 512-thread CTAs); traffic grows with the work, so the ratio scales it to this launch
        if args.precision == "fp32":
            roof["traffic"] = PCG_TRAFFIC_RATIO * pcg_b
        roof["assembly_launch"] = {"achieved": asm_b / (asm_ms / 1e3) / 1e9, "frac": asm_b / (asm_ms / 1e3) / 1e9 / peak,
                                   "algorithmic_bytes_per_launch": asm_b, "launch_ms": asm_ms}
        split = b3g.batch_assembly_split(ctx)
        if split["elem_mid"]:
            # group 2's element launch runs beside group 1's row launch: four launches, no single
            # element / row boundary to time
            roof["assembly_launch"]["split"] = {
                "group2_first_element": split["elem_mid"], "group2_first_slice": split["slice_mid"],
                "group2_element_ctas_per_sm": split["element_ctas_per_sm"],
                "group1_row_ctas_per_sm": split["row_ctas_per_sm"]}
        else:
            roof["assembly_launch"]["element_launch_ms"] = lt["elements_ms"] / lt["steps"]
            roof["assembly_launch"]["row_launch_ms"] = (lt["assembly_ms"] - lt["elements_ms"]) / lt["steps"]
    roof["whole_step"] = step_roof
    sched = b3g.batch_schedule(ctx) if not per_op else None

    extras = {}
    if not args.no_extras and rank == 0 and not single:
        # e2e through the C ABI with pinned host buffers: H2D external forces, step, D2H x and v
        f_h = torch.zeros(3 * nverts, dtype=torch.float32).pin_memory()
        x_h = torch.empty(3 * nverts, dtype=torch.float32).pin_memory()
        v_h = torch.empty(3 * nverts, dtype=torch.float32).pin_memory()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def e2e_step():
            # inputs up on the context's upload stream (the copy for step k overlaps step k - 1),
            # the step, then the results read back on its second stream: the copy of step k
            # overlaps step k + 1 (the host arrays of step k are complete when the next read is
            # queued; every copy is complete when the timed region ends)
            b3g.batch_apply_forces(ctx, bodies, f_h.data_ptr())
            step_once()
            b3g.batch_get_state_async(ctx, bodies, x_h.data_ptr(), v_h.data_ptr())

        # warm-up like the device-timed steps (the first transfer call sizes its staging buffer),
        # then the timed steps from the same state as the device-timed ones
        restore(start_state)
        for _ in range(max(args.warmup, 3)):
            e2e_step()
        b3g.batch_wait_state(ctx)
        restore(start_state)
        torch.cuda.synchronize(local)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        b3g.batch_wait_state(ctx)  # the context stream now waits for the last copy
        e1.record(stream)
        torch.cuda.synchronize(local)
        e2e_ms = e0.elapsed_time(e1)
        # the host arrays hold the last step's state
        x_chk = np.zeros((infos[0]["vertices"], 3), np.float32)
        x_chk[:] = bodies[0].state()[0]
        e2e_ok = bool(np.array_equal(x_h[:3 * infos[0]["vertices"]].numpy().reshape(-1, 3), x_chk))
        extras["e2e"] = {"value": nverts * args.steps / (e2e_ms / 1e3), "unit": "vertex-steps/s",
                         "h2d_bytes_per_step": 12 * nverts, "d2h_bytes_per_step": 24 * nverts,
                         "upload": "upload stream, overlapping the step before",
                         "read_back": "second stream, overlapping the next step", "host_arrays_match": e2e_ok}
        # plain one-body-at-a-time GPU path (per-op kernels) on a size-stratified sample
        sample = sorted(range(len(bodies)), key=lambda k: -infos[k]["vertices"])[::16] if len(bodies) > 16 else list(
            range(len(bodies)))
        for k in sample[:2]:
            bodies[k].step(dt, scfg, stats=False)
        ctx.synchronize()
        p0 = time.perf_counter()
        for k in sample:
            bodies[k].step(dt, scfg, stats=False)
        ctx.synchronize()
        plain_s = time.perf_counter() - p0
        plain_vs = sum(infos[k]["vertices"] for k in sample) / plain_s
        extras["plain"] = {"value": plain_vs, "unit": "vertex-steps/s", "bodies": len(sample),
                           "batched_over_plain": value / plain_vs}
        # solver outcome of the last timed-region step of every body
        last = [b.stats() for b in bodies]
        # CPU baseline: the oracle restatement on this host's cores, every body of the workload,
        # PARITY_STEPS steps from the initial state (FP32, as the reference's float build)
        threads = os.cpu_count() or 1
        cvs, csec, c_its, c_xs, c_vs = run_cpu(descs, PARITY_STEPS, dt, mx, threads)
        extras["cpu_baseline"] = {"value": cvs, "unit": "vertex-steps/s", "cores": threads, "kind": "port",
                                  "sample": f"all {len(descs)} bodies ({nverts} vertices), {PARITY_STEPS} steps from "
                                            f"the initial state, oracle C restatement FP32, {csec:.2f} s"}
        # parity: the GPU batch (the timed kernels, through the graph) from the same initial
        # state against the FP32 restatement on every body and the FP64 restatement on a
        # size-stratified sample
        for b, d, i in zip(bodies, descs, infos):
            b.set_state(d.x, d.v)
            if i["tets"]:
                q = np.zeros((i["tets"], 4), np.float32)
                q[:, 3] = 1.0
                b.set_rotations(q)
        ctx.synchronize()
        pst = b3g.step_batch(ctx, bodies, dt, PARITY_STEPS, scfg, stats=True)
        g_state = [b.state() for b in bodies]
        e32 = [rel_errors(x, v, c_xs[k], c_vs[k], descs[k].x) for k, (x, v) in enumerate(g_state)]
        pick = stratified(len(descs), [d.n for d in descs], 8)
        _, _, p_its, p_xs, p_vs = run_cpu([descs[k] for k in pick], PARITY_STEPS, dt, mx, threads, bits=64)
        e64 = [rel_errors(*g_state[k], p_xs[j], p_vs[j], descs[k].x) for j, k in enumerate(pick)]
        extras["parity"] = {
            "oracle": f"FP64 restatement of the reference step, {len(pick)} of {len(descs)} bodies (every 8th by "
                      f"size), {PARITY_STEPS} steps from the initial state through the timed batch kernels",
            "rel_x_max": max(e[0] for e in e64), "rel_v_max": max(e[1] for e in e64),
            "iters_diff_max": int(max(abs(int(pst[k]["pcg_iterations"]) - int(p_its[j][-1]))
                                      for j, k in enumerate(pick))),
            "vs_fp32_all_bodies": {"rel_x_max": max(e[0] for e in e32), "rel_v_max": max(e[1] for e in e32),
                                   "iters_diff_max": int(max(abs(int(pst[k]["pcg_iterations"]) - int(c_its[k][-1]))
                                                             for k in range(len(descs))))},
            "x_error": "|x - x_oracle| / |x_oracle - x0| per body", "v_error": "|v - v_oracle| / |v_oracle| per body",
            "bodies_max_iterations": sum(1 for s in last if s["solve_status"] != "converged"),
            "residual_ratio_max": max(float(s["residual_ratio"]) for s in last),
            "solver_outcome": "last timed step of every body: solves not converged, largest sqrt(delta/delta0)"}

    # persistent path: two launches per step (elements + assembly, then PCG + final update), plus
    # a 16-byte memset of the work counters that is not a kernel. Per-op path per step: begin,
    # one element kernel per element kind, assembly, then per PCG iteration the fused
    # direction/SpMV/dot kernel and the update kernel (launched in chunks of 8 iterations between
    # convergence checks), the true-residual refresh when due, and the final update; in bf16 mode
    # the outer iterations of the flexible CG instead (counted below).
    if per_op:
        i0 = infos[0]
        per_step = 1 + (1 if i0["tets"] else 0) + (1 if i0["tris"] else 0) + (1 if i0["springs"] else 0) + 1 + 1
        launches = per_step * args.steps
        refresh = scfg.refresh_period
        for it in iters:  # total over the timed steps; every step of a run takes about the same
            per = int(it) / max(args.steps, 1)
            if args.precision == "bf16":
                # per outer iteration: inner begin (2), 2 per inner iteration, z.q_prev (not on the
                # first), direction / product, update, refresh check
                outer = int(round(per))
                launches += args.steps * (outer * (2 + 2 * bf16_inner() + 4) - 1)
                continue
            launched = min(-(-int(round(per)) // 8) * 8, mx)
            resid = sum(1 for j in range(launched) if refresh > 0 and j % refresh == 0)
            launches += args.steps * (2 * launched + resid)
        roof["kernel"] = "per-op step: k_dir_spmv_dot (70 % of the kernel time) + k_update + refresh"
    else:
        # single Newton iteration: the flat element launch, the flat row launch and the PCG
        # launch; several: one whole-step launch
        if scfg.force_iterations > 1:
            launches = args.steps
        else:
            has_elements = any(i["tets"] or i["tris"] or i["springs"] for i in infos)
            # the split assembly launches elements and rows twice each (two body groups)
            per_step = (3 if has_elements else 2) + (2 if b3g.batch_assembly_split(ctx)["elem_mid"] else 0)
            launches = per_step * args.steps
    line = {"metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "strong" if args.split else "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "fp64": "f64", "bf16": "bf16+f32"}[args.precision],
            "data": "synthetic (seeded meshes)",
            "config": dict(cfg, vertices=nverts, l2="inputs larger than L2 (no flush needed)",
                           precision=args.precision, setup_s=round(setup_s, 2)),
            "p50_step_ms": statistics.median(step_ms), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "roofline": roof, "clocks": clk, "gpu_launches": launches}
    if world > 1:
        line["ranks"] = rank_stats
    if sched:
        line["schedule"] = {k: sched[k] for k in ("cluster", "threshold", "cluster_bodies", "ctas", "autotuned", "order")}
        line["schedule"]["candidates_timed"] = len(sched["candidates_ms"])
        # the chosen schedule per size bucket: which team steps the bucket's bodies
        edges = [0, 1024, 2048, 4096, 8192, 16384, 32768, 1 << 31]
        iters_all = [b.stats()["pcg_iterations"] for b in bodies] if not per_op else []
        buckets = []
        for lo, hi in zip(edges[:-1], edges[1:]):
            ks = [k for k, i in enumerate(infos) if lo <= i["vertices"] < hi]
            if not ks:
                continue
            clustered = sched["threshold"] >= 0 and sched["cluster"] > 1 and lo >= sched["threshold"]
            buckets.append({"vertices": f"[{lo},{hi})" if hi < (1 << 31) else f"[{lo},)", "bodies": len(ks),
                            "team": f"cluster of {sched['cluster']} CTAs" if clustered else "one CTA",
                            "mean_pcg_iterations": float(np.mean([iters_all[k] for k in ks])) if iters_all else None})
        line["schedule"]["buckets"] = buckets
    line.update(extras)
    for b in bodies:
        b.close()
    ctx.close()
    return line if rank == 0 else None


# ------------------------------------------------------------------ serving
def serve_arm(args, rank, local):
    """Continuous-batching server under a Poisson request stream; the same stream through the
    plain one-body-at-a-time path on a bounded sample. Returns the line (rank 0)."""
    from bounce_softbody_gb300 import b3g, meshes

    pool = meshes.serving_bodies(args.serve_pool, seed=5 + 1000 * rank)
    scfg = b3g.solver_config(max_pcg_iterations=PCG_MAX, pcg_tolerance=PCG_TOL)
    rng = np.random.default_rng(7 + 1000 * rank)
    gaps = rng.exponential(1.0 / args.serve_rate, size=int(args.serve_rate * args.serve_seconds * 1.5) + 16)
    arrival = np.cumsum(gaps)
    arrival = arrival[arrival < args.serve_seconds]
    req_body = rng.integers(0, len(pool), size=arrival.size)
    req_steps = rng.integers(1, 31, size=arrival.size)
    demand = float(sum(pool[b].n * s for b, s in zip(req_body, req_steps))) / args.serve_seconds

    ctx = b3g.Context(local)
    srv = b3g.Server(ctx, int(args.serve_budget_gb * (1 << 30)), args.serve_max_active, DT, scfg)
    for d in pool:
        srv.add_body(d)
    srv.start()
    t0 = time.perf_counter()
    for k in range(len(pool)):  # warm-up: every body created on the device and stepped once
        srv.submit(k, 1)
    srv.drain(timeout=1800)
    setup_s = time.perf_counter() - t0
    srv.reset_stats()

    clocks = Clocks(local)
    results = []
    t0 = time.perf_counter()
    i = 0
    while i < arrival.size:
        now = time.perf_counter() - t0
        while i < arrival.size and arrival[i] <= now:
            srv.submit(int(req_body[i]), int(req_steps[i]))
            i += 1
        results += srv.poll()
        time.sleep(0.0002)
    end = t0 + args.serve_seconds + args.serve_grace
    while time.perf_counter() < end and srv.pending() > 0:
        results += srv.poll()
        time.sleep(0.001)
    results += srv.poll()
    st = srv.stats()
    queued = srv.pending()
    clk = clocks.stop()
    srv.close()

    done = [r for r in results if r["status"] == "done"]
    lat = np.array([r["latency_seconds"] for r in done]) * 1e3
    per_step = np.array([r["latency_seconds"] / r["steps"] for r in done]) * 1e3
    value = st["vertex_steps"] / st["wall_seconds"] if st["wall_seconds"] > 0 else 0.0

    # plain path: the same stream, one request after another, one body step per call
    plain = {}
    if args.serve_plain_seconds > 0:
        cache = {}
        order = list(range(arrival.size))
        for k in order[:64]:  # create the sample's bodies outside the timed region
            b = int(req_body[k])
            if b not in cache:
                cache[b] = b3g.Body(ctx, pool[b])
        step_ms, vsteps = [], 0
        p0 = time.perf_counter()
        for k in order[:64]:
            body = cache[int(req_body[k])]
            for _ in range(int(req_steps[k])):
                s0 = time.perf_counter()
                body.step(DT, scfg, stats=True)  # waits for the step
                step_ms.append(1e3 * (time.perf_counter() - s0))
                vsteps += body.n
            if time.perf_counter() - p0 > args.serve_plain_seconds:
                break
        psec = time.perf_counter() - p0
        plain = {"value": vsteps / psec, "unit": "vertex-steps/s", "requests": k + 1,
                 "p50_step_ms": float(np.median(step_ms)), "p99_step_ms": float(np.percentile(step_ms, 99)),
                 "note": "same request stream served one request after another by b3g_body_step"}
        for b in cache.values():
            b.close()
    ctx.close()

    line = {"metric": "serving: vertex-steps/s and p50/p99 step latency under Poisson arrivals", "value": value,
            "unit": "vertex-steps/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded meshes and arrivals)",
            "config": {"workload": f"Poisson arrivals {args.serve_rate:g} req/s for {args.serve_seconds:g} s over "
                                   f"{len(pool)} bodies (tet 1e3..1e5 vertices log-uniform / cloth 32^2..256^2), "
                                   f"1..30 steps per request, h=1/60",
                       "pool_vertices": int(sum(d.n for d in pool)), "max_active": args.serve_max_active,
                       "budget_gb": args.serve_budget_gb, "pcg_tol": PCG_TOL, "pcg_max_iter": PCG_MAX,
                       "team": f"clusters of {st['cluster_ctas']} CTAs from {st['cluster_threshold']} vertices",
                       "setup_s": round(setup_s, 1)},
            "demand_vertex_steps_per_s": demand,
            "requests": {"submitted": int(arrival.size), "completed": len(done), "queued_at_end": queued,
                         "rejected": int(st["rejected"]), "evictions": int(st["evictions"])},
            "request_latency_ms": {"p50": float(np.median(lat)) if lat.size else None,
                                   "p99": float(np.percentile(lat, 99)) if lat.size else None},
            "request_latency_per_step_ms": {"p50": float(np.median(per_step)) if per_step.size else None,
                                            "p99": float(np.percentile(per_step, 99)) if per_step.size else None},
            "p50_step_ms": st["step_ms_p50"], "p99_step_ms": st["step_ms_p99"],
            "launches": int(st["iterations"]), "gpu_busy_frac": st["gpu_seconds"] / st["wall_seconds"] if st["wall_seconds"] else None,
            "clocks": clk, "gpu_launches": int(st["iterations"]), "plain": plain}
    return line if rank == 0 else None


SERVING_KEYS = ["config", "demand_vertex_steps_per_s", "requests", "request_latency_ms", "request_latency_per_step_ms",
                "p50_step_ms", "p99_step_ms", "launches", "gpu_busy_frac", "clocks", "plain"]


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    rc = 0
    if args.impl == "ours" and args.workload == "serve":
        line = serve_arm(args, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
    elif args.impl == "reference":
        rc = reference_arm(args, world, rank, pg)
    else:
        line = ours(args, world, rank, local, pg)
        if line is not None and args.workload == "batch" and world == 1 and not args.no_serve and not args.no_extras:
            # the serving workload (continuous batching under Poisson arrivals) on the same GPU,
            # after the batch's bodies are released
            srv = serve_arm(args, rank, local)
            line["serving"] = {"metric": srv["metric"], "value": srv["value"], "unit": srv["unit"],
                               **{k: srv[k] for k in SERVING_KEYS}}
        if line is not None:
            print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
