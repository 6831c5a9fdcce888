"""Benchmark of the guiding step (one JSON line on rank 0).

Workload ("full guiding step", hash-grid network): each step is
  * one guided query pass over a 1920x1080 wavefront (2,073,600 queries:
    featurise -> hash-grid/SH/one-blob encode -> 80-64-64-64-48 MLP -> 8-lobe
    vMF mixture with cosine lobe -> sample + pdf), and
  * one training step on 2^18 records (forward, KL loss + adjoint, backward
    through MLP and grid, Adam + EMA over 12.6 M parameters).
Inputs are seeded synthetic data with the shapes and distributions of that
workload (neural-mixture-guiding_gb300/synth.py), resident in HBM.

value = guided queries/s of the measured path (default: fused BF16 on
tcgen05) over whole steps: a step's 2,073,600 queries over the time of its
query pass plus its training step (train_samples_per_s likewise counts the
step's 2^18 samples over that time); query_pass and train_step give each
phase's own rate, and plain_fp32 the plain FP32 path's numbers from the same
run. L2 is flushed (a 256 MiB write, then a
256 MiB read) before every timed step; each step is timed with CUDA events
on the launching stream, excluding the flush.

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement of the reference's guiding step (oracle/), OpenMP over
all host threads, on a bounded sample of the same workload.
"""
import argparse
import ctypes
import importlib
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "neural-mixture-guiding_gb300"

N_QUERIES = 1920 * 1080
N_TRAIN = 1 << 18
FLOP_PER_QUERY = 2 * (80 * 64 + 64 * 64 + 64 * 64 + 64 * 48)  # 32,768 executed (padded) MLP FLOP
BYTES_PER_QUERY = 12 + 12 + 12 + 4 + 16 + 12 + 4 + 4 + 4      # pos, wo, n, rough, u4 in; dir, pdf, lobe, sel out
# dram__bytes_read.sum + dram__bytes_write.sum of one k_fused_query_ws launch over the same
# 2,073,600-query wavefront (ncu capture summarised in profiles/k_fused_query_ws_hashgrid_2073600.md)
TRAFFIC_QUERY_BYTES = 141_316_608 + 35_742_464
# l1tex__m_xbar2l1tex_read_bytes.sum of the same capture: the hash-grid corner gathers reaching L2
# (the 24 MB table stays in L2), in 32-byte sectors; about one sector request per cycle per SM is
# the ceiling a gather-only kernel of the same 128 corners per query reaches
L2_TO_L1_BYTES = 4.686e9


# The hash-grid network (NMG_PRESET_HASHGRID) as the oracle describes it; the CPU legs build it from this
# spec so that the reference arm never loads the product library (tests/test_bench_host.py checks that it
# equals the library's preset).
HASHGRID_NET = dict(input_mode=1, grid_hash=1, grid_levels=16, grid_feats=2, grid_log2_T=19, grid_base_res=16,
                    grid_scale=1.447, grid_smoothstep=0, sh_degree=4, oneblob_bins=4, width=64, n_hidden=3,
                    n_out=33)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "200 ms samples under the same load, from before the timed steps to after them"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return ws, rank


def barrier_max(x, ws):
    """Maximum of x over the ranks (the job's time is its slowest replica's)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank, base=7272):
    """Each replica draws its own synthetic wavefront and training batch."""
    return base + rank


def make_inputs(synth, torch, seed=7272):
    q = synth.wavefront(N_QUERIES, seed=seed)
    field = synth.TrainField(seed=seed)
    x, rec = synth.train_batch(field, N_TRAIN, seed=seed + 1, input_mode=1, selection=True)
    return q, x, rec


def run_ours(args):
    import numpy as np
    import torch

    nmg = importlib.import_module(PKG)
    synth = importlib.import_module(PKG + ".synth")
    ws, rank = dist_setup()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    q, x, rec = make_inputs(synth, torch, seed=replica_seed(rank))
    dq = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in q.items()}
    dx, drec = torch.from_numpy(x).cuda(), torch.from_numpy(rec).cuda()
    flush = L2Flush(torch)
    path = {"bf16": nmg.PATH_BF16, "fp16": nmg.PATH_FP16, "fp32": nmg.PATH_FP32}[args.path]

    def measure(path_id, steps, warmup, clocks=None):
        """Times `steps` steps of a freshly created field after `warmup` steps. Every step trains on a
        fresh batch of records drawn on the GPU from the ground-truth field (as a renderer records new
        paths each frame), drawn before the step's first event. The clock sampler's warm-up load runs on
        a separate field, so the timed steps are the field's first steps after its warm-up (gradient norm
        reported per step), not steps of a network that hundreds of load steps at the configured learning
        rate drove into the exp clamp."""
        cfg = nmg.config(nmg.PRESET_HASHGRID, path=path_id, n_lobes=args.lobes)
        f = nmg.GuidingField(cfg, max_queries=N_QUERIES, max_batch=N_TRAIN)
        if args.tiling and path_id != nmg.PATH_FP32:
            f.set_query_tiling(args.tiling)
        src = synth.TorchTrainSource(synth.TrainField(seed=replica_seed(rank)), seed=replica_seed(rank) + 3)
        out = {"dir": torch.empty((N_QUERIES, 3), device="cuda"), "pdf": torch.empty(N_QUERIES, device="cuda"),
               "lobe": torch.empty(N_QUERIES, device="cuda", dtype=torch.int32),
               "selection": torch.empty(N_QUERIES, device="cuda")}
        stats = torch.zeros((max(steps, 1), 2), device="cuda", dtype=torch.float64)
        st = torch.cuda.current_stream()
        ev = [(torch.cuda.Event(True), torch.cuda.Event(True), torch.cuda.Event(True)) for _ in range(steps)]
        for _ in range(warmup):
            bx, brec = src(N_TRAIN, selection=True)
            f.query(dq["pos"], dq["wo"], dq["normal"], dq["rough"], dq["u4"], outputs=out)
            f.train_step(bx, brec, stats=stats[0])
        torch.cuda.synchronize()

        if clocks:
            # clock samples bracket the timed steps: at least two readings under the same load before
            # them and two after (the timed region itself is shorter than the sampling interval); the
            # load runs on a field of its own
            fl = nmg.GuidingField(cfg, max_queries=N_QUERIES, max_batch=N_TRAIN)

            def untimed_until(n_samples, limit_s):
                t_end = time.perf_counter() + limit_s
                while len(clocks.lines) < n_samples and time.perf_counter() < t_end:
                    for _ in range(20):
                        fl.query(dq["pos"], dq["wo"], dq["normal"], dq["rough"], dq["u4"], outputs=out)
                        fl.train_step(dx, drec)
                    torch.cuda.synchronize()

            clocks.start()
            untimed_until(2, 10.0)
            before = len(clocks.lines)
        batches = [None] * steps
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for i in range(steps):
            batches[i] = src(N_TRAIN, selection=True)  # drawn outside the step's events
            flush(i)
            a, b, c = ev[i]
            a.record(st)
            f.query(dq["pos"], dq["wo"], dq["normal"], dq["rough"], dq["u4"], outputs=out)
            b.record(st)
            f.train_step(batches[i][0], batches[i][1], stats=stats[i])
            c.record(st)
            batches[i] = None
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if ws > 1:
            torch.distributed.barrier()
        if clocks:
            untimed_until(before + 2, 5.0)
            fl.close()
        cl = clocks.stop() if clocks else None
        tq = sum(a.elapsed_time(b) for a, b, _ in ev) / 1e3
        tt = sum(b.elapsed_time(c) for _, b, c in ev) / 1e3
        st_np = stats.cpu().numpy()
        t_steps = [b.elapsed_time(c) for _, b, c in ev]
        gn = st_np[:steps, 1]
        healthy = gn >= 1e-3 * gn[0]
        health = {"grad_norm_first": float(st_np[0, 1]), "grad_norm_last": float(st_np[steps - 1, 1]),
                  "mean_loss_first": float(st_np[0, 0]), "mean_loss_last": float(st_np[steps - 1, 0]),
                  "steps_before_first_timed": warmup, "grad_norm_per_step": [float(v) for v in gn],
                  "train_ms_per_step": [float(v) for v in t_steps],
                  # the step's work does not depend on the gradient's size: compare the steps whose gradient
                  # norm is still within 1e-3 of the first timed step's with the rest
                  "train_ms_healthy_steps": float(np.mean([t for t, h in zip(t_steps, healthy) if h])),
                  "train_ms_other_steps": float(np.mean([t for t, h in zip(t_steps, healthy) if not h]))
                  if not healthy.all() else None}
        # Adam at the configured learning rate (1e-2, common/configs/nn/base.json) drives the kappa logits
        # into the exp clamp within a few steps on this field, in every path alike (the plain FP32 line
        # runs the same steps); the per-step times above show the step's cost does not depend on it
        health["grad_norm_below_1e-6_of_first"] = bool(health["grad_norm_last"] < 1e-6 * health["grad_norm_first"])
        if not np.all(np.isfinite(st_np[:steps])):
            raise RuntimeError("non-finite loss or gradient norm during the timed steps: %r" % health)
        f.L.nmg_check_errors.argtypes = [ctypes.c_void_p]
        nmg.check(f.L.nmg_check_errors(f.h))
        res = {"t_query": barrier_max(tq, ws), "t_train": barrier_max(tt, ws), "wall": wall, "clocks": cl,
               "loss": st_np[steps - 1].tolist(), "health": health, "field": f, "out": out}
        return res

    if args.mixture_only:
        # the mixture-only kernels' row alone, for profiling
        if rank == 0:
            print(json.dumps({"mixture_only": True, "mixture_kernels": mixture_kernels(nmg, synth, torch, flush,
                                                                                     peaks()[0])}), flush=True)
        return
    if args.steps_only:
        # the guiding step alone, for profiling: `warmup` + `steps` steps of a fresh field (no clock
        # sampler, no other measurements); the line carries only the step times
        ours = measure(path, args.steps, args.warmup)
        ours["field"].close()
        if rank == 0:
            print(json.dumps({"steps_only": True, "steps": args.steps, "warmup": args.warmup,
                              "query_ms": ours["t_query"] * 1e3 / args.steps,
                              "train_ms": ours["t_train"] * 1e3 / args.steps}), flush=True)
        return
    ours = measure(path, args.steps, args.warmup, Clocks())
    # the plain FP32 path over the same steps after the same warm-up: its health record is comparable
    plain = measure(nmg.PATH_FP32, args.steps, args.warmup) if path != nmg.PATH_FP32 else ours
    frame = frame_graph(nmg, synth, torch, np, dx, drec, path) if path != nmg.PATH_FP32 and not args.no_frame else None
    mix = mixture_kernels(nmg, synth, torch, flush, peaks()[0])
    nxt = next_rows(nmg, torch, ours["field"], dq, ours["out"]["dir"], flush) if path != nmg.PATH_FP32 else None

    # end to end through the public API on host buffers (nmg_query_host / nmg_train_step_host): pinned host
    # inputs in, host results out, every step; the library pipelines the copies with the kernels
    f = ours["field"]
    hq = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in q.items()}
    hx, hrec = torch.from_numpy(x).pin_memory(), torch.from_numpy(rec).pin_memory()
    # the query's results an integrator consumes: direction, pdf and (learned selection) the selection
    # probability; the lobe index is diagnostic and stays on the device
    hout = {"dir": torch.empty((N_QUERIES, 3)).pin_memory(), "pdf": torch.empty(N_QUERIES).pin_memory(),
            "selection": torch.empty(N_QUERIES).pin_memory()}
    hstats = torch.empty(2, dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * t.element_size() for k, t in hq.items() if k != "aabb") + hx.numel() * 4 + hrec.numel() * 4
    d2h = sum(t.numel() * t.element_size() for t in hout.values()) + hstats.numel() * 8

    def e2e_step():
        f.query_host(hq["pos"], hq["wo"], hq["normal"], hq["rough"], hq["u4"], hout)
        f.train_step_host(hx, hrec, stats=hstats)

    e2e_step()  # first call allocates the device staging
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
    # back-to-back steps from an idle GPU, as a renderer issues them frame after frame: the first
    # step's input copy is exposed, the later ones run under the previous step's kernels
    e2e_steps = max(20, args.steps)
    e0.record()
    for _ in range(e2e_steps):
        e2e_step()
    e1.record()
    torch.cuda.synchronize()
    t_e2e = barrier_max(e0.elapsed_time(e1) / 1e3, ws)
    e2e_loss = float(hstats[0])

    # kernel-only timing of the fused query kernel (dominant kernel) on its own stream
    st = torch.cuda.current_stream()
    kk = []
    for i in range(5):
        flush(i)
        a, b = torch.cuda.Event(True), torch.cuda.Event(True)
        a.record(st)
        f.query(dq["pos"], dq["wo"], dq["normal"], dq["rough"], dq["u4"], outputs=ours["out"])
        b.record(st)
        kk.append((a, b))
    torch.cuda.synchronize()
    t_kernel = sorted(a.elapsed_time(b) for a, b in kk)[2] / 1e3

    if rank != 0:
        return
    hbm, bf16, src = peaks()
    steps = args.steps
    # a step is one query pass over the wavefront plus one training step: the step rates count the
    # queries and samples of a step over both phases' time; the phase rates over their own phase
    t_step = ours["t_query"] + ours["t_train"]
    step_qps, step_tps = ws * N_QUERIES * steps / t_step, ws * N_TRAIN * steps / t_step
    qps = ws * N_QUERIES * steps / ours["t_query"]
    tps = ws * N_TRAIN * steps / ours["t_train"]
    p_steps = steps  # the plain path runs the same steps as the measured one
    plain_qps = N_QUERIES * p_steps / plain["t_query"]
    plain_tps = N_TRAIN * p_steps / plain["t_train"]
    plain_step_qps = N_QUERIES * p_steps / (plain["t_query"] + plain["t_train"])
    tflops = FLOP_PER_QUERY * N_QUERIES / t_kernel / 1e12
    gbs = BYTES_PER_QUERY * N_QUERIES / t_kernel / 1e9
    cpu = cpu_baseline(q, x, rec, seconds=args.cpu_seconds) if not args.no_cpu else None
    line = {
        "metric": "guided queries/s & train samples/s, BF16 fused vs FP32 plain, 1 GB300",
        "value": step_qps,
        "unit": "queries/s",
        "n_gpus": ws,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": t_step / steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"bf16": "bf16", "fp16": "fp16", "fp32": "f32"}[args.path],
        "data": "synthetic (seeded wavefront + ground-truth radiance field; no scene data)",
        "config": {"workload": "full guiding step: 2,073,600-query wavefront (1920x1080) + 2^18-sample train step",
                   "network": "hash grid 16x2 (2^19/level, base 16, x1.447) + SH4(wo) + SH4(n) + OneBlob4(r) "
                              "-> 80-64-64-64-48 MLP, K=8 lobes + selection",
                   "path": args.path, "l2": "flushed before each timed step (256 MiB write, then a 256 MiB read that writes the dirty lines back outside the timed region)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "train_samples_per_s": step_tps,
        "rates": "value and train_samples_per_s: a step's 2,073,600 queries and 2^18 training samples over the "
                 "step's time (query pass + training step); query_pass / train_step: each over its own phase",
        "query_pass": {"queries_per_s": qps, "ms": ours["t_query"] / steps * 1e3},
        "train_step": {"samples_per_s": tps, "ms": ours["t_train"] / steps * 1e3},
        "query_ms": ours["t_query"] / steps * 1e3,
        "train_ms": ours["t_train"] / steps * 1e3,
        "plain_fp32": {"step_queries_per_s": plain_step_qps, "query_pass_queries_per_s": plain_qps,
                       "train_step_samples_per_s": plain_tps,
                       "query_ms": plain["t_query"] / p_steps * 1e3, "train_ms": plain["t_train"] / p_steps * 1e3,
                       "final_stats": {"mean_loss": plain["loss"][0], "grad_norm": plain["loss"][1]},
                       "train_health": plain["health"]},
        "speedup_vs_plain_fp32": {"step": step_qps / ws / plain_step_qps, "queries": qps / ws / plain_qps,
                                  "train": tps / ws / plain_tps},
        "final_stats": {"mean_loss": ours["loss"][0], "grad_norm": ours["loss"][1]},
        "train_health": ours["health"],
        "e2e": {"value": ws * N_QUERIES * e2e_steps / t_e2e, "unit": "queries/s",
                "what": "query pass + training step per step, host buffers in and out",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "api": "nmg_query_host + nmg_train_step_host (pinned host memory; inputs copied in, results "
                       "written by the kernels through the host mapping)", "final_loss": e2e_loss},
        "gpu_launches": None,
        "roofline": {"kernel": "k_fused_query_ws" if path != nmg.PATH_FP32 else "plain query kernels",
                     "bound": "tensor", "achieved": tflops, "peak": bf16, "unit": "TFLOP/s",
                     "frac": tflops / bf16, "peak_source": src,
                     "traffic": TRAFFIC_QUERY_BYTES if path == nmg.PATH_BF16 else None,
                     "traffic_unit": "bytes per launch (ncu)",
                     "limiter": "hash-grid gathers: ~70 L2 sector requests per query, L1->L2 request path 74% busy "
                                "(ncu), not HBM or the tensor pipe",
                     "hbm_achieved_gbs": gbs, "hbm_frac": gbs / hbm,
                     "l2_sector_requests": l2_request_roofline(t_kernel, ours["clocks"]),
                     "per_unit": {"flop_per_query": FLOP_PER_QUERY, "hbm_bytes_per_query": BYTES_PER_QUERY},
                     "kernel_ms": t_kernel * 1e3},
        "cpu_baseline": cpu,
        "clocks": ours["clocks"],
        "frame_graph": frame,
        "mixture_kernels": mix,
        "next_rows": nxt,
    }
    line["gpu_launches"] = launches_per_step(path) * steps
    print(json.dumps(line), flush=True)


BOUNCE_SIZES = [2_073_600, 1_400_000, 900_000, 550_000, 300_000, 150_000, 70_000]


def frame_graph(nmg, synth, torch, np, dx, drec, path, lobes=(8, 16), frames=5, warmup=3):
    """The uneven 7-bounce frame (queues of 2,073,600 ... 70,000 queries, each followed by a 2^18-record
    training step) captured once as a CUDA graph and replayed; the same frame issued launch by launch is
    timed beside it. Inputs of a frame (5.4 M queries, 0.44 GB) exceed L2, so no flush is needed."""
    qs = []
    for i, n in enumerate(BOUNCE_SIZES):
        q = synth.wavefront(n, seed=7272 + 100 + i)
        qs.append({k: torch.from_numpy(np.ascontiguousarray(q[k])).cuda() for k in ("pos", "wo", "normal", "rough", "u4")})
    res = {"bounce_queries": BOUNCE_SIZES, "train_batch": int(dx.shape[0]),
           "l2": "not flushed: a frame's inputs (0.44 GB) exceed L2"}
    st = torch.cuda.current_stream()
    for K in lobes:
        f = nmg.GuidingField(nmg.config(nmg.PRESET_HASHGRID, path=path, n_lobes=K), max_queries=BOUNCE_SIZES[0],
                             max_batch=int(dx.shape[0]))
        outs, bounces = [], []
        for q in qs:
            n = q["pos"].shape[0]
            o = {"dir": torch.empty((n, 3), device="cuda"), "pdf": torch.empty(n, device="cuda"),
                 "lobe": torch.empty(n, device="cuda", dtype=torch.int32), "selection": torch.empty(n, device="cuda")}
            outs.append(o)
            bounces.append(nmg.GuidingField.bounce(q["pos"], q["wo"], q["normal"], q["rough"], q["u4"], o,
                                                   count=torch.tensor([n], device="cuda", dtype=torch.int32),
                                                   train=(dx, drec, None, None)))
        tiling = f.autotune(qs[0]["pos"], qs[0]["wo"], qs[0]["normal"], qs[0]["rough"], qs[0]["u4"])
        fr = f.capture_frame(bounces)

        def timed(run):
            for _ in range(warmup):
                run()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(True), torch.cuda.Event(True)
            a.record(st)
            for _ in range(frames):
                run()
            b.record(st)
            torch.cuda.synchronize()
            return a.elapsed_time(b) / 1e3 / frames

        t_graph = timed(fr.launch)
        t_eager = timed(lambda: f.run_frame_eager(bounces))
        f.check_errors()
        res["K%d" % K] = {"ms_per_frame_graph": t_graph * 1e3, "ms_per_frame_eager": t_eager * 1e3,
                          "queries_per_s": sum(BOUNCE_SIZES) / t_graph,
                          "train_samples_per_s": len(BOUNCE_SIZES) * int(dx.shape[0]) / t_graph,
                          "graph_nodes": fr.nodes, "query_tiling_warpgroups": tiling}
        fr.close()
        f.close()
    return res


def l2_request_roofline(t_kernel, clocks, sms=152):
    """The query kernel's real limiter: L2 -> L1 sector requests per SM and cycle (ncu byte count of
    one launch / 32 B, over the CUDA-event kernel time at the SM clock sampled in the timed region)
    against the ~1 request / cycle / SM ceiling of a gather-only kernel."""
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    sectors = L2_TO_L1_BYTES / 32
    per_sm_clk = sectors / (t_kernel * sms * mhz * 1e6)
    return {"sectors_per_query": sectors / N_QUERIES, "achieved_per_sm_per_clk": per_sm_clk,
            "ceiling_per_sm_per_clk": 1.0, "frac": per_sm_clk, "source": "ncu byte count, live kernel time"}


class L2Flush:
    """Empties L2 between timed steps: writes a 256 MiB buffer (twice L2) and then reads another
    256 MiB one, so that L2 holds only clean lines of the read buffer when the timed region
    starts -- the flush's own dirty lines are written back before it, not inside it."""

    def __init__(self, torch):
        self.w = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.r = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")

    def __call__(self, i):
        self.w.fill_(i & 0xFF)
        self.r.sum()


def mixture_kernels(nmg, synth, torch, flush, hbm, n=1 << 21, K=8, reps=10):
    """The mixture-only workload (K = 8 raw outputs per query, no network) at a size whose traffic
    dwarfs L2, 2^21 queries: sample+pdf, pdf at given directions (the MIS pdf) and KL loss+gradient,
    CUDA events, L2 flushed. Algorithmic bytes per query: 164 (raw 128 + uniforms 16 in; direction 12,
    pdf 4, lobe 4 out), 144 (raw 128 + direction 12 in; pdf 4 out) and 280 (raw 128 + record 24 in;
    gradient 128 out)."""
    raw, u4, rec = synth.mixture_batch(n, K, seed=7272, selection=False)
    r, u, rc = (torch.from_numpy(a).cuda() for a in (raw, u4, rec))
    d = torch.empty((n, 3), device="cuda")
    p = torch.empty(n, device="cuda")
    p2 = torch.empty(n, device="cuda")
    lb = torch.empty(n, device="cuda", dtype=torch.int32)
    g = torch.empty_like(r)
    lib = nmg.lib()
    opts = nmg.mixture_opts(K, r.shape[1])
    ws_bytes = lib.nmg_mixture_loss_workspace_bytes(n)
    ws = torch.empty(max(ws_bytes, 16), dtype=torch.uint8, device="cuda")
    tot = torch.empty(1, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())

    def sample():
        nmg.check(lib.nmg_mixture_sample(ctypes.byref(opts), ptr(r), ptr(u), None, n, ptr(d), ptr(p), ptr(lb),
                                         ctypes.c_void_p(st.cuda_stream)))

    def pdf():  # at the directions sample() drew
        nmg.check(lib.nmg_mixture_pdf(ctypes.byref(opts), ptr(r), ptr(d), None, n, ptr(p2),
                                      ctypes.c_void_p(st.cuda_stream)))

    def loss():
        nmg.check(lib.nmg_mixture_loss_grad(ctypes.byref(opts), ptr(r), ptr(rc), rc.shape[1], n, ctypes.c_float(128.0),
                                            ptr(g), None, ptr(tot), ptr(ws), ctypes.c_size_t(ws_bytes),
                                            ctypes.c_void_p(st.cuda_stream)))

    out = {"queries": n, "K": K, "l2": "flushed before each timed launch (256 MiB write, then a 256 MiB read)"}
    for name, fn, per in (("sample_pdf", sample, 164), ("pdf", pdf, 144), ("loss_grad", loss, 280)):
        for _ in range(3):
            fn()
        ts = []
        for i in range(reps):
            flush(i)
            a, b = torch.cuda.Event(True), torch.cuda.Event(True)
            a.record(st)
            fn()
            b.record(st)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        t = sorted(ts)[reps // 2]
        gbs = per * n / t / 1e9
        out[name] = {"us": t * 1e6, "bytes_per_query": per, "achieved_gbs": gbs, "hbm_frac": gbs / hbm}
    return out


def next_rows(nmg, torch, f, dq, dirs, flush, reps=5, depth=6):
    """The calls built around the guiding step, timed through the C ABI with CUDA events (L2 flushed before
    each launch, median of `reps`):
      * the MIS pdf at given directions over the 1920x1080 wavefront (nmg_pdf: featurise, encode, MLP and
        the mixture pdf in one fused pass, no raw outputs through HBM);
      * training-record extraction from the per-pixel radiance records of a 1920x1080 frame with `depth`
        bounces per pixel, every pixel a training pixel (nmg_extract_records; the call also resets its
        4-byte append counter). Records: seeded uniform values, bounce counts uniform in 0..depth."""
    st = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(3):
            fn()
        ts = []
        for i in range(reps):
            flush(i)
            a, b = torch.cuda.Event(True), torch.cuda.Event(True)
            a.record(st)
            fn()
            b.record(st)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return sorted(ts)[reps // 2]

    t_pdf = timed(lambda: f.pdf(dq["pos"], dq["wo"], dq["normal"], dq["rough"], dirs))
    res = (1920, 1080)
    n = res[0] * res[1]
    g = torch.Generator(device="cuda").manual_seed(11)

    def u(*shape, lo=0.0, hi=1.0):
        return torch.rand(*shape, device="cuda", generator=g) * (hi - lo) + lo

    def angles():
        return torch.stack([u(n, hi=math.pi), u(n, hi=2 * math.pi)], 1).contiguous()

    recs = [{"L": u(n, 3), "thp": u(n, 3), "pos": u(n, 3), "dir": angles(), "wi_pdf": u(n, lo=0.01, hi=2.0),
             "bsdf_pdf": u(n, lo=0.01, hi=2.0), "mis_weight": u(n), "delta": (u(n) < 0.1).to(torch.uint8),
             "bsdf_val": u(n, 3), "wo": angles(), "normal": angles(), "roughness": u(n)} for _ in range(depth)]
    cur = torch.randint(0, depth + 1, (n,), device="cuda", dtype=torch.int32, generator=g)
    cap = n * depth
    outs = (torch.empty((cap, int(f.info.n_input)), device="cuda"),
            torch.empty((cap, int(f.info.record_floats)), device="cuda"),
            torch.zeros(1, dtype=torch.int32, device="cuda"))

    def extract():
        f.extract_records(recs, cur, (0, 0), (1, 1), res, res, cap, outputs=outs)

    t_ex = timed(extract)
    n_rec = int(outs[2].item())
    del outs
    row_frame = train_frame_row(nmg, torch, f.cfg, recs[:TF_DEPTH], cur.clamp(max=TF_DEPTH), res, timed)
    return {"mis_pdf": {"queries": N_QUERIES, "us": t_pdf * 1e6, "queries_per_s": N_QUERIES / t_pdf},
            "record_extraction": {"pixels": n, "bounces_per_pixel": depth, "records": n_rec, "us": t_ex * 1e6,
                                  "pixels_per_s": n / t_ex, "records_per_s": n_rec / t_ex},
            "train_frame": row_frame}


# trainStep's defaults (parameters.h:20-21, integrator.h:167-168): batch 65,536 x 8, minimum 65,536,
# 5 batches per frame, 3 training bounces
TF_BATCH, TF_MIN_BATCH, TF_BATCHES, TF_DEPTH = 524_288, 65_536, 5, 3


def train_frame_row(nmg, torch, cfg, recs, cur, res, timed):
    """One frame's training (the reference's trainStep, integrator.cpp:650-701) at its default batch plan on
    the 1920x1080 radiance records of `next_rows` cut to 3 bounces, two routes through the C ABI:
      * fused: nmg_train_frame -- vertex-id compaction, device-side batch plan, and the training kernel
        computing each record's input and GuidedOutput in its load stage;
      * reference-shaped: nmg_extract_records, the host reads the record count (trainStep synchronises
        and reads trainBuffer->size()), then one nmg_train_step per batch on the record matrix."""
    n = res[0] * res[1]
    cap = n * TF_DEPTH
    f = nmg.GuidingField(cfg, max_batch=TF_BATCH)
    ids = torch.zeros(cap, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    stats = torch.zeros((TF_BATCHES, 2), dtype=torch.float64, device="cuda")

    def fused():
        f.train_frame(recs, cur, (0, 0), (1, 1), res, res, cap, TF_BATCH, TF_BATCHES, TF_MIN_BATCH,
                      outputs=(ids, cnt, stats))

    t_fused = timed(fused)
    n_rec = int(cnt.item())
    plan = []
    for i in range(min(n_rec // TF_BATCH + 1, TF_BATCHES)):
        b = min(n_rec - i * TF_BATCH, TF_BATCH)
        b -= b % 128
        if b < TF_MIN_BATCH:
            break
        plan.append(b)
    del ids
    x = torch.empty((cap, int(f.info.n_input)), device="cuda")
    rec = torch.empty((cap, int(f.info.record_floats)), device="cuda")
    c2 = torch.zeros(1, dtype=torch.int32, device="cuda")

    def unfused():
        f.extract_records(recs, cur, (0, 0), (1, 1), res, res, cap, outputs=(x, rec, c2))
        m = int(c2.item())
        for i in range(min(m // TF_BATCH + 1, TF_BATCHES)):
            b = min(m - i * TF_BATCH, TF_BATCH)
            b -= b % 128
            if b < TF_MIN_BATCH:
                break
            f.train_step(x[i * TF_BATCH:i * TF_BATCH + b], rec[i * TF_BATCH:i * TF_BATCH + b])

    t_unfused = timed(unfused)
    f.check_errors()
    f.close()
    trained = sum(plan)
    return {"pixels": n, "bounces_per_pixel": TF_DEPTH, "records": n_rec, "batch": TF_BATCH,
            "batches": len(plan), "records_trained": trained, "us": t_fused * 1e6,
            "records_trained_per_s": trained / t_fused, "extract_then_train_us": t_unfused * 1e6,
            "fusion_speedup": t_unfused / t_fused}


def launches_per_step(path):
    """Kernels of this library launched per timed step (query pass + train step)."""
    if path == 0:
        # query: featurize, encode, 4 linear, mixture; train: encode, 4 linear, loss, 4x(wgrad+dgrad),
        # grid scatter, step counter, adam, stats
        return 7 + (1 + 4 + 1 + 8 + 1 + 1 + 1 + 1)
    return 1 + FUSED_TRAIN_LAUNCHES


FUSED_TRAIN_LAUNCHES = 5  # k_fused_train, k_step_inc, k_adam_ema, k_finish_stats, k_pack_weights


def cpu_baseline(q, x, rec, seconds=15.0, kind="port"):
    """The guiding step on the host cores (oracle/, OpenMP over every thread), on a bounded sample: the
    reference-order FP32 mixture code (bit-identical to the reference's own host build) and the FP32
    restatement of the encodings, MLP and Adam (the reference has no CPU implementation of the network).
    Builds nothing from the product library."""
    import numpy as np

    import oracle as O
    net = O.make_net(**HASHGRID_NET)
    rng = np.random.default_rng(0)
    params = np.zeros(net.n_params, np.float32)
    params[:net.n_mlp_params] = rng.uniform(-0.15, 0.15, net.n_mlp_params)
    params[net.n_mlp_params:] = rng.uniform(-1e-4, 1e-4, net.n_params - net.n_mlp_params)
    # query sample
    n = 4096
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < seconds / 2 or done == 0:
        sl = slice(done % (N_QUERIES - n), done % (N_QUERIES - n) + n)
        xi = O.featurize(net, q["pos"][sl], q["wo"][sl], q["normal"][sl], q["rough"][sl], q["aabb"])
        raw = O.network_forward_f32(net, params, xi)
        s = np.where((q["normal"][sl] * q["wo"][sl]).sum(1, keepdims=True) > 0, 1.0, -1.0).astype(np.float32)
        O.mixture_sample(raw, 8, q["u4"][sl], q["normal"][sl] * s, fp64=False)
        done += n
    tq = time.perf_counter() - t0
    # train sample
    m = 2048
    t1 = time.perf_counter()
    tdone = 0
    while time.perf_counter() - t1 < seconds / 2 or tdone == 0:
        sl = slice(tdone % (N_TRAIN - m), tdone % (N_TRAIN - m) + m)
        raw = O.network_forward_f32(net, params, x[sl])
        g, _, _ = O.mixture_loss_grad(raw, 8, rec[sl], 128.0, selection=True, fp64=False)
        O.network_backward_f32(net, params, x[sl], g)
        tdone += m
    tt = time.perf_counter() - t1
    # Adam over all parameters once per step, timed separately and amortised per sample of a 2^18 batch
    w = params.copy()
    mm, vv = np.zeros_like(w), np.zeros_like(w)
    ps, ema = np.zeros(w.size, np.uint32), w.copy()
    gr = np.zeros_like(w)
    ta = time.perf_counter()
    O.adam_ema(gr, 128.0, 1e-2, 0.9, 0.99, 1e-15, 1e-6, 0.95, 1, w, mm, vv, ps, ema, net.n_mlp_params)
    ta = time.perf_counter() - ta
    per_sample = tt / tdone + ta / N_TRAIN
    # one step of the workload: a query pass over N_QUERIES and a training step of N_TRAIN samples
    t_step = N_QUERIES * tq / done + N_TRAIN * per_sample
    return {"value": N_QUERIES / t_step, "unit": "queries/s (query pass + training step)",
            "train_samples_per_s": N_TRAIN / t_step, "query_pass_queries_per_s": done / tq,
            "train_step_samples_per_s": 1.0 / per_sample,
            "cores": O.num_threads(), "kind": kind,
            "sample": "%d queries and %d training samples of the same workload (FP32 reference-order mixture, "
                      "FP32 restated encoding + MLP + Adam, OpenMP), scaled to one step of 2,073,600 queries "
                      "and 262,144 training samples" % (done, tdone)}


def run_reference(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    synth = importlib.import_module(PKG + ".synth")
    q = synth.wavefront(N_QUERIES, seed=7272)
    field = synth.TrainField(seed=7272)
    x, rec = synth.train_batch(field, N_TRAIN, seed=7273, input_mode=1, selection=True)
    per = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_baseline(q, x, rec, seconds=1.0)
    t0 = time.perf_counter()
    vals, tvals, qvals, last = [], [], [], None
    for _ in range(args.steps):
        last = cpu_baseline(q, x, rec, seconds=per)
        vals.append(last["value"])
        tvals.append(last["train_samples_per_s"])
        qvals.append(last["query_pass_queries_per_s"])
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {
        "impl": "reference",
        "metric": "guided queries/s & train samples/s, BF16 fused vs FP32 plain, 1 GB300",
        "value": v, "unit": "queries/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / max(1, args.steps) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded wavefront + ground-truth radiance field)",
        "config": {"workload": "full guiding step: 2,073,600-query wavefront (1920x1080) + 2^18-sample train step",
                   "sample": "bounded per step; throughput scaled to the unit"},
        "train_samples_per_s": float(np.mean(tvals)),
        "rates": "value and train_samples_per_s: a step's 2,073,600 queries and 2^18 training samples over the "
                 "step's time (query pass + training step); query_pass: the query phase alone",
        "query_pass": {"queries_per_s": float(np.mean(qvals))},
        "cpu_baseline": {"value": v, "unit": "queries/s", "cores": last["cores"], "kind": "port",
                         "sample": last["sample"]},
        "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "what": "query pass + training step per step, on the host cores"},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="bf16", choices=["bf16", "fp16", "fp32"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-frame", action="store_true", help="skip the 7-bounce CUDA-graph frame measurement")
    ap.add_argument("--lobes", type=int, default=8, choices=[8, 16],
                    help="mixture lobes of the network (the measured line is quoted on 8; 16 for --steps-only profiling)")
    ap.add_argument("--steps-only", action="store_true",
                    help="time only the guiding steps (no CPU leg, plain path, frame, mixture or other rows); "
                         "the small command the ncu captures in profiles/ run")
    ap.add_argument("--tiling", type=int, default=0,
                    help="fused query tiling (0 = the default), with --steps-only, for profiling one kernel")
    ap.add_argument("--mixture-only", action="store_true",
                    help="time only the mixture-only kernels (no network), for profiling them")
    args = ap.parse_args()
    if args.tiling and not args.steps_only:
        ap.error("--tiling only with --steps-only: the measured line uses the default tiling")
    if args.lobes != 8 and not args.steps_only:
        ap.error("--lobes 16 only with --steps-only: the measured line is the 8-lobe configuration")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
