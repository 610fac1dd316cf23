#!/usr/bin/env python
"""Benchmark of the raycasting + frequency-domain propagation path on one GB300.

Workload (default): the direct + one-bounce scene at 28 GHz -- 32x32
half-wave array, 20x20 m ground plane (80,000 triangles) + 40,000 clutter
triangles, 50,000 scatter points on triangle centroids, 65,341 far-field sinks
(1 deg grid at 100 m), uniform grid with 0.5 m cells.  One step = triangle
packing + grid build + direct stage + source->scatter stage + scatter->sink
stage (visibility, field, sink sum) with the inputs resident in HBM.

Metric: paths evaluated per second, paths = N*M direct pairs + N*P*M
source-scatter-sink triples (every path gets mask + field); the visible-path
count and rate are reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same path (the reference has
no CPU implementation; its only engines run on the GPU) on the host cores, on a
bounded sample of the same workload, extrapolated stage by stage.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lyceanem-python_gb300"))
sys.path.insert(0, ROOT)

METRIC = "visible paths/s (mask+field) on 1 GB300; mixed-prec vs FP32 sweep at ≤1e-4 rel err"
OPS_PER_TEST = 30  # FP32-pipe operations of one Moller-Trumbore test (lyceanem/src/raycasting.cuh:23-59)
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) of one full-size launch of the scatter->sink grid-stage kernel, from the
# one-pass ncu capture summarised in profiles/grid_stage_kernel_bounce.md (217.43 MB + 6.39 GB; the
# writes are the per-chunk partial sums and spill lines written back).
GRID_STAGE_DRAM_BYTES = 217.43e6 + 6.39e9
# DRAM bytes of one launch of the brute-force kernel on the 8x8-array direct scene (profiles/brute_stage_kernel_direct.md)
BRUTE_STAGE_DRAM_BYTES = 153.6e3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["bounce", "direct", "bounce_small"], default="bounce",
                    help="bounce_small: the bounce scene with 2,000 scatter points and a 4 deg sink grid "
                         "(profiling case)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the mixed-precision beam-sweep measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (differentiation) measurement")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched 64-scene x 64-frequency measurement")
    ap.add_argument("--batched-scenes", type=int, default=64,
                    help="scenes of the batched measurement (the first S of the 64-scene recipe; profiling cases)")
    ap.add_argument("--batched-config", default="",
                    help="fg,chunk,blocks_per_sm for the batched launch instead of the autotuner (profiling cases)")
    ap.add_argument("--batched-cell-scale", type=float, default=0.0,
                    help="grid cell scale k of the batched scenes instead of the autotuner (profiling cases)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU time of the sampled baseline")
    return ap.parse_args()


def workload_scene(name):
    from lyceanem_gb300 import scenes
    if name == "direct":
        return scenes.direct_scene()
    if name == "bounce_small":
        return scenes.bounce_scene(n_scatter=2000, el_n=46, az_n=91)
    return scenes.bounce_scene()


def describe(s, name):
    N, M, P, T = s.src.shape[0], s.snk.shape[0], s.scat.shape[0], s.faces.shape[0]
    paths = N * M + N * P * M
    if name == "direct":
        wl = "direct path, 10 GHz, 8x8 array, 2,664 sinks at 10 m, 1,024 obstruction triangles, brute force"
    elif name == "bounce_small":
        wl = ("profiling case: bounce scene with 2,000 scatter points and 4,186 sinks (4 deg grid at 100 m), "
              "0.5 m grid")
    else:
        wl = ("direct + one bounce, 28 GHz, 32x32 array, 80,000 ground + 40,000 clutter triangles, "
              "50,000 scatter points, 65,341 sinks at 100 m, 0.5 m grid")
    return {"workload": wl, "n_sources": N, "n_scatter": P, "n_sinks": M, "n_triangles": T, "paths_per_step": paths,
            "grid_cell_m": s.cell, "l2": "flushed by a 256 MiB device write before every timed step"}, paths


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")
        self.gpu_index = gpu_index

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        mhz = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ ours
def max_over_ranks(value, device):
    """The largest of `value` over the ranks of the process group (the slowest replica sets the
    whole job's time); `value` itself without a group or with one rank."""
    import torch
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, world, steps, total_ms):
    """Units per second of the whole job: every rank processes units_per_step each step (weak scaling)."""
    return units_per_step * world * steps / (total_ms / 1e3)


def run_ours(args, rank, world):
    import numpy as np
    import torch

    from lyceanem_gb300 import propagation as P

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    s = workload_scene(args.workload)
    cfg, paths = describe(s, args.workload)
    beta = 2 * np.pi / s.wavelength
    t = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    src, E, snk, snk_n = t(s.src), t(s.E), t(s.snk), t(s.snk_n)
    scat, scat_n = t(s.scat), t(s.scat_n)
    verts, faces = t(s.verts), t(s.faces)
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    cnt_s2 = torch.zeros(2, dtype=torch.int64, device=dev)
    cnt_all = torch.zeros(2, dtype=torch.int64, device=dev)
    vis_scat_in = torch.zeros(Pn, dtype=torch.int32, device=dev)
    vis_scat_out = torch.zeros(Pn, dtype=torch.int32, device=dev)
    vis_direct = torch.zeros(M, dtype=torch.int32, device=dev)
    ev = {}

    def step(mark=False):
        tris = P.pack_triangles(verts, faces)
        if args.workload == "direct":
            out = P.pair_stage(src, E, snk, snk_n, beta=beta, tris=tris, counters=cnt_all, snk_visible=vis_direct)
            if mark:
                ev["s2"] = (None, None)
            return out.sink
        grid = P.UniformGrid(tris, cell=s.cell)
        o_scat = P.spatial_order(scat)  # scatter points are traced in Morton order
        o_snk = P.direction_order(snk, grid.centre)  # sinks in direction order from the scene
        out = P.pair_stage(src, E, snk, snk_n, beta=beta, grid=grid, counters=cnt_all, snk_visible=vis_direct,
                           snk_order=o_snk).sink
        e_p = P.pair_stage(src, E, scat, scat_n, beta=beta, grid=grid, counters=cnt_all,
                           snk_visible=vis_scat_in, snk_order=o_scat).sink
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        P.pair_stage(scat, e_p, snk, snk_n, beta=beta, grid=grid, src_W=e_p, sink_out=out, accumulate=True,
                     counters=cnt_s2, src_visible=vis_scat_out, src_order=o_scat, snk_order=o_snk)
        b.record()
        if mark:
            ev.setdefault("s2_list", []).append((a, b))
        return out

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # counters describe one step: zero them after warm-up, divide by K afterwards
    for c in (cnt_s2, cnt_all, vis_scat_in, vis_scat_out, vis_direct):
        c.zero_()
    fma_rate = P.fp32_fma_rate()
    clocks = ClockSampler(dev.index)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = P.kernel_launches()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        step(mark=True)
        b.record()
        step_ms.append((a, b))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches = P.kernel_launches() - launches0
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in step_ms), dev)
    K = args.steps
    ms_per_step = total_ms / K
    value = whole_job_rate(paths, world, K, total_ms)
    st, flags = P.device_errors()
    if st != 0 or flags != 0:
        raise RuntimeError(f"device error word {flags:#x}")
    vis_direct_total = int(vis_direct.sum().item()) // K
    if args.workload != "direct":
        vin = vis_scat_in.double() / K
        vout = vis_scat_out.double() / K
        visible_paths = vis_direct_total + float((vin * vout).sum().item())
    else:
        visible_paths = vis_direct_total
    rays = N * M + (N * Pn + Pn * M if args.workload != "direct" else 0)
    res = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
           "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 (visibility bit-specified FP32; field FP32 with FP64 phase)", "data": "synthetic",
           "config": dict(cfg, parallelism="replicas" if world > 1 else "single GPU"),
           "visible_paths_per_step": visible_paths, "visible_paths_per_s": visible_paths * world * K / (total_ms / 1e3),
           "rays_per_s": rays * world * K / (total_ms / 1e3), "gpu_launches": launches}
    # roofline of the dominant kernel (scatter->sink grid stage; direct stage for the direct workload)
    T = int(faces.shape[0])
    if args.workload != "direct":
        s2_ms = sum(a.elapsed_time(b) for a, b in ev["s2_list"]) / K
        tests = int(cnt_s2[1].item()) / K
        brute_tests = float(Pn) * M * T
        kernel = "grid_stage_kernel (scatter->sink stage incl. its partial-sum reduction)"
    else:
        s2_ms = ms_per_step
        tests = int(cnt_all[1].item()) / K
        brute_tests = float(N) * M * T
        kernel = "brute_stage_kernel (whole step)"
    achieved = tests * OPS_PER_TEST / (s2_ms / 1e3) / 1e12
    peak = fma_rate / 1e12
    res["roofline"] = {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                       "frac": achieved / peak,
                       "traffic": GRID_STAGE_DRAM_BYTES if args.workload == "bounce" else
                       (BRUTE_STAGE_DRAM_BYTES if args.workload == "direct" else None),
                       "peak_source": "measured FP32 FMA lane-op rate (lyem_fp32_fma_probe, same run; FMA = 1 op)",
                       "tests_per_launch": tests, "ops_per_test": OPS_PER_TEST, "launch_ms": s2_ms,
                       "share_of_step": s2_ms / ms_per_step,
                       # the same launch counted in brute-force tests (every ray against every triangle)
                       "effective_tests_per_s": brute_tests / (s2_ms / 1e3),
                       "effective_frac": brute_tests * OPS_PER_TEST / (s2_ms / 1e3) / 1e12 / peak}
    if clk:
        res["clocks"] = clk
    if rank == 0 and world == 1 and not args.no_sweep:
        res["sweep"] = run_sweep(args)
    if rank == 0 and world == 1 and not args.no_adjoint:
        res["adjoint"] = run_adjoint(args)
    if rank == 0 and world == 1 and not args.no_batched:
        res["batched"] = run_batched(args)
    if rank == 0 and world == 1 and not args.no_e2e:
        res["e2e"] = run_e2e(args, s, paths)
    if rank == 0 and world == 1 and not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(args, s, paths)
    return res


def run_e2e(args, s, paths):
    """Same metric through the reference-shaped host API: numpy in, numpy out, copies inside the timed region."""
    import numpy as np
    import torch

    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import frequency_domain as FD
    beta = 2 * np.pi / s.wavelength
    solid = Mesh(s.verts, [("triangle", s.faces)])
    ap = Mesh(s.src, point_data={"Normals": s.src_n, "Area": np.ones(s.src.shape[0], np.float32)})
    sk = Mesh(s.snk, point_data={"Normals": s.snk_n})
    sc = Mesh(s.scat, point_data={"Normals": s.scat_n}) if s.scat.shape[0] else None
    scattering = 0 if args.workload == "direct" else 1
    axis = np.array([1.0, 0.0, 0.0])

    def call():
        return FD.calculate_scattering(ap, sk, solid, axis, scatter_points=sc, wavelength=s.wavelength,
                                       scattering=scattering, beta=beta, cuda=True, grid_cell=s.cell)

    call()
    torch.cuda.synchronize()
    K = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(K):
        Ex, Ey, Ez = call()
    dt = (time.perf_counter() - t0) / K
    V, T = s.verts.shape[0], s.faces.shape[0]
    h2d = (3 * (V * 12 + T * 12) + s.src.nbytes + s.src.shape[0] * 24 + s.snk.nbytes + s.snk_n.nbytes
           + s.scat.nbytes + s.scat_n.nbytes)
    d2h = Ex.nbytes + Ey.nbytes + Ez.nbytes
    return {"value": paths / dt, "unit": "paths/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "seconds_per_step": dt,
            "api": "lyceanem_gb300.models.frequency_domain.calculate_scattering (host numpy in/out, "
                   "acceleration structure built inside the call)"}


# ------------------------------------------------------------------ sweep
def run_sweep(args, n_check=256, reps=5):
    """Mixed-precision beam sweep: 64x64 array at 28 GHz, ground + 20,000 clutter triangles, 65,341 sinks,
    K = 2,048 steering vectors.  Times the three component GEMMs per mode on the formed network and measures
    each mode's error against an FP64 product on a seeded sample of sinks (oracle network, all beams)."""
    import numpy as np
    import torch

    from lyceanem_gb300 import beam_sweep as BS
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes
    from oracle import oracle as O
    s = scenes.sweep_scene()
    beta = 2 * np.pi / s.wavelength
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    grid = P.UniformGrid(tris, cell=s.cell)
    N, M, K = s.src.shape[0], s.snk.shape[0], s.weights.shape[0]
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    G = BS.form_network(t(s.src), s.pol, t(s.snk), t(s.snk_n), beta=beta, grid=grid)
    b.record()
    torch.cuda.synchronize()
    form_ms = a.elapsed_time(b)
    W = t(s.weights)
    rng = np.random.default_rng(7)
    pick = np.sort(rng.choice(M, size=n_check, replace=False))
    flops = 8.0 * M * N * K * 3
    res = {"n_elements": N, "n_sinks": M, "n_beams": K, "network_form_ms": form_ms,
           "algorithmic_flops": flops}
    outs = {}
    for mode in ("fp32", "bf16x3", "fp16x3", "bf16x3g", "fp16x3g"):
        sw = BS.BeamSweep(G, mode)
        out = sw.run(W)
        torch.cuda.synchronize()
        ev = []
        for _ in range(reps):
            x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            x.record()
            sw.run(W, out=out)
            y.record()
            ev.append((x, y))
        torch.cuda.synchronize()
        ms = min(x.elapsed_time(y) for x, y in ev)
        outs[mode] = sw.fields(out)[torch.from_numpy(pick).cuda()].cpu().numpy()
        res[mode] = {"ms": ms, "tflops_algorithmic": flops / (ms * 1e-3) / 1e12}
        del sw, out
        torch.cuda.empty_cache()
    del G
    # FP64 reference on the sampled sinks: oracle visibility + FP64 network, FP64 product
    og = O.Grid(O.pack_triangles(s.verts, s.faces), s.cell)
    snk, snk_n = s.snk[pick], s.snk_n[pick]
    mask = og.mask(s.src, snk, self_to_self=True)  # the network tests every pair (sink indices are sampled)
    G64 = O.pair_field(s.src, np.tile(s.pol, (N, 1)), snk, snk_n, mask, 0.0, beta)
    E64 = np.einsum("nmc,kn->mkc", G64, s.weights.astype(np.complex128), optimize=True)
    for mode, E in outs.items():
        res[mode]["rel_err_fp64"] = float(np.linalg.norm(E - E64) / np.linalg.norm(E64))
    res["speedup_bf16x3_vs_fp32"] = res["fp32"]["ms"] / res["bf16x3"]["ms"]
    res["speedup_fp16x3_vs_fp32"] = res["fp32"]["ms"] / res["fp16x3"]["ms"]
    res["speedup_bf16x3g_vs_fp32"] = res["fp32"]["ms"] / res["bf16x3g"]["ms"]
    res["speedup_fp16x3g_vs_fp32"] = res["fp32"]["ms"] / res["fp16x3g"]["ms"]
    res["error_sample"] = f"{n_check} seeded sinks x {K} beams x 3 components, relative Frobenius norm"
    return res


# ------------------------------------------------------------------ batched
BATCH_TUNE_CANDIDATES = [(2, 64, 8), (2, 64, 6), (1, 64, 8), (4, 64, 8)]
# grid cell edge per scene = k * (box volume / triangles)^(1/3); the autotuner picks k
BATCH_TUNE_CELL_SCALES = [1.0, 1.25, 1.5]


def run_batched(args, reps=2):
    """Batched uneven workload: 64 scenes (square half-wave arrays of 16-16,384 elements and 1e3-5e5
    triangles, both log-uniform, ground + clutter recipe scaled to the count, scatter points on 10% of the
    triangles up to 10,000), 10,000 Fibonacci sinks at 50 m, 64 frequencies 24-30 GHz, direct + one bounce.
    One persistent launch per step, replayed from a captured CUDA graph; configuration and grid cell
    scale picked by the autotuner on a cost-stratified quarter of the scenes.  Checked against the per-scene pair-stage path
    (three scenes, first/middle/last frequency) and against the FP64 oracle on the smallest scene."""
    import numpy as np
    import torch

    from lyceanem_gb300 import batched as B
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes as SC
    from oracle import oracle as O
    scenes, snk, snk_n, freqs = SC.batched_scenes(n_scenes=args.batched_scenes)
    t0 = time.time()
    fixed = args.batched_config and args.batched_cell_scale > 0
    bs = B.BatchedScattering(scenes, snk, snk_n, freqs, cell_scale=args.batched_cell_scale if fixed else 1.0)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    t0 = time.time()
    if fixed:
        bs.configure(tuple(int(v) for v in args.batched_config.split(",")))
        tune = {}
    else:
        proxy = B.BatchedScattering([scenes[i] for i in B.stratified_subset(scenes, snk.shape[0])], snk, snk_n,
                                    freqs, cell_scale=1.0)
        cands = [tuple(int(v) for v in args.batched_config.split(","))] if args.batched_config else \
            BATCH_TUNE_CANDIDATES
        scales = [args.batched_cell_scale] if args.batched_cell_scale > 0 else BATCH_TUNE_CELL_SCALES
        tune = bs.autotune(candidates=cands, proxy=proxy, use_cache=False, cell_scales=scales)
        del proxy
        torch.cuda.empty_cache()
    tune_s = time.time() - t0
    bs.capture()
    bs.run()
    torch.cuda.synchronize()
    ev = []
    for _ in range(reps):
        x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        x.record()
        bs.run()
        y.record()
        ev.append((x, y))
    torch.cuda.synchronize()
    times = [x.elapsed_time(y) for x, y in ev]
    st, flags = P.device_errors()
    cnt = bs.counters.cpu().numpy()
    ms = statistics.mean(times)
    paths = bs.paths()
    res = {"workload": "64 uneven scenes x 64 frequencies (24-30 GHz), direct + one bounce, 10,000 sinks at 50 m",
           "n_scenes": bs.n_scenes, "n_freq": bs.n_freq, "n_sinks": bs.n_snk,
           "elements_total": int(sum(d.src.shape[0] for d in bs.data)),
           "triangles_total": int(sum(d.n_tris for d in bs.data)),
           "scatter_total": int(sum(d.scat.shape[0] for d in bs.data)),
           "config": {"freq_group": bs.config[0], "src_chunk": bs.config[1], "blocks_per_sm": bs.config[2],
                      "blocks": bs.blocks, "cell_scale": bs.cell_scale,
                      "grid_cell_m": {"min": min(bs.grid_cells()), "median": statistics.median(bs.grid_cells()),
                                      "max": max(bs.grid_cells())}},
           "autotune_ms": {str(list(k)): v for k, v in tune.items()}, "autotune_s": tune_s, "setup_s": setup_s,
           "items": bs.items(), "ms_per_launch": ms, "ms_runs": times,
           "paths_per_launch": paths, "paths_per_s": paths / (ms / 1e3),
           "visibility_pairs_per_launch": bs.pairs(),
           "visible_pairs": [int(v) for v in cnt[:, :3].sum(0)],
           "ray_triangle_tests": int(cnt[:, 3].sum()), "tests_per_s": float(cnt[:, 3].sum() / (ms / 1e3)),
           "graph": "1 persistent kernel + 2 memsets per replay", "kernels_per_step": 1,
           "device_errors": [int(st), int(flags)]}
    # per-scene pair stages at the same frequency (FP64 phase path)
    worst = 0.0
    field = bs.field
    for si in (0, len(scenes) // 2, len(scenes) - 1):
        d, sc = bs.data[si], scenes[si]
        scat, scat_n = torch.from_numpy(sc.scat).cuda(), torch.from_numpy(sc.scat_n).cuda()
        E = np.array([1, 0, 0], np.complex64)
        for f in (0, bs.n_freq // 2, bs.n_freq - 1):
            kw = dict(grid=d.grid, alpha=0.0, beta=float(bs.betas[f]), self_to_self=False)
            out = P.pair_stage(sc.src, E, snk, snk_n, **kw).sink
            ep = P.pair_stage(sc.src, E, scat, scat_n, **kw).sink
            P.pair_stage(scat, ep, snk, snk_n, src_W=ep, sink_out=out, accumulate=True, **kw)
            ref = out.cpu().numpy()
            worst = max(worst, float(np.abs(field[si, f].cpu().numpy() - ref).max() / np.abs(ref).max()))
    res["rel_err_vs_pair_stages"] = worst
    # FP64 oracle (brute-force visibility on the host) on the scene with the fewest ray-triangle tests,
    # first and last frequency; skipped when even that scene is too large for a bounded CPU check
    costs = [(d.src.shape[0] * (bs.n_snk + d.scat.shape[0]) + d.scat.shape[0] * bs.n_snk) * d.n_tris for d in bs.data]
    si = int(np.argmin(costs))
    if costs[si] > 5e10:
        res["rel_err_fp64_oracle"] = None
        res["oracle_scene"] = "skipped: smallest scene needs more than 5e10 host ray-triangle tests"
        return res
    sc = scenes[si]
    t12 = O.pack_triangles(sc.verts, sc.faces)
    m0, m1, m2 = O.mask_brute(sc.src, snk, t12), O.mask_brute(sc.src, sc.scat, t12), O.mask_brute(sc.scat, snk, t12)
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (sc.src.shape[0], 1))
    worst = 0.0
    for f in (0, bs.n_freq - 1):
        b_ = float(bs.betas[f])
        e = O.sink_field(sc.src, E, snk, snk_n, 0.0, b_, mask=m0)
        ep = O.sink_field(sc.src, E, sc.scat, sc.scat_n, 0.0, b_, mask=m1)
        e = e + O.sink_field(sc.scat, ep, snk, snk_n, 0.0, b_, srcW=ep, mask=m2)
        worst = max(worst, float(np.abs(field[si, f].cpu().numpy() - e).max() / np.abs(e).max()))
    res["rel_err_fp64_oracle"] = worst
    res["oracle_scene"] = {"index": si, "elements": int(sc.src.shape[0]), "scatter": int(sc.scat.shape[0]),
                           "triangles": int(sc.faces.shape[0])}
    return res


# ------------------------------------------------------------------ adjoint
def _model_fp64(a, x, y, pol, y_n, scat, scat_n, m0, m1, m2, beta, chunk=256):
    """FP64 torch restatement of the forward sink field (em_wave composed as the reference's one bounce),
    visibility from the given masks, chunked over scatter points; runs on the GPU in float64."""
    import numpy as np
    import torch
    kappa = 1j * beta
    front = -1.0 / (2 * np.pi)

    def G(s, e, t, t_n, mask):
        rv = t[None, :, :] - s[:, None, :]
        r = torch.sqrt((rv * rv).sum(-1))
        d = rv / r[..., None]
        F = front * (-(kappa / r + 1.0 / r ** 2)) * torch.exp(-kappa * r)
        sd = (t_n[None, :, :] * d).sum(-1)
        q = e[:, None, :] - (e[:, None, :] * d).sum(-1, keepdim=True) * d
        return mask[..., None] * (F * sd)[..., None] * q

    E_src = a[:, None] * pol
    E = G(x, E_src, y, y_n, m0).sum(0)
    w = G(x, E_src, scat, scat_n, m1).sum(0)
    for p0 in range(0, scat.shape[0], chunk):
        p1 = min(p0 + chunk, scat.shape[0])
        E = E + (w[p0:p1, None, :] * G(scat[p0:p1], w[p0:p1], y, y_n, m2[p0:p1])).sum(0)
    return E


def run_adjoint(args, reps=3):
    """Differentiation scene: 16x16 array, 10,000 scatter points, 32,761 front-hemisphere sinks; loss
    sum |E - E_target|^2 with E_target the field of a seeded random-phase excitation.  Times forward and
    backward and checks gradient components against FP64 central differences (step 1e-4 wavelengths for
    positions) of an FP64 restatement of the forward model with the same masks."""
    import numpy as np
    import torch

    from lyceanem_gb300 import adjoint as A
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes
    s = scenes.adjoint_scene()
    beta = 2 * np.pi / s.wavelength
    dev = torch.device("cuda")
    t = lambda z: torch.from_numpy(np.ascontiguousarray(z)).to(dev)  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    grid = P.UniformGrid(tris, cell=s.cell)
    x0, y0, pol = t(s.src), t(s.snk), t(s.E)
    sn, sc, scn = t(s.snk_n), t(s.scat), t(s.scat_n)
    kw = dict(beta=beta, grid=grid)
    with torch.no_grad():
        target = A.sink_field(t(s.target_excitation), x0, y0, pol, sn, sc, scn, **kw).clone()
    N, M, Pn = x0.shape[0], y0.shape[0], sc.shape[0]
    fw, bw = [], []
    for _ in range(reps + 1):
        a = torch.ones(N, dtype=torch.complex64, device=dev, requires_grad=True)
        x = x0.clone().requires_grad_(True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        E = A.sink_field(a, x, y0, pol, sn, sc, scn, **kw)
        loss = ((E - target).abs() ** 2).sum()
        e1.record()
        loss.backward()
        e2.record()
        torch.cuda.synchronize()
        fw.append(e0.elapsed_time(e1))
        bw.append(e1.elapsed_time(e2))
    ga, gx = a.grad.detach(), x.grad.detach()
    # masks of the forward's three stages (deterministic), then FP64 central differences
    m0 = P.pair_stage(x0, pol, y0, sn, want_mask=True, **kw).mask().double()
    m1 = P.pair_stage(x0, pol, sc, scn, want_mask=True, **kw).mask().double()
    m2 = P.pair_stage(sc, pol[:1].expand(Pn, 3), y0, sn, want_mask=True, **kw).mask().double()
    d64 = lambda z: z.detach().to(torch.float64)  # noqa: E731
    c64 = lambda z: z.detach().to(torch.complex128)  # noqa: E731
    args64 = (d64(y0), c64(pol), d64(sn), d64(sc), d64(scn), m0, m1, m2, beta)

    def L(a_, x_):
        with torch.no_grad():
            E_ = _model_fp64(a_, x_, args64[0], args64[1], *args64[2:])
            return float(((E_ - c64(target)).abs() ** 2).sum())

    a64, x64 = torch.ones(N, dtype=torch.complex128, device=dev), d64(x0)
    h = 1e-4 * s.wavelength
    rng = np.random.default_rng(11)
    errs = []
    for n in rng.choice(N, size=2, replace=False):
        for part in (1.0, 1j):
            da = torch.zeros_like(a64)
            da[n] = part * 1e-4
            fd = (L(a64 + da, x64) - L(a64 - da, x64)) / 2e-4
            got = ga[n].real if part == 1.0 else ga[n].imag
            errs.append(abs(float(got) - fd) / float(ga.abs().max()))
    for n, k in zip(rng.choice(N, size=2, replace=False), (0, 2)):
        dx = torch.zeros_like(x64)
        dx[n, k] = h
        fd = (L(a64, x64 + dx) - L(a64, x64 - dx)) / (2 * h)
        errs.append(abs(float(gx[n, k]) - fd) / float(gx.abs().max()))
    return {"n_elements": N, "n_scatter": Pn, "n_sinks": M, "forward_ms": min(fw[1:]), "backward_ms": min(bw[1:]),
            "fd_components": len(errs), "fd_max_rel_err": max(errs),
            "fd_check": "FP64 central differences of an FP64 restatement of the forward with the forward's masks; "
                        "error = |grad - fd| / max|grad| over 4 excitation and 2 position components"}


# ------------------------------------------------------------------ CPU
def cpu_sample(s, stride_snk, stride_scat, nthreads):
    """Times the oracle on every stride-th sink / scatter point; returns per-stage seconds."""
    import numpy as np

    from oracle import oracle as O
    beta = 2 * np.pi / s.wavelength
    snk, snk_n = s.snk[::stride_snk], s.snk_n[::stride_snk]
    scat, scat_n = s.scat[::stride_scat], s.scat_n[::stride_scat]
    t0 = time.perf_counter()
    tris = O.pack_triangles(s.verts, s.faces)
    grid = O.Grid(tris, s.cell) if s.cell else None
    kw = dict(grid=grid, tris12=None if grid else tris, nthreads=nthreads)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.sink_field(s.src, s.E, snk, snk_n, 0.0, beta, **kw)
    t_direct = time.perf_counter() - t0
    t_s1 = t_s2 = 0.0
    if scat.shape[0]:
        t0 = time.perf_counter()
        e_p = O.sink_field(s.src, s.E, scat, scat_n, 0.0, beta, **kw)
        t_s1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.sink_field(scat, e_p, snk, snk_n, 0.0, beta, srcW=e_p, **kw)
        t_s2 = time.perf_counter() - t0
    return dict(build=t_build, direct=t_direct, s1=t_s1, s2=t_s2, n_snk=snk.shape[0], n_scat=scat.shape[0])


def cpu_extrapolate(s, paths, nthreads, target_s):
    """Calibrate a sample size for ~target_s of CPU work, time it, extrapolate per stage to the full workload."""
    M, P = s.snk.shape[0], s.scat.shape[0]
    cal = cpu_sample(s, 256, 256, nthreads)
    # direct and source->scatter work scale with 1/stride, scatter->sink with 1/stride^2
    stride = 256
    while stride > 1:
        nxt = stride // 2
        est = (cal["direct"] + cal["s1"]) * (256 / nxt) + cal["s2"] * (256 / nxt) ** 2
        if est > target_s:
            break
        stride = nxt
    r = cpu_sample(s, stride, stride, nthreads)
    full = (r["build"] + r["direct"] * M / r["n_snk"]
            + (r["s1"] * P / r["n_scat"] + r["s2"] * (P * M) / (r["n_scat"] * r["n_snk"]) if r["n_scat"] else 0.0))
    sample_s = r["build"] + r["direct"] + r["s1"] + r["s2"]
    desc = (f"oracle (FP32 bit-faithful visibility on a CPU uniform grid, FP64 field) on every {stride}th sink "
            f"({r['n_snk']}) and scatter point ({r['n_scat']}) with all {s.src.shape[0]} sources; "
            f"{sample_s:.1f} s measured, extrapolated per stage (direct x M/M', source->scatter x P/P', "
            f"scatter->sink x PM/(P'M')) to {full:.1f} s for the full step")
    return paths / full, desc, full


def cpu_baseline(args, s, paths):
    from oracle import oracle as O
    n = O.max_threads()
    value, desc, _ = cpu_extrapolate(s, paths, n, args.cpu_seconds)
    return {"value": value, "unit": "paths/s", "cores": n, "kind": "port", "sample": desc}


def run_reference(args, rank, world):
    """CPU restatement of the path on the host cores (the reference has no CPU engine)."""
    from oracle import oracle as O
    s = workload_scene(args.workload)
    cfg, paths = describe(s, args.workload)
    n = O.max_threads()
    vals, descs, fulls = [], [], []
    for _ in range(max(1, args.steps)):
        v, d, full = cpu_extrapolate(s, paths, n, args.cpu_seconds / max(1, args.steps))
        vals.append(v)
        descs.append(d)
        fulls.append(full)
    value = len(vals) / sum(1.0 / v for v in vals)
    ms = 1e3 * sum(fulls) / len(fulls)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 visibility / f64 field (CPU)", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": n, "kind": "port", "sample": descs[-1]},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)), flush=True)
        return 0
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
