"""Benchmark: frames/s of PBRRenderer.step(return_pixels=True) on one GB300.

Workload (headline): CartPole render, 4096 scenes x 64x64 RGB uint8, two unit
cubes per scene (the benchmark CartPole scene of pybatchrender_gb300.workloads),
seeded synthetic states.  A step = write the step's states into the scene
+ one render of all scenes: ``step(state)``, which for this scene is one
kernel launch (the cart x, pole x and pole pitch columns of the state are
bound to the node poses with ``bind_state`` and read by the raster launch).
One frame = one scene image (steps x scenes / s, as the reference's cartpole
benchmark counts).

Reported variants (all on the same scene and states):
  value        the step above, inputs resident in HBM; per-step CUDA-event
               time with the L2 flushed (a 256 MiB write) before every step,
               flush excluded.
  e2e          the same call through the public API with host buffers:
               states copied from pinned host memory and pixels copied back to
               pinned host memory inside the timed region (wall clock); the
               device-to-host copy of step i runs on a second stream while
               step i+1 uploads and renders.
  variants     plain per-launch path (host-built matrices, a host-to-device
               copy per node, one launch per node, a synchronise); the fused
               step replayed as a CUDA graph (the state copied into the graph's
               static input, then the captured launch); the step
               through ``_step``'s torch copies + render captured in a CUDA
               graph; fused_over_plain / graph_over_plain: the fused launch and
               the graph replay against the plain path; soft_fwd (differentiable soft-coverage forward, float32)
               and fwd_bwd (soft forward + adjoint kernel with a constant
               dL/dout) on the same scene; env_step_eager / env_step_graph:
               the CartPole-v0 env step (dynamics, termination, reward,
               auto-reset, pixels) from Python and replayed as one CUDA graph.
  roofline     the hard-raster kernel alone: algorithmic bytes per launch /
               mean CUDA-event duration, against the measured HBM copy peak.
  cpu_baseline the oracle's FP32 rasteriser (a CPU port of the reference's
               shader path) on all host threads, bounded sample.

--impl reference runs that CPU port as the reference arm (the reference's own
render path is Panda3D + OpenGL, which cannot run without a graphics stack).
Under torchrun every rank renders its own 4096 scenes (independent replicas,
weak scaling); value = all frames / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "frames/s, 4096 scenes @64x64: plain vs batched graph vs fwd+bwd; %HBM peak"
UNIT = "frames/s"
BYTES_PER_INSTANCE = 80  # 4x4 f32 matrix or pose + RGBA f32 colour
BYTES_PER_SCENE = 80     # VP 4x4 f32 + light/tile


def algorithmic_bytes_per_frame(C: int, H: int, W: int, inst: int) -> int:
    return C * H * W + inst * BYTES_PER_INSTANCE + BYTES_PER_SCENE


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy burst)"
    return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` on `workload` from the committed ncu
    summary (profiles/traffic.txt: 'kernel workload bytes'), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == workload:
            return float(parts[2])
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the GPU works."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(os.environ.get("PBR_CLOCKS_DIR", tempfile.gettempdir()), f"clocks_gpu{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                rows.append((float(p[1]), float(p[2]), float(p[3]) if p[3] not in ("[N/A]", "") else 0.0, p[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        load = [r for r in rows if r[2] > 0] or rows
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in load:
            for n, v in zip(names, r[3]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def l2_flusher(device):
    buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)

    def flush():
        buf.fill_(1.0)
    return flush


def time_steps(fn, steps: int, flush, stream, pre=None) -> list[float]:
    """Per-step CUDA-event times (ms) on `stream`, L2 flushed before each step;
    `pre(i)`, if given, runs before the flush, outside the timed region."""
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        if pre is not None:
            pre(i)
        flush()
        evs[i][0].record(stream)
        fn(i)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def cpu_port_fps(num_scenes: int, res: int, seed: int, budget_s: float, threads: int, steps: int | None = None):
    """Frames/s of the oracle's FP32 rasteriser on `threads` host threads."""
    from oracle import oracle
    from pybatchrender_gb300 import workloads

    oracle.build()
    r = workloads.cartpole_bench(num_scenes=num_scenes, res=res, seed=seed, device="cpu")
    frames, elapsed, n = 0, 0.0, 0
    while True:
        r._step(workloads.cartpole_states(num_scenes, seed=1000 + n))
        sc, me, no = r.export_scene()
        t0 = time.perf_counter()
        oracle.render_hard(sc, me, no, precision="f32", nthreads=threads)
        elapsed += time.perf_counter() - t0
        frames += num_scenes
        n += 1
        if (steps is not None and n >= steps) or (steps is None and elapsed >= budget_s):
            break
    return frames / elapsed, n, elapsed


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for w in range(args.warmup):
        cpu_port_fps(args.scenes, args.res, 0, 0.0, threads, steps=1)
    fps, n, elapsed = cpu_port_fps(args.scenes, args.res, 0, 0.0, threads, steps=args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"cartpole_bench {args.scenes} scenes {args.res}x{args.res} RGB u8",
                   "parallelism": "cpu threads"},
        "cpu_baseline": {"value": fps, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} full steps of {args.scenes} scenes (oracle FP32 rasteriser, "
                                   "a CPU port of the reference's basic.vert/basic.frag path)"},
        "e2e": {"value": fps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference renders through Panda3D/OpenGL, unavailable on this box (no graphics stack)",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    from pybatchrender_gb300 import _capi, workloads

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    _capi.load(build_if_missing=True)
    N, res = args.scenes, args.res
    stream = torch.cuda.current_stream(device)
    flush = l2_flusher(device)
    states = [workloads.cartpole_states(N, seed=100 + i, device=device) for i in range(16)]

    graph_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", cuda_graph=True)
    tuned = graph_r.autotune() if args.autotune else None
    eager_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", reuse_output=True)
    if tuned:
        eager_r.cfg.raster_kernel = tuned["kernel"]
        eager_r.cfg.raster_threads, eager_r.cfg.bin_size = tuned["threads"], tuned["bin_px"]
        eager_r.cfg.persistent, eager_r.cfg.tri_cap = bool(tuned["persistent"]), tuned["tri_cap"]
        eager_r._build_context()
    plain_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", raster_method="plain")
    # the same step through _step's torch copies, graph-captured (no state binding)
    copy_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", cuda_graph=True)
    copy_r._state_bindings = []
    if tuned:
        copy_r.cfg.raster_kernel = tuned["kernel"]
        copy_r.cfg.raster_threads, copy_r.cfg.bin_size = tuned["threads"], tuned["bin_px"]
        copy_r.cfg.persistent, copy_r.cfg.tri_cap = bool(tuned["persistent"]), tuned["tri_cap"]
        copy_r._build_context()
    states_cpu = [s.cpu() for s in states]

    with ClockSampler(local) as clocks:
        # warm-up (graph capture happens on the first step)
        for i in range(max(3, args.warmup)):
            graph_r.step(states[i % 16])
            copy_r.step(states[i % 16])
        torch.cuda.synchronize()

        # headline: the env step (state -> poses -> pixels) as one launch, inputs resident in HBM
        barrier(world)
        t = time_steps(lambda i: graph_r.step(states[i % 16]), args.steps, flush, stream)
        barrier(world)
        graph_ms = reduce_max(sum(t), world)
        ms_per_step = graph_ms / args.steps
        value = world * N * args.steps / (graph_ms / 1000.0)

        # the same step with _step's torch copies, captured in a CUDA graph with the render
        t = time_steps(lambda i: copy_r.step(states[i % 16]), args.steps, flush, stream)
        copy_fps = N * args.steps / (reduce_max(sum(t), world) / 1000.0)

        # the fused step replayed as a CUDA graph: the step's state copied into the graph's static input,
        # then the captured state-bound launch
        static_state = states[0].clone()
        for i in range(3):
            graph_r.step(static_state)
        torch.cuda.synchronize()
        fused_graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(fused_graph):
            graph_r.step(static_state)

        def write_state(i):
            static_state.copy_(states[i % 16], non_blocking=True)

        def fused_graph_step(i):
            write_state(i)
            fused_graph.replay()
        for i in range(3):
            fused_graph_step(i)
        # the replay alone: the step's state is written into the graph's input beforehand, as an env's dynamics
        # write it in place (outside the timed region, like the states the eager step reads)
        t = time_steps(lambda i: fused_graph.replay(), args.steps, flush, stream, pre=write_state)
        fused_graph_fps = N * args.steps / (reduce_max(sum(t), world) / 1000.0)
        # the same with the state copied into the graph's input inside the timed step (a second launch)
        t = time_steps(fused_graph_step, args.steps, flush, stream)
        fused_graph_copy_fps = N * args.steps / (reduce_max(sum(t), world) / 1000.0)

        # plain per-launch path (wall clock: it synchronises every step)
        plain_steps = max(3, min(args.steps, args.plain_steps))
        for i in range(2):
            plain_r.step(states_cpu[i % 16])
        barrier(world)
        t0 = time.perf_counter()
        for i in range(plain_steps):
            plain_r.step(states_cpu[i % 16])
        torch.cuda.synchronize()
        plain_fps = N * plain_steps / reduce_max(time.perf_counter() - t0, world)

        # the hard-raster kernel alone (roofline)
        kt = time_steps(lambda i: eager_r.render(), args.steps, flush, stream)
        kernel_ms = statistics.mean(kt)

        # differentiable soft mode on the same scene: forward, and forward + adjoint
        soft_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", raster_mode="soft")
        gout = torch.full((N, 3, res, res), 1.0 / (N * 3 * res * res), device=device)
        soft_steps = max(3, min(args.steps, args.soft_steps))

        def soft_fwd(i):
            soft_r._step(states[i % 16])
            soft_r._soft_forward(None)

        def soft_fwd_bwd(i):
            soft_r._step(states[i % 16])
            out, st = soft_r._soft_forward(None)
            soft_r._soft_backward(out, st, gout)
        for i in range(2):
            soft_fwd_bwd(i)
        t = time_steps(soft_fwd, soft_steps, flush, stream)
        soft_fwd_fps = N * soft_steps / (reduce_max(sum(t), world) / 1000.0)
        t = time_steps(soft_fwd_bwd, soft_steps, flush, stream)
        fwd_bwd_fps = N * soft_steps / (reduce_max(sum(t), world) / 1000.0)

        # the CartPole env step (dynamics, termination, reward, auto-reset, pixels): eager, and replayed as
        # one CUDA graph
        import pybatchrender_gb300 as pbr
        env = pbr.envs.make("CartPole-v0", num_scenes=N, tile_resolution=(res, res), device="cuda")
        td0 = env.reset()
        env_obs, env_sc = td0["observation"].clone(), td0["step_count"].clone()
        env_acts = [torch.randint(0, 2, (N,), device=device) for _ in range(16)]

        def env_eager(i):
            env._step(pbr.env.TensorDict({"observation": env_obs, "action": env_acts[i % 16], "step_count": env_sc},
                                         batch_size=[N]))
        genv = pbr.GraphedEnvStep(env)

        def env_graph(i):
            genv({"observation": env_obs, "action": env_acts[i % 16], "step_count": env_sc})
        env_steps = max(3, min(args.steps, 200))
        for i in range(3):
            env_eager(i)
            env_graph(i)
        t = time_steps(env_eager, env_steps, flush, stream)
        env_eager_fps = N * env_steps / (reduce_max(sum(t), world) / 1000.0)
        t = time_steps(env_graph, env_steps, flush, stream)
        env_graph_fps = N * env_steps / (reduce_max(sum(t), world) / 1000.0)

        # end to end through the public API with host buffers: each step copies its states from pinned host
        # memory, renders into a fresh device tensor, and copies the pixels back to pinned host memory on a
        # second stream, so that step i's device-to-host copy overlaps step i+1's upload and render
        e2e_r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", reuse_output=False)
        host_in = [s.pin_memory() for s in states_cpu]
        host_out = [torch.empty((N, 3, res, res), dtype=torch.uint8).pin_memory() for _ in range(2)]
        dev_in = torch.empty((N, 4), dtype=torch.float32, device=device)
        copy_stream = torch.cuda.Stream(device)

        def e2e_step(i):
            dev_in.copy_(host_in[i % 16], non_blocking=True)
            pix = e2e_r.step(dev_in)
            copy_stream.wait_stream(stream)
            with torch.cuda.stream(copy_stream):
                host_out[i % 2].copy_(pix, non_blocking=True)
            pix.record_stream(copy_stream)
        for i in range(3):
            e2e_step(i)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for i in range(args.steps):
            e2e_step(i)
        torch.cuda.synchronize()
        e2e_s = reduce_max(time.perf_counter() - t0, world)
        e2e_fps = world * N * args.steps / e2e_s
    clk = clocks.summary()

    if rank != 0:
        return
    hbm_peak, peak_src = measured_peak()
    bpf = algorithmic_bytes_per_frame(3, res, res, 2)
    achieved = bpf * N / (kernel_ms / 1000.0) / 1e9
    workload_name = f"cartpole{N}x{res}"
    kname = "small_kernel" if eager_r.cfg.raster_kernel in ("warp", "auto") else "hard_kernel"
    traffic = ncu_traffic(kname, workload_name)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"cartpole_bench {N} scenes {res}x{res} RGB u8, 2 unit cubes/scene, seeded states",
                   "step": "state [N,4] -> cart x, pole x, pole pitch -> pixels in one launch (state columns bound "
                           "to poses); variants.batched_graph_step_copies = _step torch copies + render in a graph",
                   "global_batch": N * world, "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MiB write) before every timed step, flush excluded",
                   "launch": tuned or {"kernel": graph_r.cfg.raster_kernel, "threads": graph_r.cfg.raster_threads,
                                       "bin_px": graph_r.cfg.bin_size}},
        "variants": {"batched_fused_step": value / world, "batched_graph_fused_step": fused_graph_fps,
                     "batched_graph_fused_step_copy": fused_graph_copy_fps,
                     "batched_graph_step_copies": copy_fps, "plain": plain_fps,
                     "fused_over_plain": (value / world) / plain_fps,
                     "graph_over_plain": fused_graph_fps / plain_fps,
                     "soft_fwd": soft_fwd_fps, "fwd_bwd": fwd_bwd_fps, "soft_fwd_over_fwd_bwd": soft_fwd_fps / fwd_bwd_fps,
                     "env_step_eager": env_eager_fps, "env_step_graph": env_graph_fps},
        "e2e": {"value": e2e_fps, "unit": UNIT, "h2d_bytes_per_step": int(N * 4 * 4),
                "d2h_bytes_per_step": int(N * 3 * res * res)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "kernel": kname,
                     "kernel_ms": kernel_ms, "bytes_per_launch": bpf * N, "peak_source": peak_src},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if args.cpu_baseline and world == 1:
        threads = os.cpu_count() or 1
        fps, n, elapsed = cpu_port_fps(N, res, 0, args.cpu_budget, threads)
        line["cpu_baseline"] = {"value": fps, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{n} full steps of {N} scenes in {elapsed:.1f}s (oracle FP32 rasteriser)"}
    if args.workloads and world == 1:
        del graph_r, eager_r, plain_r, copy_r
        torch.cuda.empty_cache()
        line["workloads"] = run_workloads_inline(args, world, rank, local)
    print(json.dumps(line), flush=True)


def run_workload(args, world, rank, local, name: str | None = None, emit: bool = True) -> dict:
    """One of the other configurations, on its own JSON line (not the headline):
    many_cubes (1024 scenes 128x128 RGB + depth, 64 cubes), uneven (4096 scenes
    84x84, 1..512 instances of mixed meshes, graph-captured step with in-place
    pose updates), soft_cartpole (512 scenes 64x64 soft forward + adjoint),
    soft_large (16384 scenes 128x128 soft forward + adjoint, 128 instances)."""
    from pybatchrender_gb300 import _capi, workloads

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    _capi.load(build_if_missing=True)
    stream = torch.cuda.current_stream(device)
    flush = l2_flusher(device)
    name = name or args.workload
    hbm_peak, peak_src = measured_peak()
    line = {"workload": name, "unit": UNIT, "n_gpus": world, "higher_is_better": True, "scaling": "weak",
            "data": "synthetic", "steps": args.steps, "warmup": args.warmup}
    torch.cuda.reset_peak_memory_stats(device)
    free0, _ = torch.cuda.mem_get_info(device)
    if name in ("many_cubes", "uneven"):
        ns = {"num_scenes": args.workload_scenes} if args.workload_scenes > 0 else {}
        # a fixed tile-kernel launch (for profiling one configuration; the autotuner still runs unless disabled)
        for opt, field in (("raster_threads", "raster_threads"), ("bin_size", "bin_size"), ("tri_cap", "tri_cap")):
            if getattr(args, opt):
                ns[field] = getattr(args, opt)
        if args.raster_kernel != "auto":
            ns["raster_kernel"] = args.raster_kernel
        if name == "many_cubes":
            r = workloads.many_cubes(seed=rank, return_depth=True, reuse_output=True, **ns)
            n_inst = 64.0
            px_bytes = 3 + 4
            desc = f"{r.num_scenes} scenes 128x128 RGB u8 + f32 depth, 64 unit cubes/scene, random poses, hard raster"
        else:
            r = workloads.uneven(seed=rank, cuda_graph=True, persistent=True, **ns)
            n_inst = float(r.total_counts.float().mean())
            px_bytes = 3
            desc = (f"{r.num_scenes} scenes 84x84 RGB u8, log-uniform 1..512 instances/scene of cube/cylinder-64/icosphere-3, "
                    "per-scene camera, step = in-place HPR update + render, CUDA graph, persistent launch")
            nodes = r.uneven_nodes

            def upd():
                for nd in nodes:
                    nd.hpr.add_(0.01)
            r._step = lambda *a, **k: upd()
        tuned = r.autotune() if args.autotune else None
        N = r.num_scenes
        W, H = r.cfg.tile_resolution
        step = (lambda i: r.step()) if name == "uneven" else (lambda i: r.render())
        for i in range(max(3, args.warmup)):
            step(i)
        torch.cuda.synchronize()
        with ClockSampler(local) as clocks:
            t = time_steps(step, args.steps, flush, stream)
        line["clocks"] = clocks.summary()
        ms = reduce_max(sum(t), world) / args.steps
        bpf = W * H * px_bytes + n_inst * BYTES_PER_INSTANCE + BYTES_PER_SCENE
        fps = world * N / (ms / 1000.0)
        line.update({"metric": f"frames/s, {name}", "value": fps, "ms_per_step": ms, "dtype": "u8",
                     "config": {"workload": desc, "launch": tuned, "mean_instances": n_inst},
                     "roofline": {"bound": "hbm", "achieved": bpf * N / (ms / 1000.0) / 1e9, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": bpf * N / (ms / 1000.0) / 1e9 / hbm_peak,
                                  "bytes_per_frame": bpf, "peak_source": peak_src}})
    else:
        if name == "soft_cartpole":
            N, res = args.workload_scenes or 512, 64
            r = workloads.cartpole_bench(num_scenes=N, res=res, seed=rank, device="cuda", raster_mode="soft",
                                         **({} if args.raster_kernel == "auto" else {"raster_kernel": args.raster_kernel}))
            n_inst = 2
            desc = f"{N} scenes 64x64 f32 soft coverage (sigma 0.5 px edge, gamma 1e-3), CartPole bench scene"
            states = [workloads.cartpole_states(N, seed=100 + i, device=device) for i in range(16)]
            pre = lambda i: r._step(states[i % 16])
        else:
            N, res = args.workload_scenes or 16384, 128
            r = workloads.soft_large(num_scenes=N, res=res, seed=rank,
                                     **({} if args.raster_kernel == "auto" else {"raster_kernel": args.raster_kernel}))
            n_inst = 128
            desc = f"{N} scenes 128x128 f32 soft coverage, 128 instances/scene (64 icosphere-s2 + 64 cubes)"
            pre = lambda i: None
        gout = torch.full((N, 3, res, res), 1.0 / (N * 3 * res * res), device=device)

        def fwd(i):
            pre(i)
            r._soft_forward(None)

        def fwd_bwd(i):
            pre(i)
            out, st = r._soft_forward(None)
            r._soft_backward(out, st, gout)
        for i in range(max(3, args.warmup)):
            fwd_bwd(i)
        torch.cuda.synchronize()
        graphed = name == "soft_large"
        if graphed:
            # the step (forward + adjoint, gradient buffers zeroed inside) captured once and replayed: the
            # scene is static, so nothing is copied in per step
            torch.cuda.empty_cache()  # the footprint below is the graphs' memory, not the eager warm-up's cache
            g_f, g_b = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            with torch.cuda.graph(g_b):
                fwd_bwd(0)
            with torch.cuda.graph(g_f, pool=g_b.pool()):  # replays never overlap: one memory pool
                fwd(0)
            for i in range(2):
                g_f.replay()
                g_b.replay()
            torch.cuda.synchronize()
            with ClockSampler(local) as clocks:
                tf = time_steps(lambda i: g_f.replay(), args.steps, flush, stream)
                tb = time_steps(lambda i: g_b.replay(), args.steps, flush, stream)
        else:
            with ClockSampler(local) as clocks:
                tf = time_steps(fwd, args.steps, flush, stream)
                tb = time_steps(fwd_bwd, args.steps, flush, stream)
        line["clocks"] = clocks.summary()
        ms_f = reduce_max(sum(tf), world) / args.steps
        ms_b = reduce_max(sum(tb), world) / args.steps
        b_fwd = res * res * 12 + n_inst * BYTES_PER_INSTANCE + BYTES_PER_SCENE
        b_bwd = b_fwd + res * res * 12 + n_inst * 36 + 12
        line.update({"metric": f"frames/s, {name} forward + adjoint", "value": world * N / (ms_b / 1000.0),
                     "ms_per_step": ms_b, "dtype": "f32",
                     "forward": {"value": world * N / (ms_f / 1000.0), "ms_per_step": ms_f},
                     "fwd_over_fwd_bwd": ms_b / ms_f,
                     "config": {"workload": desc, "step": "CUDA graph replay" if graphed else "eager launches"},
                     "roofline": {"bound": "hbm", "achieved": b_bwd * N / (ms_b / 1000.0) / 1e9, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": b_bwd * N / (ms_b / 1000.0) / 1e9 / hbm_peak,
                                  "bytes_per_frame": b_bwd, "peak_source": peak_src}})
    # device memory in use beyond what was in use before the workload: tensors (PyTorch's cache at its
    # peak), the library's own scratch (e.g. the binned soft kernel's slabs) and graph pools
    free1, _ = torch.cuda.mem_get_info(device)
    line["hbm_footprint_bytes"] = int(free0 - free1)
    line["torch_peak_allocated_bytes"] = int(torch.cuda.max_memory_allocated(device))
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


WORKLOADS = ("many_cubes", "uneven", "soft_cartpole", "soft_large")


def run_workloads_inline(args, world, rank, local) -> dict:
    """The other configurations measured in the same run as the headline (one GPU), each with
    `--workload-steps` timed steps after 3 warm-up steps, summarised under the headline line's `workloads`."""
    import copy

    out = {}
    for name in WORKLOADS:
        a = copy.copy(args)
        a.steps, a.warmup, a.workload_scenes = args.workload_steps, 3, 0
        try:
            wl = run_workload(a, world, rank, local, name=name, emit=False)
            keep = ("metric", "value", "unit", "ms_per_step", "steps", "dtype", "forward", "fwd_over_fwd_bwd",
                    "hbm_footprint_bytes", "torch_peak_allocated_bytes", "clocks")
            d = {k: wl[k] for k in keep if k in wl}
            d["config"] = {k: wl["config"][k] for k in ("workload", "launch", "step") if k in wl.get("config", {})}
            d["roofline"] = {k: wl["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac",
                                                            "bytes_per_frame") if k in wl.get("roofline", {})}
            out[name] = d
        except Exception as e:  # a failing configuration is reported, not fatal to the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--res", type=int, default=64)
    ap.add_argument("--plain-steps", type=int, default=50)
    ap.add_argument("--soft-steps", type=int, default=100)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--workload-scenes", type=int, default=0,
                    help="scene count for --workload (0: the configuration's own; smaller for profiling)")
    ap.add_argument("--raster-kernel", default="auto", choices=["auto", "warp", "tile", "binned"],
                    help="--workload lines: the raster kernel (auto: the library's choice)")
    ap.add_argument("--raster-threads", type=int, default=0, help="many_cubes/uneven: tile kernel threads per CTA")
    ap.add_argument("--bin-size", type=int, default=0, help="many_cubes/uneven: tile kernel bin size in pixels")
    ap.add_argument("--tri-cap", type=int, default=0, help="many_cubes/uneven: tile kernel chunk size in triangles")
    ap.add_argument("--no-workloads", dest="workloads", action="store_false",
                    help="headline run only: skip the other configurations' summaries")
    ap.add_argument("--workload-steps", type=int, default=10,
                    help="timed steps of each configuration measured inside the headline run")
    ap.add_argument("--workload", default="cartpole",
                    choices=["cartpole", "many_cubes", "uneven", "soft_cartpole", "soft_large"],
                    help="cartpole = the headline; the others print their own line (see run_workload)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        elif args.workload != "cartpole":
            run_workload(args, world, rank, local)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
