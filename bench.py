"""Benchmark of the chunk-meshing path on GB300.

Default workload (the large clipmap sweep): 4096 chunks of 64^3 voxels over
clipmap LODs 0-5 (voxel sizes 1-32), the union of SelectActiveClipmapNodes
along a seeded camera path, nearest first; density = 2D fBm heightfield (8
octaves, 1/256, lacunarity 2, gain 0.5, amplitude 48) + 3D fBm caves (6
octaves, 1/64, amplitude 12), noise seed 1; 64 seeded CSG operations (half
sphere-subtract, half box-union, radii / half extents U[2, 12] voxels) stored
and replayed per chunk through the plain path.  A step meshes every chunk
from a fresh field (caches bypassed): field, CSG, edges, hermite data,
leaves + QEF, cuckoo tables, mesh, seams.

  value  plain-path chunks/s with outputs left in device memory (per-step
         CUDA events on the library's stream; L2 flushed between steps,
         outside the timed events)
  e2e    chunks/s through the same C-ABI call with host output arrays
         (pinned), device-to-host copies inside the timed region
  surrogate
         the learned density: sampled and trained on the GPU (2^24 fresh
         plain samples, 20k Adam steps at batch 65,536), then the same 4096
         chunks meshed with it under its per-chunk probe gate; surrogate
         chunks/s, fallback rate, mesh Hausdorff distance to the plain
         meshes, density error against FP32 and FP64, training time and
         tensor throughput

`--impl reference` times the CPU restatement of the reference algorithm
(oracle/, the reference's OpenCL cannot run here) on all host threads over
a bounded sample of the same workload.

Other workloads (`--workload`): `tiled`, 128 LOD0 chunks tiling a
512 x 128 x 512-voxel region of the 2D fBm terrain with 32 seeded CSG
operations; `clipmap`, 1024 chunks over clipmap LODs 0-4 around a moving
seeded camera, caves density, followed by the octree simplification at QEF
error 0.05 (CPU baseline: the same, simplification included); `one`, a single
LOD0 chunk.  `--workload select`: the clipmap's active-node selection
(SelectActiveClipmapNodes) for 4096 cameras on 64 seeded paths through the
2^15-unit world, one launch per step (its own JSON line, impl "lvn-select";
the reference arm times the oracle's recursion on all host threads).
`--workload seams`: the seam meshes (GenerateClipmapSeamMesh) of all 428
active clipmap nodes one camera selects (LOD 0-5, caves density), from their
seam nodes as the batch meshing left them in device memory (its own JSON line, impl "lvn-seams"; the
reference arm times the oracle's octree construction and contouring on all
host threads).
`--workload collapse`: the engine's edge-collapse simplification
(ngMeshSimplifier) of the same 428 meshes, each with its node's options as
ConstructClipmapNodeData sets them (its own JSON line, impl "lvn-collapse";
the reference arm times the oracle's simplifier on all host threads).
`--surrogate`: the surrogate leg alone, on the 1024-chunk clipmap set with
the 2D fBm density (its own JSON line, impl "lvn-surrogate").
"""
import argparse
import ctypes as C
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 129 * 1024 * 1024
METRIC = "64\u00b3 chunks meshed/sec on 1 GB300, plain vs learned-density at \u22640.05-voxel Hausdorff"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="lvn", choices=["lvn", "reference"])
    p.add_argument("--cpu-sample", type=int, default=0, help="chunks per CPU-baseline sample (0 = whole-workload passes for >= 10 s; reference arm: about 2 s per step)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true", help="keep the built-in persistent-grid shapes")
    p.add_argument("--surrogate", action="store_true",
                   help="learned-density run: train the surrogate (2^24 samples of the 2D fBm density, Adam), then "
                        "mesh the 1024-chunk clipmap set plain and with the surrogate")
    p.add_argument("--train-steps", type=int, default=20000)
    p.add_argument("--gate", type=float, default=0.5, help="surrogate probe gate (voxels of each chunk)")
    p.add_argument("--mesh-chunks", type=int, default=0, help="surrogate run: mesh only the first N chunks (0 = all)")
    p.add_argument("--simplify", type=float, default=None,
                   help="octree simplification QEF-error threshold (voxel^2); default 0.05 for the clipmap "
                        "workload, off otherwise; < 0 = off")
    p.add_argument("--workload", default="sweep",
                   choices=["sweep", "tiled", "clipmap", "one", "select", "seams", "collapse"],
                   help="sweep: 4096 chunks over LOD 0-5, caves + 64 CSG ops, plain and surrogate (default); "
                        "tiled: 128 LOD0 chunks + 32 CSG ops; clipmap: 1024 chunks over LOD 0-4 with "
                        "3D caves; one: a single LOD0 chunk; select: clipmap node selection for 4096 cameras; "
                        "seams: the seam meshes of one camera's clipmap; collapse: the engine's edge-collapse "
                        "simplification of that clipmap's meshes")
    p.add_argument("--no-surrogate", action="store_true", help="sweep: skip the learned-density leg")
    p.add_argument("--inflight", type=int, default=3,
                   help="batches in flight on as many contexts for the pipelined end-to-end figure (>= 2)")
    p.add_argument("--chunks", type=int, default=0,
                   help="mesh only the workload's first N chunks (0 = all; for small profiler captures)")
    p.add_argument("--hermite-form", type=int, default=0, choices=[0, 1, 2],
                   help="LVN_OPT_HERMITE_FORM: 0 = by batch size, 1 = shared-memory tables, 2 = global tables "
                        "(so that a small capture can profile the form a large batch takes)")
    return p.parse_args()


def interval_summary(stamps):
    """min / median / max of the host-clock gaps between consecutive batch
    completions of the pipelined run (a diagnostic of its steadiness)."""
    gaps = [1e3 * (b - a) for a, b in zip(stamps, stamps[1:])]
    if not gaps:
        return None
    return {"min": round(min(gaps), 3), "median": round(statistics.median(gaps), 3), "max": round(max(gaps), 3),
            "all": [round(g, 2) for g in gaps]}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, world, device):
    """Each figure's maximum over the ranks (an all-reduce MAX over the
    process group; the identity for one rank): the replicas' step time is the
    slowest rank's."""
    if world <= 1:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def replicas_rate(world, chunks_per_rank, ms):
    """Whole-job chunks/s of `world` independent replicas, each meshing
    `chunks_per_rank` chunks a step, from the slowest rank's step time."""
    return world * chunks_per_rank / (ms / 1e3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


WORKLOAD = "sweep"
CHUNKS = 0


def simplify_threshold(args):
    if args.simplify is not None:
        return args.simplify
    return 0.05 if WORKLOAD == "clipmap" else -1.0


def simp_name(thr):
    return f"octree QEF error <= {thr} voxel^2" if thr >= 0 else None


def workload():
    wl = _workload()
    if CHUNKS and CHUNKS < len(wl.chunks):
        from leven_gb300 import workloads as W

        wl = W.Workload(f"{wl.name}-first{CHUNKS}", wl.chunks[:CHUNKS], wl.ops, wl.density, wl.noise_seed,
                        wl.voxels_per_chunk)
    return wl


def _workload():
    from leven_gb300 import workloads as W

    if WORKLOAD == "sweep":
        return W.clipmap_sweep()
    if WORKLOAD == "clipmap":
        return W.clipmap_caves()
    if WORKLOAD == "one":
        return W.plain_one_chunk()
    return W.tiled_csg()


def density_name(wl):
    d = wl.density
    if d["mode"] == 2:
        return f"fbm2d-{d['octaves2']}oct + caves fbm3d-{d['octaves3']}oct, seed {wl.noise_seed}"
    if d["mode"] == 1:
        return f"fbm2d-{d['octaves2']}oct, seed {wl.noise_seed}"
    return f"reference terrain, seed {wl.noise_seed}"


def lod_range(wl):
    lods = sorted({(s // 256).bit_length() - 1 for _, s in wl.chunks})
    return lods[0] if len(lods) == 1 else f"{lods[0]}-{lods[-1]}"


class CpuBaseline:
    """The oracle (CPU restatement of the reference algorithm) meshing chunks of
    the workload on `threads` host threads, one orc_mesh_chunks call per pass."""

    def __init__(self, wl, threads, simplify=-1.0):
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as O
        from leven_gb300 import workloads as W

        O.build()
        O.set_seed(wl.noise_seed)
        self.O, self.threads, self.n, self.simplify = O, threads, len(wl.chunks), simplify
        d = wl.density
        self.dens = O.density(mode=d["mode"], octaves2=d["octaves2"], freq2=d["freq2"], lac2=d["lacunarity2"],
                              gain2=d["gain2"], amp2=d["amp2"], octaves3=d.get("octaves3", 6),
                              freq3=d.get("freq3", 1.0 / 64), lac3=d.get("lacunarity3", 2.0),
                              gain3=d.get("gain3", 0.5), amp3=d.get("amp3", 12.0))
        self.args = (O.ChunkArgs * self.n)()
        self.keep = []
        for j, (mn, size) in enumerate(wl.chunks):
            mine = W.ops_for_chunk(wl.ops, mn, size)
            ops = O.make_ops([op.as_tuple() for op in mine])
            self.keep.append(ops)
            self.args[j] = O.ChunkArgs((C.c_int32 * 3)(*mn), size, wl.voxels_per_chunk, 0, 0, len(mine),
                                       C.cast(ops, C.POINTER(O.CsgOp)), 5489)

    def run(self, count):
        """Mesh `count` chunks spread evenly over the workload; returns seconds."""
        if count >= self.n:
            arr, m = self.args, self.n
        else:
            arr = (self.O.ChunkArgs * count)()
            for j in range(count):
                arr[j] = self.args[int(j * self.n / count)]
            m = count
        t0 = time.perf_counter()
        self.O.lib().orc_mesh_chunks_simplified(C.byref(self.dens), arr, m, self.threads, self.simplify)
        return time.perf_counter() - t0

    def rate(self, target_s):
        """Whole-workload passes until at least target_s seconds of CPU work."""
        done, total = 0, 0.0
        while total < target_s:
            total += self.run(self.n)
            done += self.n
        return done / total, total, done

    def step_chunks(self, step_s):
        """Chunks one step of about step_s seconds meshes (calibrated on a small sample)."""
        m = min(self.n, max(self.threads, 16))
        r = m / self.run(m)
        return int(min(self.n, max(self.threads, r * step_s)))


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if WORKLOAD == "select":
        return run_select_reference(args)
    if WORKLOAD == "seams":
        return run_seams_reference(args)
    if WORKLOAD == "collapse":
        return run_collapse_reference(args)
    wl = workload()
    threads = host_threads()
    cb = CpuBaseline(wl, threads, simplify_threshold(args))
    sample = args.cpu_sample or cb.step_chunks(2.0)
    vals = []
    for _ in range(args.warmup):
        cb.run(min(sample, threads))
    for _ in range(args.steps):
        vals.append(sample / cb.run(sample))
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "chunks/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sample / value, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "chunks_per_step": sample, "voxels_per_chunk": 64, "csg_ops": len(wl.ops),
                   "density": density_name(wl), "simplify": simp_name(simplify_threshold(args)),
                   "sample": f"{sample} of {len(wl.chunks)} chunks per step"},
        "cpu_baseline": {"value": round(value, 3), "unit": "chunks/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} chunks of the {len(wl.chunks)}-chunk workload per step"},
        "e2e": {"value": round(value, 3), "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# algorithmic work per stage, used for the roofline of the dominant kernel
def stage_work(stage, res, n_chunks, vpc=64):
    F = (vpc + 2) ** 3
    C3 = vpc ** 3
    E = int(res[:, 6].sum())
    V = int(res[:, 7].sum())
    T = int(res[:, 3].sum()) // 2
    S = int(res[:, 5].sum())
    nbytes = {
        "field": 2 * F * n_chunks,                              # corner words written
        "edge_count": 2 * F * n_chunks,                         # corner words read
        "edge_scatter": 2 * F * n_chunks + 8 * E,               # corners read, keys + chunk ids written
        "vox_count": 2 * F * n_chunks,
        "vox_scatter": 2 * F * n_chunks + 12 * V,
        "leaf": 12 * V + 16 * E + 48 * V,                       # codes/info/chunk, hermite, vertices
        "mesh_count": 12 * V + 48 * V,                          # codes/info/chunk in, quad scratch out
        "mesh_scatter": 48 * V + 12 * V + 24 * T + 48 * S,
        "hash_fill": 8 * (2 * E + 2 * V),
        "edge_insert": 8 * E + 16 * E,
        "node_insert": 8 * V + 16 * V,
    }
    return nbytes.get(stage)


def run_lvn(args):
    import numpy as np
    import torch

    import leven_gb300 as lvn

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    wl = workload()
    rc = lvn.initialise(wl.noise_seed, 0, 2)
    lvn.set_density(**wl.density)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    mg = lvn.MeshGen(wl.voxels_per_chunk)
    mg.set_option(lvn.LVN_OPT_CACHE, 0)
    mg.set_option(lvn.LVN_OPT_HERMITE_FORM, args.hermite_form)
    simp = simplify_threshold(args)
    if simp >= 0:
        mg.set_simplify(simp)
    stream = torch.cuda.ExternalStream(mg.stream(), device=dev)
    n = len(wl.chunks)
    descs = (lvn.ChunkDesc * n)()
    for i, (mn, size) in enumerate(wl.chunks):
        descs[i] = lvn.ChunkDesc((C.c_int32 * 3)(*mn), size)
    results = (lvn.ChunkResult * n)()

    # launch shapes for this batch (outside the timed region, like a compile)
    tuned = None if args.no_autotune else mg.autotune(wl.chunks)
    # size the outputs once from a first run
    _, _, _, res = mg.generate_chunks(wl.chunks)
    tot_v = int(res[:, 7].sum())
    tot_t = int(res[:, 3].sum())
    tot_s = int(res[:, 5].sum())
    cap_v, cap_t, cap_s = tot_v + 1024, tot_t + 2048, tot_s + 1024
    d_vert = torch.empty(cap_v * 12, dtype=torch.float32, device=dev)
    d_tri = torch.empty(cap_t * 3, dtype=torch.int32, device=dev)
    d_seam = torch.empty(cap_s * 12, dtype=torch.int32, device=dev)
    h_vert = torch.empty(cap_v * 12, dtype=torch.float32).pin_memory()
    h_tri = torch.empty(cap_t * 3, dtype=torch.int32).pin_memory()
    h_seam = torch.empty(cap_s * 12, dtype=torch.int32).pin_memory()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)

    def batch_out(device_mem):
        if device_mem:
            return lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, d_vert.data_ptr(), cap_v, 0, d_tri.data_ptr(), cap_t, 0,
                                d_seam.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
        return lvn.BatchOut(lvn.LVN_MEMORY_HOST, h_vert.data_ptr(), cap_v, 0, h_tri.data_ptr(), cap_t, 0,
                            h_seam.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))

    def step(device_mem):
        bo = batch_out(device_mem)
        r = mg.generate_chunks_raw(descs, n, bo)
        if r != 0:
            raise lvn.LvnError(r, "generate_chunks")
        return bo

    def timed(device_mem, steps, warmup):
        for _ in range(warmup):
            step(device_mem)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        times = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)  # evict the previous step from L2 (outside the events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bo = step(device_mem)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return times, bo

    # end to end with batches in flight: further contexts, each with its own
    # stream and pinned host arrays; while one batch's outputs cross to the
    # host, the next batches' kernels run (lvn_meshgen_generate_chunks_async).
    # With three in flight a batch's transfer may take up to twice a batch's
    # kernel time before the next submission on its context waits for it.
    extra = []
    for _ in range(max(2, args.inflight) - 1):
        mgx = lvn.MeshGen(wl.voxels_per_chunk)
        mgx.set_option(lvn.LVN_OPT_CACHE, 0)
        mgx.set_option(lvn.LVN_OPT_HERMITE_FORM, args.hermite_form)
        # copy-engine transfers, so that a batch's transfer leaves the SMs to the others' kernels
        mgx.set_option(lvn.LVN_OPT_HOST_WRITES, 0)
        # the contexts' kernels run batch after batch; only transfers overlap kernels
        mgx.set_option(lvn.LVN_OPT_COMPUTE_ORDER, 1)
        if simp >= 0:
            mgx.set_simplify(simp)
        # the tuned shapes are process-wide: every context runs those the
        # first context's autotuning chose
        resx = (lvn.ChunkResult * n)()
        hv = torch.empty(cap_v * 12, dtype=torch.float32).pin_memory()
        ht = torch.empty(cap_t * 3, dtype=torch.int32).pin_memory()
        hs = torch.empty(cap_s * 12, dtype=torch.int32).pin_memory()
        bo = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), cap_t, 0,
                          hs.data_ptr(), cap_s, 0, C.cast(resx, C.POINTER(lvn.ChunkResult)))
        extra.append((mgx, torch.cuda.ExternalStream(mgx.stream(), device=dev), bo, (resx, hv, ht, hs)))
    ctxs = [(mg, stream)] + [(x[0], x[1]) for x in extra]
    bo_pipe = [batch_out(False)] + [x[2] for x in extra]
    inflight = len(ctxs)

    done_at = []  # host clock when each timed batch's wait returned (diagnostics only)

    def pipelined(steps, warmup):
        def run(count, stamps=None):
            for k in range(count):
                c, _ = ctxs[k % inflight]
                if k >= inflight:
                    r = c.wait()
                    if r != 0:
                        raise lvn.LvnError(r, "generate_chunks_async")
                    if stamps is not None:
                        stamps.append(time.perf_counter())
                r = c.generate_chunks_async_raw(descs, n, bo_pipe[k % inflight])
                if r != 0:
                    raise lvn.LvnError(r, "generate_chunks_async")
            for j in range(inflight):
                c, _ = ctxs[(count + j) % inflight]
                r = c.wait()
                if r != 0:
                    raise lvn.LvnError(r, "generate_chunks_async")
                if stamps is not None:
                    stamps.append(time.perf_counter())
        mg.set_option(lvn.LVN_OPT_HOST_WRITES, 0)
        mg.set_option(lvn.LVN_OPT_COMPUTE_ORDER, 1)
        run(warmup)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _, sx in ctxs[1:]:
            sx.wait_event(e0)
        run(steps, done_at)
        for _, sx in ctxs[1:]:
            eb = torch.cuda.Event()
            eb.record(sx)
            stream.wait_event(eb)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        mg.set_option(lvn.LVN_OPT_HOST_WRITES, 1)
        mg.set_option(lvn.LVN_OPT_COMPUTE_ORDER, 0)
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / steps

    with ClockSampler(local) as clocks:
        t_dev, bo_dev = timed(True, args.steps, args.warmup)
        t_e2e, bo_host = timed(False, args.steps, max(3, args.warmup // 2))
        # two untimed rounds over the contexts: each has run its batch graph twice
        ms_pipe = pipelined(args.steps, max(2 * inflight, args.warmup))
    ms = sum(t_dev) / len(t_dev)
    ms_single = sum(t_e2e) / len(t_e2e)
    for x in extra:
        x[0].close()
    ms, ms_single, ms_pipe = max_over_ranks([ms, ms_single, ms_pipe], world, dev)
    value = replicas_rate(world, n, ms)
    ms_e2e = ms_pipe
    e2e = replicas_rate(world, n, ms_e2e)
    e2e_single = replicas_rate(world, n, ms_single)

    # per-stage device times (profiled pass, synchronising between stages)
    mg.reset_stage_times()
    mg.set_option(lvn.LVN_OPT_PROFILE, 1)
    prof_steps = 5
    for _ in range(prof_steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        step(True)
    mg.set_option(lvn.LVN_OPT_PROFILE, 0)
    stages = mg.stage_times()
    res_np = np.ctypeslib.as_array(C.cast(results, C.POINTER(C.c_int32)), shape=(n, 8)).copy()
    launched = {k: v[1] // prof_steps for k, v in stages.items() if v[1]}
    gpu_launches = (sum(launched.values()) + 1) * args.steps  # + the per-batch state reset kernel

    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dominant = max((k for k in stages if stages[k][1]), key=lambda k: stages[k][0])
    dom_ms = stages[dominant][0] / stages[dominant][1]
    stage_ms = {k: round(v[0] / v[1], 4) for k, v in stages.items() if v[1]}
    E = int(res_np[:, 6].sum())
    traffic = None  # no profiler inside the timed run; a committed ncu figure is quoted separately
    traffic_note = committed_traffic(dominant)
    df = density_flops(wl)
    if dominant in ("hermite", "field") and df is not None and (dominant == "hermite" or wl.density["mode"] == 2):
        # FP32 issue-rate roofline: SMs x 128 lanes x 2 flop x clock
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        clk = (clocks.summary()["sm_mhz"] or peaks.get("clocks_under_load", {}).get("sm_mhz_median", 1477.0))
        fp32_peak = sms * 128 * 2 * clk * 1e6 / 1e12
        if dominant == "hermite":
            fxz, fy = hermite_edge_flops(*df)
            nxz, ny = edge_axis_counts(mg, lvn, n)
            flops = nxz * fxz + ny * fy
        else:  # every field point of every chunk: the height per column, the cave term per point
            fd = wl.voxels_per_chunk + 2
            flops = n * (fd * fd * df[0] + fd ** 3 * df[1])
        ach = flops / (dom_ms / 1e3) / 1e12
        roof = {"bound": "fp32", "achieved": round(ach, 3), "peak": round(fp32_peak, 2),
                "unit": "TFLOP/s", "frac": round(ach / fp32_peak, 4), "traffic": traffic,
                "traffic_from_profile": traffic_note,
                "kernel": dominant, "ms_per_launch": round(dom_ms, 4), "peak_source": f"SMs x 128 x 2 x {clk} MHz",
                "flop_per_launch": int(flops)}
    else:
        b = stage_work(dominant, res_np, n)
        ach = b / (dom_ms / 1e3) / 1e9 if b else None
        roof = {"bound": "hbm", "achieved": round(ach, 1) if ach else None, "peak": hbm_peak, "unit": "GB/s",
                "frac": round(ach / hbm_peak, 4) if ach else None, "traffic": traffic,
                "traffic_from_profile": traffic_note, "kernel": dominant,
                "ms_per_launch": round(dom_ms, 4), "peak_source": peak_src}

    bo = bo_host
    h2d = C.sizeof(lvn.ChunkDesc) * n + 48 * len(wl.ops)  # descriptors + stored operations per chunk (upper bound)
    d2h = 80 * n + 48 * bo.total_vertices + 12 * bo.total_triangles + 48 * bo.total_seams

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "step_ms": {"min": round(min(t_dev), 4), "median": round(statistics.median(t_dev), 4),
                    "max": round(max(t_dev), 4)},
        "config": {"workload": wl.name, "chunks_per_step": n, "voxels_per_chunk": wl.voxels_per_chunk,
                   "csg_ops": len(wl.ops), "density": density_name(wl), "lod": lod_range(wl),
                   "simplify": simp_name(simp), "leaf_vertices": int(res_np[:, 7].sum()),
                   "launch_shapes": {"autotuned_ctas_per_sm": tuned} if tuned else "built-in",
                   "hermite_form": ["by batch size", "shared-memory tables", "global tables"][args.hermite_form],
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed between steps (256 MiB write) for value and the single-call e2e; the pipelined "
                         "e2e's batches touch far more than L2 (several GB each)",
                   "vertices": int(bo.total_vertices), "triangles": int(bo.total_triangles),
                   "edges": E, "seams": int(bo.total_seams)},
        "e2e": {"value": round(e2e, 2), "unit": "chunks/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(ms_e2e, 4),
                "mode": f"pinned host outputs moved by the copy engine (LVN_OPT_HOST_WRITES 0); {inflight} "
                        "contexts, a batch in flight on each (lvn_meshgen_generate_chunks_async), their kernels in "
                        "one device-wide order (LVN_OPT_COMPUTE_ORDER 1) so that one batch's transfer overlaps the "
                        "next batches' kernels; CUDA events from the first batch's start to the last one's end "
                        "over all the streams",
                "batches_in_flight": inflight,
                "completion_interval_ms": interval_summary(done_at),
                "single_call": {"value": round(e2e_single, 2), "ms_per_step": round(ms_single, 4),
                                "mode": "one synchronous lvn_meshgen_generate_chunks call per step, the kernels "
                                        "writing the pinned host arrays (LVN_OPT_HOST_WRITES 1)"}},
        "gpu_launches": int(gpu_launches),
        "roofline": roof,
        "stage_ms": stage_ms,
        "clocks": clocks.summary(),
    }
    # achieved HBM bandwidth of each memory-bound stage: its algorithmic bytes
    # (stage_work) over its profiled time, against the measured copy peak
    stage_gbs = {}
    for k, ms_k in stage_ms.items():
        b = stage_work(k, res_np, n)
        if b and ms_k > 0:
            gbs = b / (ms_k / 1e3) / 1e9
            stage_gbs[k] = {"gbs": round(gbs, 1), "frac": round(gbs / hbm_peak, 4), "bytes": int(b)}
    line["stage_gbs"] = stage_gbs
    line["stage_gbs_peak"] = {"hbm_gbs": hbm_peak, "source": peak_src}
    # density samples a step determines: every field point of every chunk, and
    # the 23 evaluations (17 search + 6 normal) of each plain edge's hermite data
    nxz, ny = edge_axis_counts(mg, lvn, n) if n <= 8192 else (0, 0)
    samples = n * (wl.voxels_per_chunk + 2) ** 3 + 23 * (nxz + ny)
    line["density_samples_per_s"] = round(samples / (ms / 1e3), 1)
    line["density_samples_per_step"] = int(samples)
    # the FP32 leaf solve against an FP64 solve of the same crossings, over
    # every leaf of the last (device-output) step: a GPU measurement pass
    step(True)
    qmax, qmean, qleaves, qfar = mg.qef_fp64_error()
    line["qef_fp64"] = {"max_voxels": qmax, "mean_voxels": qmean, "leaves": qleaves,
                        "leaves_beyond_1e-3_voxel": qfar,
                        "what": "|x_fp32 - x_fp64| of each leaf vertex, in its chunk's voxels"}
    if rank == 0 and WORKLOAD == "sweep" and not args.no_surrogate:
        line["surrogate"] = surrogate_leg(args, wl, mg, descs, results, value, stream, flush, local)
    if rank == 0 and not args.no_cpu_baseline:
        threads = host_threads()
        cb = CpuBaseline(wl, threads, simp)
        if args.cpu_sample or n > 1024:
            # a bounded sample: about 12 s of CPU work spread over the workload
            m = min(args.cpu_sample or cb.step_chunks(12.0), n)
            dt = cb.run(m)
            v = m / dt
            what = f"{m} chunks spread evenly over the {n}-chunk workload, {dt:.1f} s"
        else:
            v, dt, m = cb.rate(10.0)
            what = f"{m // n} passes over the {n}-chunk workload ({m} chunks), {dt:.1f} s"
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "chunks/s", "cores": threads, "kind": "port",
                                "sample": what}
    if rank == 0:
        print(json.dumps(line), flush=True)
    mg.close()
    if world > 1:
        torch.distributed.destroy_process_group()


PROFILE_TAG = {"tiled": "tiled_csg_128", "clipmap": "clipmap_caves_1024", "one": "one_chunk",
               "select": "select_4096", "seams": "clipmap_frame_428", "sweep": "clipmap_sweep_4096"}


def committed_traffic(kernel):
    """DRAM bytes per launch of `kernel` on this workload as a committed ncu
    summary states them (profiles/<kernel>_<workload>.md, the table row
    `dram_bytes_per_launch`), with the file: a figure from an earlier capture,
    not a measurement of this run."""
    if CHUNKS:
        return None
    path = ROOT / "profiles" / f"{kernel}_{PROFILE_TAG.get(WORKLOAD, WORKLOAD)}.md"
    try:
        for line in path.read_text().splitlines():
            if "dram_bytes_per_launch" in line:
                return {"dram_bytes_per_launch": int(line.split("|")[2].strip()),
                        "file": str(path.relative_to(ROOT))}
    except (OSError, ValueError, IndexError):
        pass
    return None


# FP32 operations of the restated density arithmetic, as the oracle counts
# them (orc_flop_counts: add, sub, mul, div, sqrt and floor 1, an fma 2,
# compares, min / max and abs free, every simplex corner taken;
# tests/test_flop_counts.py holds these figures to that count):
# one simplex2 evaluation 51, one octave of 2D fBm 56, the 8-octave height
# term 8 * 56 + 4 = 452; one simplex3 evaluation 93, one octave of 3D fBm 99,
# the 6-octave cave term 6 * 99 + 3 = 597 plus its fma; y - amp h is one fma.
FLOP_HEIGHT8 = 452
FLOP_CAVES6 = 597 + 2
# FindEdgeIntersectionInfo outside its 23 density samples: the edge vector,
# 17 search positions (3 fmas and the parameter step each), the crossing
# (3 fmas), six normal offsets, three differences and the normalisation
FLOP_EDGE_EXTRA = 146


def density_flops(wl):
    """(per-column height term, rest of a density sample) FP32 operations, or None."""
    d = wl.density
    if d["mode"] == 1 and d["octaves2"] == 8:
        return FLOP_HEIGHT8, 2
    if d["mode"] == 2 and d["octaves2"] == 8 and d["octaves3"] == 6:
        return FLOP_HEIGHT8, 2 + FLOP_CAVES6
    return None


def hermite_edge_flops(h, p):
    """The operations k_hermite performs for a plain edge: 23 density samples
    (the rest p each) and the edge arithmetic, plus the height terms it
    evaluates: an x or z edge 15 (its end points' heights come from the
    field's height map) and 4 for the x and z normal samples; a y edge the 4
    normal heights only (its own height is the map's, and the y normal pair
    shares it)."""
    xz = 19 * h + 23 * p + FLOP_EDGE_EXTRA
    y = 4 * h + 23 * p + FLOP_EDGE_EXTRA
    return xz, y


def edge_axis_counts(mg, lvn, n):
    """Plain x/z and y edge counts of the last batch (CSG-created edges excluded)."""
    import numpy as np

    nxz = ny = 0
    for c in range(n):
        keys = mg.debug_fetch(lvn.DEBUG_EDGE_KEYS, c, np.int32)
        plain = mg.debug_fetch(lvn.DEBUG_PLAIN_EDGES, c, np.int32, max_elems=1)
        axes = keys[:plain] & 3
        ny += int((axes == 1).sum())
        nxz += int(plain - (axes == 1).sum())
    return nxz, ny


def hausdorff_voxels(va, vb, voxel):
    """Symmetric Hausdorff distance between two vertex sets, in voxels."""
    from scipy.spatial import cKDTree

    if len(va) == 0 or len(vb) == 0:
        return None
    d1 = cKDTree(vb).query(va)[0].max()
    d2 = cKDTree(va).query(vb)[0].max()
    return float(max(d1, d2)) / voxel


def surrogate_leg(args, wl, mg, descs, results, plain_value, stream, flush, gpu_index):
    """The learned density on the sweep: sample 2^24 fresh plain samples of
    the workload's density over the chunk set's x / z extent (y in [-128,
    128], extrapolated beyond), train 20k Adam steps at batch 65,536 on the
    tensor cores, then mesh the same chunks with the surrogate under its
    per-chunk probe gate (in voxels of each chunk); plain and surrogate meshes
    of every surrogate chunk are compared by symmetric Hausdorff distance."""
    import numpy as np
    import torch

    import leven_gb300 as lvn

    n = len(wl.chunks)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    lo = [min(mn[i] for mn, _ in wl.chunks) / 4.0 for i in range(3)]
    hi = [max(mn[i] + s for mn, s in wl.chunks) / 4.0 for i in range(3)]
    lo[1], hi[1] = -128.0, 128.0
    sur = lvn.Surrogate(tuple(lo), tuple(hi), seed=1)
    t0 = time.perf_counter()
    sur.sample(1 << 24, seed=1)
    t_sample = time.perf_counter() - t0
    steps = args.train_steps
    t0 = time.perf_counter()
    losses = sur.train(steps, batch=65536, lr=1e-3)
    t_train = time.perf_counter() - t0
    train_flop = 3 * 2 * (96 * 128 + 3 * 128 * 128 + 128) * 65536 * steps
    train_tflops = train_flop / t_train / 1e12
    sustained = peaks.get("bf16_tflops_sustained")

    # plain meshes of this batch (host copies), then the surrogate's
    Vp, Tp, Sp, resp = mg.generate_chunks(wl.chunks)
    mg.set_surrogate(sur, args.gate)
    try:
        Vs, Ts, Ss, ress = mg.generate_chunks(wl.chunks)
        use = mg.surrogate_chunks(n)
        cap_v = max(int(resp[:, 7].sum()), int(ress[:, 7].sum())) + 1024
        cap_t = max(Tp.shape[0], Ts.shape[0]) + 4096
        cap_s = max(Sp.shape[0], Ss.shape[0]) + 1024
        d_vert = torch.empty(cap_v * 12, dtype=torch.float32, device="cuda")
        d_tri = torch.empty(cap_t * 3, dtype=torch.int32, device="cuda")
        d_seam = torch.empty(cap_s * 12, dtype=torch.int32, device="cuda")
        bo = lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, d_vert.data_ptr(), cap_v, 0, d_tri.data_ptr(), cap_t, 0,
                          d_seam.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
        for _ in range(max(3, args.warmup // 2)):
            assert mg.generate_chunks_raw(descs, n, bo) == 0
        torch.cuda.synchronize()
        ts = []
        with ClockSampler(gpu_index) as clocks:
            for _ in range(max(3, args.steps // 2)):
                with torch.cuda.stream(stream):
                    flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                assert mg.generate_chunks_raw(descs, n, bo) == 0
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
        ms_sur = sum(ts) / len(ts)
        # the gate swept: fallback rate against mesh Hausdorff distance (up to
        # 256 surrogate chunks spread over those a gate lets through)
        gate_sweep = []
        for gate in (0.5, 1.0, 2.0, 4.0, 8.0, 16.0, 32.0):
            mg.set_surrogate(sur, gate)
            Vg, Tg, Sg, resg = mg.generate_chunks(wl.chunks)
            ug = np.flatnonzero(mg.surrogate_chunks(n))
            pick = ug[np.linspace(0, len(ug) - 1, min(len(ug), 256)).astype(int)] if len(ug) else ug
            hg = []
            for c in pick:
                rp, rs = resp[c], resg[c]
                h = hausdorff_voxels(Vp[rp[0]:rp[0] + rp[1], :3], Vg[rs[0]:rs[0] + rs[1], :3],
                                     4.0 * wl.chunks[c][1] / 256)
                if h is not None:
                    hg.append(h)
            gate_sweep.append({"gate_voxels": gate, "fallback_rate": round(1 - len(ug) / n, 4),
                               "hausdorff_voxels_mean": round(float(np.mean(hg)), 4) if hg else None,
                               "hausdorff_voxels_max": round(float(np.max(hg)), 4) if hg else None,
                               "hausdorff_chunks": len(hg)})
            del Vg, Tg, Sg
    finally:
        mg.set_surrogate(None)
    hd = []
    for c in np.flatnonzero(use):
        rp, rs = resp[c], ress[c]
        voxel = 4.0 * wl.chunks[c][1] / 256  # world units per voxel of this chunk
        h = hausdorff_voxels(Vp[rp[0]:rp[0] + rp[1], :3], Vs[rs[0]:rs[0] + rs[1], :3], voxel)
        if h is not None:
            hd.append(h)
    # density error against the plain FP32 density and the FP64 density, on
    # fresh samples
    pts = sur.sample(1 << 16, seed=99, fetch=True)
    d_sur = sur.eval(pts)
    d64 = lvn.density_f64(pts)
    err = np.abs(d_sur - pts[:, 3])
    err64 = np.abs(d_sur - d64)
    lods = np.array([(s // 256).bit_length() - 1 for _, s in wl.chunks])
    on = use.astype(bool)
    samples_sur = int(on.sum()) * (wl.voxels_per_chunk + 2) ** 3 + 512 * n
    sur.close()
    hd_a = np.array(hd) if hd else np.zeros(0)
    return {
        "value": round(n / (ms_sur / 1e3), 2), "unit": "chunks/s", "ms_per_step": round(ms_sur, 3),
        "vs_plain": round(n / (ms_sur / 1e3) / plain_value, 4),
        "gate_voxels": args.gate, "chunks_on_surrogate": int(on.sum()), "fallback_rate": round(1 - on.sum() / n, 4),
        "on_surrogate_by_lod": {str(k): int((on & (lods == k)).sum()) for k in sorted(set(lods.tolist()))},
        "hausdorff_voxels_mean": round(float(hd_a.mean()), 4) if hd else None,
        "hausdorff_voxels_max": round(float(hd_a.max()), 4) if hd else None,
        "chunks_within_bar": int(((hd_a <= 0.5)).sum()) if hd else 0,
        "density_samples_per_s": round(samples_sur / (ms_sur / 1e3), 1),
        "density_abs_err_mean": float(err.mean()), "density_abs_err_p99": float(np.quantile(err, 0.99)),
        "density_abs_err_vs_fp64_mean": float(err64.mean()),
        "density_abs_err_vs_fp64_p99": float(np.quantile(err64, 0.99)),
        "plain_fp32_abs_err_vs_fp64_max": float(np.abs(pts[:, 3] - d64).max()),
        "train": {"samples": 1 << 24, "steps": steps, "batch": 65536, "lr": 1e-3, "sample_s": round(t_sample, 2),
                  "train_s": round(t_train, 2), "network_tflops": round(train_tflops, 2),
                  "tensor_frac_of_sustained_bf16": round(train_tflops / sustained, 4) if sustained else None,
                  "loss_first": float(losses[0]) if len(losses) else None,
                  "loss_last100": float(np.mean(losses[-100:])) if len(losses) else None},
        "domain": [lo, hi], "clocks": clocks.summary(), "gate_sweep": gate_sweep,
    }


def run_surrogate(args):
    """Plain vs learned-density meshing of the clipmap chunk set (LOD 0-4)
    with the 2D fBm density the surrogate is trained on."""
    import numpy as np
    import torch

    import leven_gb300 as lvn
    from leven_gb300 import workloads as W

    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    chunks = W.clipmap_caves().chunks
    if args.mesh_chunks:
        chunks = chunks[:args.mesh_chunks]
    lvn.initialise(1, 0, 2)
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    lo, hi = (-1024.0, -128.0, -1024.0), (1024.0, 128.0, 1024.0)
    sur = lvn.Surrogate(lo, hi, seed=1)
    t0 = time.perf_counter()
    sur.sample(1 << 24, seed=1)
    t_sample = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = sur.train(args.train_steps, batch=65536, lr=1e-3)
    t_train = time.perf_counter() - t0
    train_flop = 3 * 2 * (96 * 128 + 3 * 128 * 128 + 128) * 65536 * args.train_steps

    n = len(chunks)
    descs = (lvn.ChunkDesc * n)()
    for i, (mn, size) in enumerate(chunks):
        descs[i] = lvn.ChunkDesc((C.c_int32 * 3)(*mn), size)
    results = (lvn.ChunkResult * n)()
    mg = lvn.MeshGen(64)
    mg.set_option(lvn.LVN_OPT_CACHE, 0)
    stream = torch.cuda.ExternalStream(mg.stream(), device=dev)
    Vp, Tp, Sp, resp = mg.generate_chunks(chunks)
    mg.set_surrogate(sur, args.gate)  # the surrogate's meshes size the outputs too
    Vs, Ts, Ss, ress = mg.generate_chunks(chunks)
    use = mg.surrogate_chunks(n)
    mg.set_surrogate(None)
    cap_v = max(int(resp[:, 7].sum()), int(ress[:, 7].sum())) + 1024
    cap_t = max(Tp.shape[0], Ts.shape[0]) + 4096
    cap_s = max(Sp.shape[0], Ss.shape[0]) + 1024
    d_vert = torch.empty(cap_v * 12, dtype=torch.float32, device=dev)
    d_tri = torch.empty(cap_t * 3, dtype=torch.int32, device=dev)
    d_seam = torch.empty(cap_s * 12, dtype=torch.int32, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)

    def timed(steps, warmup):
        bo = lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, d_vert.data_ptr(), cap_v, 0, d_tri.data_ptr(), cap_t, 0,
                          d_seam.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
        for _ in range(warmup):
            assert mg.generate_chunks_raw(descs, n, bo) == 0
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert mg.generate_chunks_raw(descs, n, bo) == 0
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return sum(ts) / len(ts)

    with ClockSampler(local) as clocks:
        ms_plain = timed(args.steps, args.warmup)
        mg.set_surrogate(sur, args.gate)
        ms_sur = timed(args.steps, args.warmup)
    hd = []
    for c in np.flatnonzero(use):
        rp, rs = resp[c], ress[c]
        voxel = 4.0 * chunks[c][1] / 256  # world units per voxel of this chunk
        h = hausdorff_voxels(Vp[rp[0]:rp[0] + rp[1], :3], Vs[rs[0]:rs[0] + rs[1], :3], voxel)
        if h is not None:
            hd.append(h)
    # density error of the surrogate against the plain FP32 density and against
    # the FP64 density, on fresh samples
    pts = sur.sample(1 << 16, seed=99, fetch=True)
    d_sur = sur.eval(pts)
    d64 = lvn.density_f64(pts)
    err = np.abs(d_sur - pts[:, 3])
    err64 = np.abs(d_sur - d64)
    err32_64 = np.abs(pts[:, 3] - d64)
    line = {
        "metric": "64^3 chunks meshed/sec on 1 GB300, plain vs learned density", "impl": "lvn-surrogate",
        "value": round(n / (ms_sur / 1e3), 2), "plain": round(n / (ms_plain / 1e3), 2), "unit": "chunks/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_sur, 3),
        "plain_ms_per_step": round(ms_plain, 3), "higher_is_better": True, "dtype": "bf16/f32",
        "data": "synthetic", "clocks": clocks.summary(),
        "config": {"workload": f"clipmap-{n}chunks-lod0-4 with the 2D fBm density", "train_samples": 1 << 24,
                   "train_steps": args.train_steps, "batch": 65536, "lr": 1e-3, "gate": args.gate,
                   "domain": [lo, hi]},
        "surrogate": {"chunks_on_surrogate": int(use.sum()), "fallback_rate": round(1 - use.sum() / n, 4),
                      "train_s": round(t_train, 2), "sample_s": round(t_sample, 2),
                      "train_tflops": round(train_flop / t_train / 1e12, 2),
                      "loss_first": float(losses[0]) if len(losses) else None,
                      "loss_last100": float(np.mean(losses[-100:])) if len(losses) else None,
                      "density_abs_err_mean": float(err.mean()), "density_abs_err_p99": float(np.quantile(err, 0.99)),
                      "density_abs_err_vs_fp64_mean": float(err64.mean()),
                      "density_abs_err_vs_fp64_p99": float(np.quantile(err64, 0.99)),
                      "plain_fp32_abs_err_vs_fp64_max": float(err32_64.max()),
                      "hausdorff_voxels_mean": round(float(np.mean(hd)), 4) if hd else None,
                      "hausdorff_voxels_max": round(float(np.max(hd)), 4) if hd else None,
                      "chunks_within_0.05_mean_0.5_max": int(sum(h <= 0.5 for h in hd))},
    }
    print(json.dumps(line), flush=True)
    mg.close()
    sur.close()


SELECT_METRIC = "clipmap camera selections/sec on 1 GB300 (SelectActiveClipmapNodes, 2^15 root)"


class SelectBaseline:
    """The oracle's SelectActiveClipmapNodes recursion over the cameras on
    `threads` host threads (one orc_clipmap_select_many call per pass)."""

    def __init__(self, cams, threads):
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as O
        from leven_gb300 import workloads as W

        O.build()
        self.O, self.cams, self.threads, self.W = O, cams, threads, W

    def run(self):
        t0 = time.perf_counter()
        self.O.clipmap_select_many(self.cams, self.W.CLIPMAP_ROOT_MIN, self.W.CLIPMAP_ROOT_SIZE, self.threads)
        return time.perf_counter() - t0

    def rate(self, target_s):
        done, total = 0, 0.0
        while total < target_s:
            total += self.run()
            done += len(self.cams)
        return done / total, total, done


def run_select_reference(args):
    from leven_gb300 import workloads as W

    cams = W.clipmap_cameras()
    threads = host_threads()
    cb = SelectBaseline(cams, threads)
    for _ in range(args.warmup):
        cb.run()
    vals = [len(cams) / cb.run() for _ in range(args.steps)]
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": SELECT_METRIC, "value": round(value, 1), "unit": "cameras/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * len(cams) / value, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"clipmap-select-{len(cams)}cameras", "root_size": W.CLIPMAP_ROOT_SIZE},
        "cpu_baseline": {"value": round(value, 1), "unit": "cameras/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(cams)} cameras per step"},
        "e2e": {"value": round(value, 1), "unit": "cameras/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_select(args):
    """The clipmap's active-node selection for the 4096-camera workload: the
    device form (cameras resident, lists left in HBM) per step, and end to end
    through the host-buffer C-ABI call."""
    import numpy as np
    import torch

    import leven_gb300 as lvn
    from leven_gb300 import workloads as W

    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cams = W.clipmap_cameras()
    n = len(cams)
    rmin, rsize = W.CLIPMAP_ROOT_MIN, W.CLIPMAP_ROOT_SIZE
    stride = 1024
    d_cams = torch.from_numpy(cams).to(dev)
    d_out = torch.empty((n * stride, 4), dtype=torch.int32, device=dev)
    d_counts = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    for _ in range(max(args.warmup, 3)):
        lvn.clipmap_select_device(d_cams, rmin, rsize, d_out, stride, d_counts, stream=stream)
    torch.cuda.synchronize()
    counts = d_counts.cpu().numpy()
    assert (counts >= 0).all() and (counts <= stride).all(), "selection lists exceed the device stride"
    total_nodes = int(counts.sum())

    h_cams = torch.from_numpy(cams).pin_memory()
    h_out = torch.empty((total_nodes + 1024, 4), dtype=torch.int32).pin_memory()
    h_counts = np.zeros(n, np.int32)
    L = lvn.lib()

    def host_call():
        rc = L.lvn_clipmap_select(h_cams.data_ptr(), n, lvn._ivec3(rmin), rsize, h_out.data_ptr(), h_out.shape[0],
                                  h_counts.ctypes.data)
        assert rc == 0, rc

    for _ in range(max(args.warmup, 3)):
        host_call()
    assert int(h_counts.sum()) == total_nodes

    with ClockSampler(local) as clocks:
        ts = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lvn.clipmap_select_device(d_cams, rmin, rsize, d_out, stride, d_counts, stream=stream)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        te = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            host_call()
            te.append(time.perf_counter() - t0)
    ms = sum(ts) / len(ts)
    ms_e2e = 1e3 * sum(te) / len(te)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # algorithmic bytes of one launch: the cameras in, the lists and counts out
    algo = 12 * n + 16 * total_nodes + 4 * n
    ach = algo / (ms / 1e3) / 1e9
    line = {
        "metric": SELECT_METRIC, "impl": "lvn-select", "value": round(n / (ms / 1e3), 1), "unit": "cameras/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"clipmap-select-{n}cameras", "root_size": rsize, "nodes_listed": total_nodes,
                   "stride": stride, "l2": "flushed between steps (256 MiB write)"},
        "e2e": {"value": round(n / (ms_e2e / 1e3), 1), "unit": "cameras/s", "h2d_bytes_per_step": 12 * n,
                "d2h_bytes_per_step": 16 * total_nodes + 4 * n, "ms_per_step": round(ms_e2e, 4)},
        "gpu_launches": 2,
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(ach / hbm_peak, 4), "traffic": None,
                     "kernel": "k_clipmap_select_warp (+ k_clipmap_walk for cameras past its limits)",
                     "ms_per_launch": round(ms, 4),
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                     "algorithmic_bytes_per_launch": algo},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        threads = host_threads()
        v, dt, m = SelectBaseline(cams, threads).rate(3.0)
        line["cpu_baseline"] = {"value": round(v, 1), "unit": "cameras/s", "cores": threads, "kind": "port",
                                "sample": f"{m // n} passes over the {n} cameras, {dt:.1f} s"}
    print(json.dumps(line), flush=True)


SEAMS_METRIC = "clipmap seam meshes/sec on 1 GB300 (GenerateClipmapSeamMesh, 64^3 chunks, LOD 0-5)"
SEAM_COLOUR = (0.25, 0.5, 0.75)


def seams_inputs():
    """One camera's active clipmap nodes (a disjoint tiling of the world, as
    the engine's clipmap holds them) meshed once on the GPU: (workload, seam
    offsets, seam rows (S, 12) int32)."""
    import numpy as np
    import torch

    import leven_gb300 as lvn
    from leven_gb300 import workloads as W

    wl = W.clipmap_frame()
    lvn.initialise(wl.noise_seed, 0, 2)
    lvn.set_density(**wl.density)
    lvn.clear_csg_operations()
    g = lvn.MeshGen(64)
    try:
        _, _, s, res = g.generate_chunks(wl.chunks)
    finally:
        g.close()
    rows = np.concatenate([s[o:o + n] for o, n in zip(res[:, 4], res[:, 5])]).astype(np.int32)
    offs = np.concatenate([[0], np.cumsum(res[:, 5])]).astype(np.int32)
    return wl, offs, rows


def run_seams_reference(args):
    import torch  # noqa: F401  (the GPU meshes the inputs once, outside the timed region)

    from leven_gb300 import workloads as W

    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O

    O.build()
    wl, offs, rows = seams_inputs()
    hosts = list(range(len(wl.chunks)))
    threads = host_threads()

    def one():
        t0 = time.perf_counter()
        O.seam_generate(wl.chunks, offs, rows, 64, W.CLIPMAP_ROOT_MIN, W.CLIPMAP_ROOT_SIZE, hosts, SEAM_COLOUR,
                        threads=threads)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        one()
    vals = [len(hosts) / one() for _ in range(args.steps)]
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": SEAMS_METRIC, "value": round(value, 1), "unit": "seam meshes/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * len(hosts) / value, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"seams-{wl.name}", "seam_nodes": int(offs[-1])},
        "cpu_baseline": {"value": round(value, 1), "unit": "seam meshes/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(hosts)} hosts per step"},
        "e2e": {"value": round(value, 1), "unit": "seam meshes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_seams(args):
    """Seam meshes of every chunk of the caves clipmap set: seam nodes and
    outputs in device memory (value), and from / to pinned host arrays (e2e)."""
    import numpy as np
    import torch

    import leven_gb300 as lvn
    from leven_gb300 import workloads as W

    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl, offs, rows = seams_inputs()
    n = len(wl.chunks)
    hosts = np.arange(n, dtype=np.int32)
    descs = (lvn.ChunkDesc * n)()
    for i, (mn, size) in enumerate(wl.chunks):
        descs[i] = lvn.ChunkDesc((C.c_int32 * 3)(*mn), size)
    results = (lvn.ChunkResult * n)()
    d_rows = torch.from_numpy(rows).to(dev)
    h_rows = torch.from_numpy(rows).pin_memory()
    v, t, res = lvn.seam_generate(wl.chunks, offs, rows, 64, W.CLIPMAP_ROOT_MIN, W.CLIPMAP_ROOT_SIZE, hosts,
                                  SEAM_COLOUR)
    nv, nt = len(v), len(t)
    d_v = torch.empty((nv + 1, 12), dtype=torch.float32, device=dev)
    d_t = torch.empty((nt + 1, 3), dtype=torch.int32, device=dev)
    h_v = torch.empty((nv + 1, 12), dtype=torch.float32).pin_memory()
    h_t = torch.empty((nt + 1, 3), dtype=torch.int32).pin_memory()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)
    L = lvn.lib()
    rmin = lvn._ivec3(W.CLIPMAP_ROOT_MIN)
    colour = (C.c_float * 3)(*SEAM_COLOUR)

    def call(device):
        if device:
            bo = lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, d_v.data_ptr(), nv + 1, 0, d_t.data_ptr(), nt + 1, 0, None, 0, 0,
                              C.cast(results, C.POINTER(lvn.ChunkResult)))
            src, mem = d_rows.data_ptr(), lvn.LVN_MEMORY_DEVICE
        else:
            bo = lvn.BatchOut(lvn.LVN_MEMORY_HOST, h_v.data_ptr(), nv + 1, 0, h_t.data_ptr(), nt + 1, 0, None, 0, 0,
                              C.cast(results, C.POINTER(lvn.ChunkResult)))
            src, mem = h_rows.data_ptr(), lvn.LVN_MEMORY_HOST
        rc = L.lvn_seam_generate(descs, offs.ctypes.data, n, src, mem, 64, rmin, W.CLIPMAP_ROOT_SIZE,
                                 hosts.ctypes.data, n, colour, C.byref(bo))
        assert rc == 0 and bo.total_vertices == nv and bo.total_triangles == nt, rc

    def timed(device):
        for _ in range(max(args.warmup, 3)):
            call(device)
        ts = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call(device)  # returns once its last copy has landed
            ts.append(time.perf_counter() - t0)
        return 1e3 * sum(ts) / len(ts)

    with ClockSampler(local) as clocks:
        ms = timed(True)
        ms_e2e = timed(False)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    leaves = int(res[:, 7].sum())
    # algorithmic bytes: every seam node of every chunk gathered (48 B) and the
    # meshes written (48 B a vertex, 12 B a triangle)
    algo = 48 * leaves + 48 * nv + 12 * nt
    ach = algo / (ms / 1e3) / 1e9
    line = {
        "metric": SEAMS_METRIC, "impl": "lvn-seams", "value": round(n / (ms / 1e3), 1), "unit": "seam meshes/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"seams-{wl.name}", "seam_nodes": int(offs[-1]), "leaves": leaves,
                   "vertices": nv, "triangles": nt, "l2": "flushed between steps (256 MiB write)",
                   "timing": "host clock around the synchronous C-ABI call (its own stream, three waits)"},
        "e2e": {"value": round(n / (ms_e2e / 1e3), 1), "unit": "seam meshes/s", "h2d_bytes_per_step": int(48 * offs[-1]),
                "d2h_bytes_per_step": int(48 * nv + 12 * nt), "ms_per_step": round(ms_e2e, 4)},
        "gpu_launches": 8,
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(ach / hbm_peak, 4), "traffic": None,
                     "kernel": "k_seam_select/leaves/quads/qsort/emit (one call)", "ms_per_launch": round(ms, 4),
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                     "algorithmic_bytes_per_launch": algo},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as O

        O.build()
        threads = host_threads()
        done, total = 0, 0.0
        while total < 3.0:
            t0 = time.perf_counter()
            O.seam_generate(wl.chunks, offs, rows, 64, W.CLIPMAP_ROOT_MIN, W.CLIPMAP_ROOT_SIZE, list(hosts),
                            SEAM_COLOUR, threads=threads)
            total += time.perf_counter() - t0
            done += n
        line["cpu_baseline"] = {"value": round(done / total, 1), "unit": "seam meshes/s", "cores": threads,
                                "kind": "port", "sample": f"{done // n} passes over the {n} hosts, {total:.1f} s"}
    print(json.dumps(line), flush=True)


COLLAPSE_METRIC = "clipmap meshes simplified/sec on 1 GB300 (ngMeshSimplifier, 64^3 chunks, LOD 0-5)"


def collapse_inputs():
    """One camera's clipmap meshed once on the GPU: (workload, vertices,
    triangles, ranges (M, 4), offsets (M, 4)) for the meshes with triangles."""
    import numpy as np

    import leven_gb300 as lvn
    from leven_gb300 import workloads as W

    wl = W.clipmap_frame()
    lvn.initialise(wl.noise_seed, 0, 2)
    lvn.set_density(**wl.density)
    lvn.clear_csg_operations()
    g = lvn.MeshGen(64)
    try:
        v, t, _, res = g.generate_chunks(wl.chunks)
    finally:
        g.close()
    keep = [i for i in range(len(wl.chunks)) if res[i, 3] > 0]
    ranges = res[keep, :4].astype(np.int32)
    offsets = np.array([lvn.node_offset(*wl.chunks[i]) for i in keep], np.float32)
    sizes = [wl.chunks[i][1] for i in keep]
    return wl, v, t, ranges, offsets, sizes


def collapse_cpu(v, t, ranges, offsets, sizes, threads):
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import oracle_lib as O

    O.build()
    opts = np.ascontiguousarray(np.stack([O.simplify_options(s) for s in sizes]).astype(np.float32))
    vv = np.ascontiguousarray(v, np.float32)
    tt = np.ascontiguousarray(t, np.int32)
    rr = np.ascontiguousarray(ranges, np.int32)
    oo = np.ascontiguousarray(offsets, np.float32)

    def one():
        t0 = time.perf_counter()
        O.lib().orc_mesh_collapse_many(vv.ctypes.data, tt.ctypes.data, rr.ctypes.data, len(rr), oo.ctypes.data,
                                       opts.ctypes.data, threads)
        return time.perf_counter() - t0

    return one


def run_collapse_reference(args):
    wl, v, t, ranges, offsets, sizes = collapse_inputs()
    threads = host_threads()
    one = collapse_cpu(v, t, ranges, offsets, sizes, threads)
    for _ in range(args.warmup):
        one()
    vals = [len(ranges) / one() for _ in range(args.steps)]
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": COLLAPSE_METRIC, "value": round(value, 1), "unit": "meshes/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * len(ranges) / value, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"collapse-{wl.name}", "meshes": len(ranges), "triangles_in": int(ranges[:, 3].sum())},
        "cpu_baseline": {"value": round(value, 1), "unit": "meshes/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(ranges)} meshes per step"},
        "e2e": {"value": round(value, 1), "unit": "meshes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_collapse(args):
    """The edge-collapse simplification of one camera's clipmap meshes:
    meshes in device memory (value) and from / to pinned host arrays (e2e)."""
    import numpy as np
    import torch

    import leven_gb300 as lvn

    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl, v, t, ranges, offsets, sizes = collapse_inputs()
    m = len(ranges)
    opts = (lvn.SimplifyOptions * m)(*[lvn.engine_simplify_options(s) for s in sizes])
    offs = np.ascontiguousarray(offsets, np.float32)
    res = (lvn.ChunkResult * m)()

    def reset():
        for i in range(m):
            res[i].vertex_offset, res[i].num_vertices, res[i].triangle_offset, res[i].num_triangles = (
                int(x) for x in ranges[i])

    d_v = torch.from_numpy(v).to(dev)
    d_t = torch.from_numpy(t).to(dev)
    d_ov = torch.empty_like(d_v)
    d_ot = torch.empty_like(d_t)
    h_v = torch.from_numpy(v).pin_memory()
    h_t = torch.from_numpy(t).pin_memory()
    h_ov = torch.empty_like(h_v).pin_memory()
    h_ot = torch.empty_like(h_t).pin_memory()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)
    L = lvn.lib()

    def call(device):
        reset()
        if device:
            rc = L.lvn_mesh_simplify(d_v.data_ptr(), d_t.data_ptr(), lvn.LVN_MEMORY_DEVICE, res, m, offs.ctypes.data,
                                     opts, d_ov.data_ptr(), d_ot.data_ptr())
        else:
            rc = L.lvn_mesh_simplify(h_v.data_ptr(), h_t.data_ptr(), lvn.LVN_MEMORY_HOST, res, m, offs.ctypes.data,
                                     opts, h_ov.data_ptr(), h_ot.data_ptr())
        assert rc == 0, rc

    def timed(device):
        for _ in range(max(args.warmup, 3)):
            call(device)
        ts = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call(device)  # returns once the meshes (and their counts) are out
            ts.append(time.perf_counter() - t0)
        return 1e3 * sum(ts) / len(ts)

    with ClockSampler(local) as clocks:
        ms = timed(True)
        ms_e2e = timed(False)
    tris_out = sum(res[i].num_triangles for i in range(m))
    verts_out = sum(res[i].num_vertices for i in range(m))
    tris_in, verts_in = int(ranges[:, 3].sum()), int(ranges[:, 1].sum())
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    algo = 48 * verts_in + 12 * tris_in + 48 * verts_out + 12 * tris_out
    ach = algo / (ms / 1e3) / 1e9
    line = {
        "metric": COLLAPSE_METRIC, "impl": "lvn-collapse", "value": round(m / (ms / 1e3), 1), "unit": "meshes/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"collapse-{wl.name}", "meshes": m, "triangles_in": tris_in, "triangles_out": tris_out,
                   "vertices_in": verts_in, "vertices_out": verts_out, "l2": "flushed between steps (256 MiB write)",
                   "options": "ConstructClipmapNodeData: max error 5, edge 2.5 (x leaf size), cos 0.7",
                   "timing": "host clock around the synchronous C-ABI call"},
        "e2e": {"value": round(m / (ms_e2e / 1e3), 1), "unit": "meshes/s",
                "h2d_bytes_per_step": 48 * verts_in + 12 * tris_in,
                "d2h_bytes_per_step": 48 * verts_in + 12 * tris_in, "ms_per_step": round(ms_e2e, 4)},
        "gpu_launches": 2,
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(ach / hbm_peak, 4), "traffic": None, "kernel": "k_mesh_collapse",
                     "ms_per_launch": round(ms, 4), "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                     "algorithmic_bytes_per_launch": algo},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        threads = host_threads()
        one = collapse_cpu(v, t, ranges, offsets, sizes, threads)
        done, total = 0, 0.0
        while total < 3.0:
            total += one()
            done += m
        line["cpu_baseline"] = {"value": round(done / total, 1), "unit": "meshes/s", "cores": threads, "kind": "port",
                                "sample": f"{done // m} passes over the {m} meshes, {total:.1f} s"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    WORKLOAD = a.workload
    CHUNKS = a.chunks
    if a.impl == "reference":
        run_reference(a)
    elif a.surrogate:
        run_surrogate(a)
    elif a.workload == "select":
        run_select(a)
    elif a.workload == "seams":
        run_seams(a)
    elif a.workload == "collapse":
        run_collapse(a)
    else:
        run_lvn(a)
