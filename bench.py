"""Benchmark of the chunk-meshing path on GB300.

Workload: 128 LOD0 64^3 chunks tiling a 512 x 128 x 512-voxel region of the
2D fBm terrain (8 octaves, 1/256, lacunarity 2, gain 0.5, amplitude 48, noise
seed 1) with 32 seeded CSG operations (half sphere-subtract, half box-union,
radii / half extents U[2, 12] voxels) stored and replayed per chunk.  A step
meshes every chunk from a fresh field (caches bypassed): field, CSG, edges,
hermite data, leaves + QEF, cuckoo tables, mesh, seams.

  value  chunks/s with outputs left in device memory (per-step CUDA events
         on the library's stream; L2 flushed between steps, outside the
         timed events)
  e2e    chunks/s through the same C-ABI call with host output arrays
         (pinned), device-to-host copies inside the timed region

`--impl reference` times the CPU restatement of the reference algorithm
(oracle/, the reference's OpenCL cannot run here) on all host threads over
a bounded sample of the same workload.
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
METRIC = "64^3 chunks meshed/sec on 1 GB300 (plain path)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="lvn", choices=["lvn", "reference"])
    p.add_argument("--cpu-sample", type=int, default=0, help="chunks in the CPU-baseline sample (0 = auto)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="tiled", choices=["tiled", "clipmap", "one"],
                   help="tiled: 128 LOD0 chunks + 32 CSG ops (default); clipmap: 1024 chunks over LOD 0-4 with "
                        "3D caves; one: a single LOD0 chunk")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


WORKLOAD = "tiled"


def workload():
    from leven_gb300 import workloads as W

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


def cpu_baseline(wl, sample_chunks, threads):
    """The oracle (CPU restatement of the reference algorithm) meshing a bounded
    sample of the workload's chunks on `threads` host threads."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    from leven_gb300 import workloads as W

    O.build()
    O.set_seed(wl.noise_seed)
    d = wl.density
    dens = O.density(mode=d["mode"], octaves2=d["octaves2"], freq2=d["freq2"], lac2=d["lacunarity2"],
                     gain2=d["gain2"], amp2=d["amp2"], octaves3=d.get("octaves3", 6), freq3=d.get("freq3", 1.0 / 64),
                     lac3=d.get("lacunarity3", 2.0), gain3=d.get("gain3", 0.5), amp3=d.get("amp3", 12.0))
    # chunks spread over the workload (both y layers, with and without operations)
    idx = [int(i * len(wl.chunks) / sample_chunks) for i in range(sample_chunks)]
    args = (O.ChunkArgs * len(idx))()
    keep = []
    for j, c in enumerate(idx):
        mn, size = wl.chunks[c]
        ops = O.make_ops([op.as_tuple() for op in W.ops_for_chunk(wl.ops, mn, size)])
        keep.append(ops)
        n_ops = len(W.ops_for_chunk(wl.ops, mn, size))
        args[j] = O.ChunkArgs((C.c_int32 * 3)(*mn), size, wl.voxels_per_chunk, 0, 0, n_ops,
                              C.cast(ops, C.POINTER(O.CsgOp)), 5489)
    t0 = time.perf_counter()
    O.lib().orc_mesh_chunks(C.byref(dens), args, len(idx), threads)
    dt = time.perf_counter() - t0
    return len(idx) / dt, dt, len(idx)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workload()
    threads = host_threads()
    sample = args.cpu_sample or max(threads, 16)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(wl, min(sample, threads), threads)
    for _ in range(args.steps):
        v, dt, n = cpu_baseline(wl, sample, threads)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "chunks/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sample / value, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "chunks_per_step": sample, "voxels_per_chunk": 64, "csg_ops": len(wl.ops),
                   "density": density_name(wl), "sample": f"{sample} of {len(wl.chunks)} chunks per step"},
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
    stream = torch.cuda.ExternalStream(mg.stream(), device=dev)
    n = len(wl.chunks)
    descs = (lvn.ChunkDesc * n)()
    for i, (mn, size) in enumerate(wl.chunks):
        descs[i] = lvn.ChunkDesc((C.c_int32 * 3)(*mn), size)
    results = (lvn.ChunkResult * n)()

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

    with ClockSampler(local) as clocks:
        t_dev, bo_dev = timed(True, args.steps, args.warmup)
        t_e2e, bo_host = timed(False, args.steps, max(3, args.warmup // 2))
    ms = sum(t_dev) / len(t_dev)
    ms_e2e = sum(t_e2e) / len(t_e2e)
    if world > 1:
        t = torch.tensor([ms, ms_e2e], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, ms_e2e = t.tolist()
    value = world * n / (ms / 1e3)
    e2e = world * n / (ms_e2e / 1e3)

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
    traffic = committed_traffic(dominant)
    if dominant == "hermite":
        # FP32 issue-rate roofline: SMs x 128 lanes x 2 flop x clock
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        clk = (clocks.summary()["sm_mhz"] or peaks.get("clocks_under_load", {}).get("sm_mhz_median", 1477.0))
        fp32_peak = sms * 128 * 2 * clk * 1e6 / 1e12
        if wl.density["mode"] != 1:
            flops = None  # the per-evaluation count above is for the 2D fBm terrain
        else:
            flops = hermite_flops(*edge_axis_counts(mg, lvn, n))
        ach = flops / (dom_ms / 1e3) / 1e12 if flops else None
        roof = {"bound": "fp32", "achieved": round(ach, 3) if ach else None, "peak": round(fp32_peak, 2),
                "unit": "TFLOP/s", "frac": round(ach / fp32_peak, 4) if ach else None, "traffic": traffic,
                "kernel": dominant, "ms_per_launch": round(dom_ms, 4), "peak_source": f"SMs x 128 x 2 x {clk} MHz"}
    else:
        b = stage_work(dominant, res_np, n)
        ach = b / (dom_ms / 1e3) / 1e9 if b else None
        roof = {"bound": "hbm", "achieved": round(ach, 1) if ach else None, "peak": hbm_peak, "unit": "GB/s",
                "frac": round(ach / hbm_peak, 4) if ach else None, "traffic": traffic, "kernel": dominant,
                "ms_per_launch": round(dom_ms, 4), "peak_source": peak_src}

    bo = bo_host
    h2d = C.sizeof(lvn.ChunkDesc) * n + 48 * len(wl.ops)  # descriptors + stored operations per chunk (upper bound)
    d2h = 80 * n + 48 * bo.total_vertices + 12 * bo.total_triangles + 48 * bo.total_seams

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "chunks_per_step": n, "voxels_per_chunk": wl.voxels_per_chunk,
                   "csg_ops": len(wl.ops), "density": density_name(wl), "lod": lod_range(wl),
                   "parallelism": f"replicas x{world}", "l2": "flushed between steps (256 MiB write)",
                   "vertices": int(bo.total_vertices), "triangles": int(bo.total_triangles),
                   "edges": E, "seams": int(bo.total_seams)},
        "e2e": {"value": round(e2e, 2), "unit": "chunks/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(ms_e2e, 4)},
        "gpu_launches": int(gpu_launches),
        "roofline": roof,
        "stage_ms": stage_ms,
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = host_threads()
        sample = args.cpu_sample or max(threads, 16)
        v, dt, m = cpu_baseline(wl, sample, threads)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "chunks/s", "cores": threads, "kind": "port",
                                "sample": f"{m} chunks of the {n}-chunk workload, {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    mg.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def committed_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/<kernel>_tiled_csg_128.md, line `dram_bytes_per_launch`)."""
    path = ROOT / "profiles" / f"{kernel}_tiled_csg_128.md"
    try:
        for line in path.read_text().splitlines():
            if "dram_bytes_per_launch" in line:
                return int(line.split("|")[2].strip())
    except (OSError, ValueError, IndexError):
        pass
    return None


# FP32 operations of the restated density arithmetic (an fma counts 2):
# one simplex2 evaluation with its three corners inside the kernel radius 51,
# one octave of fBm 51 + 5, an 8-octave height term 8 * 56 + 4 = 452.
FLOP_HEIGHT8 = 452
# x / z edge: 17 search samples (height + density fma + 3 mix fmas) and 4
# normal samples (height + density + offset), y normal pair, normalise;
# y edge: one height, 17 cheap samples, the same normal work.
FLOP_XZ_EDGE = 17 * (FLOP_HEIGHT8 + 2 + 6) + 4 * (FLOP_HEIGHT8 + 3) + 6 + 9 + 6
FLOP_Y_EDGE = FLOP_HEIGHT8 + 17 * (2 + 6) + 4 * (FLOP_HEIGHT8 + 3) + 6 + 9 + 6


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


def hermite_flops(nxz, ny):
    return nxz * FLOP_XZ_EDGE + ny * FLOP_Y_EDGE



if __name__ == "__main__":
    a = parse()
    WORKLOAD = a.workload
    if a.impl == "reference":
        run_reference(a)
    else:
        run_lvn(a)
