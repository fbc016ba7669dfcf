"""Benchmark: Gpixel-iter/s of the 1e100 FHD atlas on one GB300.

Workload (one step, `fhd_atlas_e100`): every keyframe of a 1920x1080 atlas
with keyframe factor 8 from zoom 1e0 to 1e100 -- the reference's
_atlas_geometry([0, 100], 8) ladder (visualizer.py:7628-7661): levels
i = 0..111, log10 zoom i*log10(8) -- with the reference's per-tile caps
max_iterations(min(100, (i+1)*log10(8)), 2000, 3000, 200000)
(visualizer.py:6958-6979, 11567-11580), centred on a seeded Misiurewicz
point (tests/golden/centres.json "fhd_stack_e50", 1200-bit Newton, 360
digits).  Levels below 1e12 are direct-path levels, deeper ones render from
the shared MPFR reference and its BLA tiers, as the reference pipeline does.
The 55-keyframe FHD stack (levels 0..54, to 1e48.8, caps up to 151k,
`fhd_keyframe_stack`) is measured beside it.  Work unit: a pixel-iteration,
i.e. the sum of uint32 iteration counts (escape index, or the cap for
interior pixels); iterations skipped by the image series or BLA count as
done (the reference's logical_iterations + series_jumps).

Forms
  chosen   floatexp form: deep levels and the direct-path levels between 1e1
           and 1e10 by FP32 perturbation in one persistent queue; the levels
           that keep the FP64 direct iteration (the whole-set view, 1e10 and
           deeper) in the FP64 lane-refill queue on a second stream
  plain    the FP64 form, bit-identical to the reference

Arms
  ours (default)      the GB300 library; `value` is device throughput with
                      the tables resident in HBM, `e2e` goes through the
                      renderer.h ABI into host memory (fields copied back).
  --impl reference    the reference's CPU implementation of the path on the
                      host cores: the reference build in oracle/_ref when it
                      exists, else the oracle port (a restatement pinned
                      bit-exact to it).  The K timed steps together render
                      the whole workload once at full size (keyframes dealt
                      round-robin over the steps).

--gpus N without a launcher starts N replica processes (one per GPU, NCCL
only for the barrier and the max-over-ranks time); under torchrun each
process is one rank.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import socket
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__  # noqa: E402

WIDTH, HEIGHT = 1920, 1080
FACTOR = 8.0
SAMPLE_DIVISOR = 4  # cpu_baseline sample: every keyframe at 480x270 (1/16 of the pixels)
E2E_THREADS = 4     # host threads calling the renderer.h ABI in the end-to-end leg
METRIC = "Gpixel-iter/s on 1e100 FHD atlas, chosen vs plain GPU at ≤1e-4 pixel mismatch"
WORKLOADS = {
    # name: (max log10 zoom of the camera path, keyframe count)
    "fhd_atlas_e100": (100.0, 112),
    "fhd_keyframe_stack": (50.0, 55),
}
HEADLINE = "fhd_atlas_e100"


def workload_levels(name: str = "fhd_keyframe_stack"):
    """(level, log10 zoom, cap) of every keyframe of a workload, and the
    ladder step log10(8)."""
    maximum, count = WORKLOADS[name]
    step = math.log10(FACTOR)
    levels = []
    for i in range(count):
        cap = min(200_000, max(64, int(2000 + 3000 * max(0.0, min(maximum, (i + 1) * step)))))
        levels.append((i, i * step, cap))
    return levels, step


def centre():
    with open(os.path.join(ROOT, "tests", "golden", "centres.json"), encoding="ascii") as handle:
        data = json.load(handle)["fhd_stack_e50"]
    return data["re"], data["im"]


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append([v.strip() for v in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.thread.join(timeout=5)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 9:
                continue
            for name, value in zip(names, r[5:9]):
                if value.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_flops(stats: dict, series_order: int) -> float:
    """Algorithmic flops of the deep render: exact step 22, linear BLA 14,
    cubic BLA 60, image series 8 per term per pixel."""
    return (22.0 * stats["exact_steps"] + 14.0 * stats["linear_blocks"] + 60.0 * stats["cubic_blocks"]
            + 8.0 * series_order * stats["series_pixels"])


def max_over_ranks(value: float) -> float:
    """The largest of every rank's value (the job's time is its slowest
    replica's); the value itself when no process group is running."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_replicas(argv: list[str], gpus: int) -> int:
    """Start one bench process per GPU (RANK / LOCAL_RANK / WORLD_SIZE and a
    127.0.0.1 rendezvous in the environment), as torchrun would; rank 0's
    line is the job's.  Returns the first non-zero exit code, else 0."""
    port = _free_port()
    children = []
    for rank in range(gpus):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(gpus),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        children.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + argv, env=env))
    codes = [child.wait() for child in children]
    return next((code for code in codes if code != 0), 0)


def cpu_library(native):
    """The reference build when present (kind "reference"), else the oracle
    port (kind "port"), built on demand."""
    ref_path = os.path.join(ROOT, "oracle", "_ref", "mandelbrot.so")
    if os.path.exists(ref_path):
        return native.load(ref_path), "reference", ref_path
    ref_path = os.path.join(ROOT, "oracle", "_ref", "liboracle.so")
    if not os.path.exists(ref_path):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "port"], check=True, capture_output=True)
    return native.load(ref_path), "port", ref_path


def cpu_render(native, stack, keyframe, width, height, cores) -> int:
    field, planes = stack.render_host(keyframe, width, height, threads=cores, planes=True)
    return int(native.iteration_counts(field, planes["orbit_iteration"], keyframe.max_iter)
               .astype(np.uint64).sum())


def run_reference_arm(args) -> int:
    """The reference's CPU path on all host cores, on the headline workload
    at full size: the keyframes are dealt round-robin over the K timed steps,
    so the K steps together render every keyframe once (K below the keyframe
    count) and value = their pixel-iterations / their time.  Warm-up steps
    render one keyframe each at 240x135."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    package = __graft_entry__._package()
    native = package.native
    atlas = package.atlas
    library, kind, ref_path = cpu_library(native)
    cores = os.cpu_count() or 1
    levels, step = workload_levels(args.workload)
    x, y = centre()
    t0 = time.perf_counter()
    stack = atlas.KeyframeStack(library, x, y, levels, step=step)
    setup_s = time.perf_counter() - t0
    keyframes = stack.keyframes
    steps = max(1, args.steps)
    # Deal the keyframes costliest-first so the steps carry similar work.
    deal = sorted(range(len(keyframes)), key=lambda i: -keyframes[i].max_iter)
    shares = [deal[k::steps] for k in range(steps)] if steps <= len(keyframes) else \
        [[deal[k % len(keyframes)]] for k in range(steps)]
    for k in range(args.warmup):
        cpu_render(native, stack, keyframes[deal[k % len(deal)]], 240, 135, cores)
    work = 0
    elapsed = 0.0
    for share in shares:
        t0 = time.perf_counter()
        for i in share:
            work += cpu_render(native, stack, keyframes[i], WIDTH, HEIGHT, cores)
        elapsed += time.perf_counter() - t0
    stack.close()
    value = work / elapsed / 1e9
    covered = len({i for share in shares for i in share})
    sample = (f"full size: {covered} of {len(keyframes)} keyframes at {WIDTH}x{HEIGHT} over the {steps} timed steps "
              f"(keyframes dealt round-robin), {elapsed:.1f} s")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "Gpixel-iter/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed / steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Misiurewicz centre, tests/golden/centres.json)",
        "config": {"workload": args.workload, "keyframes": len(keyframes), "width": WIDTH, "height": HEIGHT,
                   "keyframe_factor": FACTOR, "max_log10_zoom": levels[-1][1],
                   "max_cap": max(c for _, _, c in levels), "threads": cores,
                   "library": os.path.relpath(ref_path, ROOT), "reference_setup_s": setup_s,
                   "pixel_iterations": work,
                   **({"port_vs_reference_build": "bit-identical output; 1.62x the reference build's speed on "
                                                  "the x86-64 build host (deep FHD levels 30/40/54 at 240x135, "
                                                  "2 threads, best of 5), at least 0.9x required by "
                                                  "tests/test_oracle_port.py::test_port_runs_at_reference_speed"}
                      if kind == "port" else {})},
        "cpu_baseline": {"value": value, "unit": "Gpixel-iter/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def cpu_baseline_sample(native, atlas, levels, step, x, y) -> dict:
    """Time the CPU implementation on a bounded sample (rank 0, N=1 only):
    every keyframe of the workload at 480x270."""
    library, kind, _ = cpu_library(native)
    cores = os.cpu_count() or 1
    w, h = WIDTH // SAMPLE_DIVISOR, HEIGHT // SAMPLE_DIVISOR
    stack = atlas.KeyframeStack(library, x, y, levels, step=step)
    try:
        work = 0
        t0 = time.perf_counter()
        for keyframe in stack.keyframes:
            work += cpu_render(native, stack, keyframe, w, h, cores)
        elapsed = time.perf_counter() - t0
    finally:
        stack.close()
    return {"value": work / elapsed / 1e9, "unit": "Gpixel-iter/s", "cores": cores, "kind": kind,
            "sample": f"all {len(levels)} keyframes at {w}x{h} (1/{SAMPLE_DIVISOR**2} of the pixels), "
                      f"{elapsed:.1f} s"}


class StackBench:
    """One workload's keyframe stack on the GPU: device outputs, the claim
    order and the timed batched step."""

    def __init__(self, package, library, name, stream, world):
        import torch

        self.package, self.library, self.name, self.world = package, library, name, world
        self.native = package.native
        self.levels, self.step = workload_levels(name)
        x, y = centre()
        t0 = time.perf_counter()
        self.stack = package.atlas.KeyframeStack(library, x, y, self.levels, step=self.step)
        self.setup_s = time.perf_counter() - t0
        n = len(self.stack.keyframes)
        self.pixels = WIDTH * HEIGHT
        self.fields = torch.empty((n, self.pixels), dtype=torch.float32, device="cuda")
        self.counts = torch.empty((n, self.pixels), dtype=torch.int32, device="cuda")
        self.stream = stream
        self.handle = stream.cuda_stream
        self.targets = [(self.fields[i].data_ptr(), self.counts[i].data_ptr()) for i in range(n)]
        keyframes = self.stack.keyframes
        self.fp64_direct = [i for i, k in enumerate(keyframes) if k.reference is None and k.shallow_reference is None]
        self.shallow = [i for i, k in enumerate(keyframes) if k.shallow_reference is not None]
        self.direct = [i for i, k in enumerate(keyframes) if k.reference is None]
        self.deep = [i for i, k in enumerate(keyframes) if k.reference is not None]
        # Claim order: the direct levels first in the direct queue, the
        # deepest levels first in the perturbation queue.
        self.order = self.direct + self.deep[::-1]
        self.floatexp = self.shallow + self.deep[::-1]

    def step_device(self, form, subset=None, autotune=False, tiles=0):
        self.stack.render_batch_device(self.targets, WIDTH, HEIGHT, form=form, stream=self.handle, graph=True,
                                       autotune=autotune, order=subset if subset is not None else self.order,
                                       tiles=tiles if form == 1 else 0)

    def timed(self, form, steps, warmup, subset=None, tiles=0):
        import torch

        for _ in range(warmup):
            self.step_device(form, subset, tiles=tiles)
        torch.cuda.synchronize()
        if self.world > 1:
            torch.distributed.barrier()
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(self.stream)
        for _ in range(steps):
            self.step_device(form, subset, tiles=tiles)
        stop.record(self.stream)
        torch.cuda.synchronize()
        return max_over_ranks(start.elapsed_time(stop))

    def compare_forms(self, form):
        """Counts of both forms on the same views: work, mismatch (all and
        per keyframe) and smooth-value error where the counts agree."""
        import torch

        self.step_device(form)
        torch.cuda.synchronize()
        chosen_counts = self.counts.clone()
        chosen_field = self.fields.clone()
        work = int(self.counts.to(torch.int64).sum().item())
        per_level_work = self.counts.to(torch.int64).sum(dim=1).cpu().numpy()
        self.step_device(0)
        torch.cuda.synchronize()
        plain_work = int(self.counts.to(torch.int64).sum().item())
        differ = self.counts != chosen_counts
        per_field = (differ.sum(dim=1).to(torch.float64) / self.pixels).cpu().numpy()
        mismatch = int(differ.sum().item())
        both = torch.isfinite(self.fields) & torch.isfinite(chosen_field) & ~differ
        err = (self.fields - chosen_field).abs()
        per_field_p99 = []
        for i in range(err.shape[0]):
            e = err[i][both[i]]
            sample = e[torch.randperm(e.numel(), device="cuda")[:200_000]].float()
            per_field_p99.append(float(torch.quantile(sample, 0.99).item()) if sample.numel() else 0.0)
        e = err[both]
        sample = e[torch.randperm(e.numel(), device="cuda")[:1_000_000]].float()
        smooth = {"median": float(sample.median().item()), "p99": float(torch.quantile(sample, 0.99).item()),
                  "max": float(e.max().item())}
        del chosen_counts, chosen_field, differ, both, err
        return {"work": work, "plain_work": plain_work, "mismatch": mismatch / (self.fields.shape[0] * self.pixels),
                "per_field_mismatch": per_field, "per_field_smooth_p99": per_field_p99, "smooth": smooth,
                "per_level_work": per_level_work}

    def close(self):
        self.stack.close()


def run_dry(args) -> int:
    """The replica launch without rendering (tests of --gpus N on CPU hosts):
    ranks rendezvous over gloo at MASTER_ADDR / MASTER_PORT and each prints
    its rank and the max over ranks of rank + 1."""
    import torch.distributed as dist

    rank, world, local_rank = dist_env()
    if world > 1:
        dist.init_process_group("gloo")
    print(json.dumps({"rank": rank, "world": world, "local_rank": local_rank,
                      "max_over_ranks": max_over_ranks(float(rank + 1)),
                      "master": os.environ.get("MASTER_ADDR")}), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def measure_batch_mix(package, library, stream, steps: int, local_rank: int) -> dict:
    """The mixed batch: 64 seeded fields mixing the four formulas and the four
    sizes 720x480 .. 3840x2160, zooms log-uniform 1e10-1e100, caps
    log-uniform 1e4-1e6, counts + smooth field + derivative planes, all in
    one fractal_gb300_render_fields_device call (graph replay, launch
    shapes autotuned on the batch).  Reports Gpixel-iter/s of both forms, the
    count mismatch per formula and the derivative planes' error."""
    import torch

    from tests.golden import cases as case_defs

    mix = case_defs.batch_mix(seed=2024, count=64)
    # (The chosen form here is slow on the other formulas' FP64 fields: a
    # batch takes tens of seconds, so the leg times few batches.)
    specs = [package.fields.FieldSpec(m["formula"], m["re"], m["im"], m["log10_zoom"], m["width"], m["height"],
                                      m["max_iter"], tuple(m["julia"])) for m in mix]
    t0 = time.perf_counter()
    fields = package.fields.FieldSet(library, specs, threads=os.cpu_count() or 8,
                                     initializer=lambda: torch.cuda.set_device(local_rank))
    setup_s = time.perf_counter() - t0
    bufs = []
    for m in mix:
        n = m["width"] * m["height"]
        bufs.append((torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
                     torch.empty(n, dtype=torch.float64, device="cuda"),
                     torch.empty(n, dtype=torch.float64, device="cuda")))
    targets = [tuple(t.data_ptr() for t in b) for b in bufs]
    handle = stream.cuda_stream
    try:
        def timed(form, count, fp32=False):
            torch.cuda.synchronize()
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for _ in range(count):
                fields.render_device(targets, form=form, stream=handle, graph=True, fp32_alternates=fp32)
            stop.record(stream)
            torch.cuda.synchronize()
            return start.elapsed_time(stop) / count

        def mismatch_vs(plain_counts):
            per = {}
            for m, b, pc in zip(mix, bufs, plain_counts):
                d, t = per.get(m["formula"], (0, 0))
                per[m["formula"]] = (d + int((b[1] != pc).sum().item()), t + pc.numel())
            return {f: d / t for f, (d, t) in per.items()}

        fields.render_device(targets, form=0, stream=handle, graph=True)
        torch.cuda.synchronize()
        plain = [(b[1].clone(), b[2].clone(), b[3].clone()) for b in bufs]
        plain_counts = [p[0] for p in plain]
        plain_work = sum(int(c.to(torch.int64).sum().item()) for c in plain_counts)
        # The FP32 queue for all four formulas (opt-in): launch shapes tuned
        # on it, its throughput and its drift from the FP64 counts.
        fields.render_device(targets, form=1, stream=handle, graph=True, fp32_alternates=True, autotune=True)
        torch.cuda.synchronize()
        shapes = (ctypes.c_int * 4)()
        library.fractal_gb300_queue_shapes(shapes, 4)
        fp32_all_mismatch = mismatch_vs(plain_counts)
        fp32_all_work = sum(int(b[1].to(torch.int64).sum().item()) for b in bufs)
        fp32_all_ms = timed(1, 2, fp32=True)
        # The chosen form: Mandelbrot in the FP32 queue, the rest in FP64.
        fields.render_device(targets, form=1, stream=handle, graph=True)
        torch.cuda.synchronize()
        work = sum(int(b[1].to(torch.int64).sum().item()) for b in bufs)
        per_formula = mismatch_vs(plain_counts)
        de_err = []
        for m, b, (pc, pdx, pdy) in zip(mix, bufs, plain):
            same = (b[1] == pc) & (pc < m["max_iter"])
            pd = torch.hypot(pdx, pdy)[same]
            qd = torch.hypot(b[2], b[3])[same]
            ok = pd > 0
            if ok.any():
                de_err.append(((qd[ok] - pd[ok]).abs() / pd[ok]).float())
        de_err = torch.cat(de_err)
        de_sample = de_err[torch.randperm(de_err.numel(), device="cuda")[:1_000_000]]
        chosen_ms = timed(1, steps)
        plain_ms = timed(0, 1)  # the FP64 form takes tens of seconds per batch
        pixels = sum(m["width"] * m["height"] for m in mix)
        return {
            "workload": "batch64_mixed",
            "fields": len(mix),
            "formulas": {f: sum(1 for m in mix if m["formula"] == f) for f in
                         ("mandelbrot", "julia", "burning-ship", "tricorn")},
            "sizes": {f"{w}x{h}": sum(1 for m in mix if (m["width"], m["height"]) == (w, h))
                      for w, h in case_defs.BATCH_SIZES},
            "pixels": pixels,
            "log10_zoom_range": [round(min(m["log10_zoom"] for m in mix), 2),
                                 round(max(m["log10_zoom"] for m in mix), 2)],
            "cap_range": [min(m["max_iter"] for m in mix), max(m["max_iter"] for m in mix)],
            "outputs": "uint32 counts, float32 smooth field, float64 de_x / de_y",
            "value": work / (chosen_ms * 1e-3) / 1e9,
            "unit": "Gpixel-iter/s",
            "ms_per_batch": chosen_ms,
            "plain_value": plain_work / (plain_ms * 1e-3) / 1e9,
            "plain_ms_per_batch": plain_ms,
            "pixel_iterations": work,
            "count_mismatch_vs_plain_per_formula": per_formula,
            "form": "chosen: Mandelbrot fields in the FP32 queue, the other formulas in FP64 beside it",
            "fp32_all_formulas": {"value": fp32_all_work / (fp32_all_ms * 1e-3) / 1e9, "ms_per_batch": fp32_all_ms,
                                  "count_mismatch_vs_plain_per_formula": fp32_all_mismatch},
            "de_relative_error_vs_plain": {"median": float(de_sample.median().item()),
                                           "p99": float(torch.quantile(de_sample, 0.99).item())},
            "autotuned_queue_shapes": {"direct_chunk": shapes[0], "direct_blocks_per_sm": shapes[1],
                                       "floatexp_chunk": shapes[2], "floatexp_blocks_per_sm": shapes[3],
                                       "tuned_on": "the FP32 queue of all four formulas"},
            "reference_setup_s": setup_s,
            "launch": "one fractal_gb300_render_fields_device call replayed as a CUDA graph",
        }
    finally:
        fields.close()


def run_gpu_arm(args) -> int:
    import torch

    rank, world, local_rank = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    package = __graft_entry__._package()
    native = package.native
    library = package.load_library()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    chosen = 1 if args.form == "chosen" else 0
    run = StackBench(package, library, args.workload, stream, world)
    n_levels = len(run.stack.keyframes)

    # Launch shapes tuned once per form on this batch (graph replay; the
    # shapes change the schedule only, never a pixel).
    run.step_device(chosen, autotune=True)
    if chosen:
        run.step_device(0, autotune=True)
    compared = run.compare_forms(chosen)
    work = compared["work"]
    run.step_device(chosen)
    torch.cuda.synchronize()
    shapes = run.stack.queue_shapes()

    sampler = ClockSampler(local_rank)
    sampler.start()
    ms = run.timed(chosen, args.steps, args.warmup)
    clocks = sampler.stop()
    ms_per_step = ms / args.steps
    value = world * work * args.steps / (ms * 1e-3) / 1e9
    plain_steps = max(1, args.steps // 4)
    plain_ms = run.timed(0, plain_steps, 1) if chosen else ms
    plain_value = compared["plain_work"] * plain_steps / (plain_ms * 1e-3) / 1e9 if chosen else value

    # Each queue alone with the step's own launch shapes: the FP32
    # perturbation queue (deep + shallow-mode levels) and the FP64 direct
    # queue (levels that keep the direct iteration).
    pinned = (ctypes.c_int * 4)(*shapes)
    library.fractal_gb300_set_queue_shapes(pinned, 4)
    queue_ms = run.timed(chosen, 3, 1, subset=run.floatexp if chosen else run.deep[::-1]) / 3
    direct_subset = run.fp64_direct if chosen else run.direct
    direct_ms = run.timed(chosen, 3, 1, subset=direct_subset) / 3 if direct_subset else 0.0
    library.fractal_gb300_set_queue_shapes(None, 0)
    fp32 = ctypes.c_double(0.0)
    library.fractal_gb300_fma_peak(32, ctypes.byref(fp32))
    fp64 = ctypes.c_double(0.0)
    library.fractal_gb300_fma_peak(64, ctypes.byref(fp64))
    # Algorithmic flops of the perturbation queue: the deep levels' counters
    # (22 per exact step, 14 per linear block, 60 per cubic block, 8 per
    # series term and pixel; the reference's own counters, taken from the
    # plain form's render of the same views), plus 22 per iteration of the
    # shallow-mode levels (every iteration there is an exact perturbation
    # step: no series, no BLA, no culled pixel in those views).
    flops = 0.0
    library.fractal_set_stats_enabled(1)
    for i in run.deep:
        run.stack.render_host(run.stack.keyframes[i], WIDTH, HEIGHT)
        flops += algorithmic_flops(native.stats(library), 32)
    library.fractal_set_stats_enabled(0)
    shallow_steps = int(sum(compared["per_level_work"][i] for i in run.shallow)) if chosen else 0
    flops += 22.0 * shallow_steps
    achieved = flops / (queue_ms * 1e-3) / 1e12
    peak = fp32.value if chosen else fp64.value
    roofline = {
        "bound": "fp32-fma" if chosen else "fp64-fma",
        "achieved": achieved,
        "peak": peak,
        "unit": "TFLOP/s",
        "frac": achieved / peak if peak else None,
        "traffic": None,
        "peak_source": f"FP{'32' if chosen else '64'} FMA chains measured on this GPU by fractal_gb300_fma_peak "
                       "(MEASURED_PEAKS.json holds only HBM and bf16 tensor peaks); of measured",
        "kernel": f"floatexp_queue_kernel ({len(run.floatexp)} keyframes: {len(run.deep)} deep, "
                  f"{len(run.shallow)} shallow-mode)" if chosen else "plain_mandelbrot_kernel (deep levels)",
        "launch_ms": queue_ms,
        "flops_per_unit": "22 per exact step, 14 per linear BLA block, 60 per cubic block, 8 per series term",
        "flops_per_launch": flops,
    }

    # End to end through the renderer.h ABI: host output buffers, the field
    # copied back every keyframe, from E2E_THREADS host threads at once (the
    # reference pipeline's prefetch executor calls the library from several
    # threads, visualizer.py:11541).  Backend 4 selects the floatexp form.
    from concurrent.futures import ThreadPoolExecutor

    e2e_options = native.RenderOptions(backend=4 if chosen else 0)
    e2e_steps = max(1, args.steps // 4)
    e2e_order = [run.stack.keyframes[i] for i in run.order]

    def render_one(keyframe):
        run.stack.render_host(keyframe, WIDTH, HEIGHT, options=e2e_options)

    with ThreadPoolExecutor(E2E_THREADS) as pool:
        list(pool.map(render_one, e2e_order[:2 * E2E_THREADS]))
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            list(pool.map(render_one, e2e_order))
        e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * work * e2e_steps / e2e_s / 1e9

    # The 55-keyframe FHD stack beside the headline (N=1 replica 0 only).
    second = None
    if rank == 0 and args.workload == HEADLINE and not args.headline_only:
        del run.fields, run.counts
        torch.cuda.empty_cache()
        stack50 = StackBench(package, library, "fhd_keyframe_stack", stream, 1)
        stack50.step_device(chosen, autotune=True)
        if chosen:
            stack50.step_device(0, autotune=True)
        c50 = stack50.compare_forms(chosen)
        steps50 = max(2, args.steps // 2)
        ms50 = stack50.timed(chosen, steps50, 2)
        plain50 = stack50.timed(0, max(1, args.steps // 8), 1) if chosen else ms50
        schedules = {}
        if chosen:
            net = package.costnet.load_default(library)
            net.attach()
            for name, flags in (("tiles", native.BATCH_TILES), ("learned", native.BATCH_TILES | native.BATCH_LEARNED)):
                stack50.step_device(chosen, autotune=True, tiles=flags)
                schedules[name] = stack50.timed(chosen, steps50, 1, tiles=flags) / steps50
            library.fractal_gb300_set_cost_network(None)
            net.close()
        schedules["chunks"] = ms50 / steps50
        second = {"workload": "fhd_keyframe_stack", "keyframes": len(stack50.stack.keyframes),
                  "max_log10_zoom": stack50.levels[-1][1], "max_cap": max(c for _, _, c in stack50.levels),
                  "value": c50["work"] * steps50 / (ms50 * 1e-3) / 1e9, "ms_per_step": ms50 / steps50,
                  "plain_value": c50["plain_work"] * max(1, args.steps // 8) / (plain50 * 1e-3) / 1e9,
                  "count_mismatch_vs_plain": c50["mismatch"], "smooth_error_vs_plain": c50["smooth"],
                  "pixel_iterations_per_step": c50["work"], "schedule_ms_per_step": schedules}
        stack50.close()

    batch = None
    if rank == 0 and args.workload == HEADLINE and not args.headline_only and chosen:
        batch = measure_batch_mix(package, library, stream, 1, local_rank)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(native, package.atlas, run.levels, run.step, *centre())
    run.close()

    if rank == 0:
        per_field = compared["per_field_mismatch"]
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "Gpixel-iter/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32-floatexp" if chosen else "f64",
            "data": "synthetic (seeded Misiurewicz centre, tests/golden/centres.json)",
            "config": {
                "workload": args.workload,
                "keyframes": n_levels,
                "width": WIDTH,
                "height": HEIGHT,
                "keyframe_factor": FACTOR,
                "max_log10_zoom": run.levels[-1][1],
                "max_cap": max(c for _, _, c in run.levels),
                "form": args.form,
                "pixel_iterations_per_step": work,
                "count_mismatch_vs_plain": compared["mismatch"],
                "plain_value": plain_value,
                "chosen_vs_plain": value / plain_value if plain_value else None,
                "per_field_count_mismatch": [round(float(v), 7) for v in per_field],
                "per_field_smooth_p99_vs_plain": [round(v, 5) for v in compared["per_field_smooth_p99"]],
                "max_field_count_mismatch": float(max(per_field)),
                "smooth_error_vs_plain": compared["smooth"],
                "reference_setup_s": run.setup_s,
                "levels": {"fp64_direct": [run.stack.keyframes[i].level for i in run.fp64_direct],
                           "shallow_mode": [run.stack.keyframes[i].level for i in run.shallow],
                           "deep": len(run.deep)},
                "queue_shapes": {"direct_chunk": shapes[0], "direct_blocks_per_sm": shapes[1],
                                 "floatexp_chunk": shapes[2], "floatexp_blocks_per_sm": shapes[3]},
                "queue_ms_alone": {"floatexp_queue": queue_ms, "fp64_direct_queue": direct_ms},
                "launch": "one batched call per step replayed as a CUDA graph: FP32 perturbation queue "
                          "(floatexp + shallow mode) on the caller's stream, FP64 direct queue on a second "
                          "stream for the levels that keep it",
                "schedule": "chunks",
                "fhd_keyframe_stack": second,
                "batch64_mixed": batch,
                "l2": "outputs larger than L2 (fields + counts: "
                      f"{n_levels * WIDTH * HEIGHT * 8 / 1e6:.0f} MB per step)",
            },
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": n_levels * WIDTH * HEIGHT * 4,
                    "path": f"fractal_render_reference_ex (backend {4 if chosen else 0}) / render_fractal_ex "
                            f"into host memory, {E2E_THREADS} host threads"},
            # Per step: direct coordinates + direct queue (when the step has
            # FP64 direct levels), and a series prologue + floatexp queue per
            # 64 FP32-queue fields; the plain form launches the direct pair
            # plus one kernel per deep field.
            "gpu_launches": args.steps * ((2 if run.fp64_direct else 0) + 2 * ((len(run.floatexp) + 63) // 64)
                                          if chosen else 2 + len(run.deep)),
            "roofline": roofline,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_case(name: str) -> int:
    """One small, fixed piece of the workload for profiler captures (no
    timing output): the commands in profiles/ run these."""
    import torch

    package = __graft_entry__._package()
    library = package.load_library()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    if name == "costnet_predict_20992":
        net = package.costnet.load_default(library)
        rows = 20992
        x = torch.zeros((rows, 320), dtype=torch.int16, device="cuda")
        out = torch.empty(rows, dtype=torch.float32, device="cuda")
        for _ in range(2):
            assert library.fractal_gb300_costnet_predict(net.handle, x.data_ptr(), rows, out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        net.close()
        print("ok", name)
        return 0
    if name == "atlas_colour_3840x2160":
        # Two 4K keyframes (levels 30 and 31), then the atlas frame twice
        # (parent zoom 1.7, child fraction 1.7 / 4, as the frame-pass default).
        width, height = 3840, 2160
        levels, step = workload_levels()
        x, y = centre()
        stack = package.atlas.KeyframeStack(library, x, y, [levels[30], levels[31]], step=step)
        fields = torch.empty((2, width * height), dtype=torch.float32, device="cuda")
        counts = torch.empty((2, width * height), dtype=torch.int32, device="cuda")
        for i, keyframe in enumerate(stack.keyframes):
            stack.render_device(keyframe, fields[i].data_ptr(), counts[i].data_ptr(), width, height, form=1,
                                stream=stream.cuda_stream)
        caps = [k.max_iter for k in stack.keyframes]
        rgb = torch.empty(width * height * 3, dtype=torch.uint8, device="cuda")
        for _ in range(2):
            status = library.fractal_gb300_atlas_colourise_device(
                fields[0].data_ptr(), width, height, caps[0], fields[1].data_ptr(), width, height, caps[1],
                rgb.data_ptr(), width, height, 1.7, 0.425, 0, 0.3, 0.4, 0.7, 0.5, None, None,
                ctypes.c_void_p(stream.cuda_stream))
            assert status == 0, package.native.last_error(library)
        torch.cuda.synchronize()
        stack.close()
        print("ok", name)
        return 0
    if name in ("kfp_colour_3840x2160", "aurora_colour_3840x2160"):
        # A 4K field from the stack's level 30 view, then the colour pass
        # twice (device buffers in and out).
        width, height = 3840, 2160
        levels, step = workload_levels()
        x, y = centre()
        stack = package.atlas.KeyframeStack(library, x, y, [levels[30]], step=step)
        keyframe = stack.keyframes[0]
        field = torch.empty(width * height, dtype=torch.float32, device="cuda")
        counts = torch.empty(width * height, dtype=torch.int32, device="cuda")
        stack.render_device(keyframe, field.data_ptr(), counts.data_ptr(), width, height, form=1,
                            stream=stream.cuda_stream)
        rgb = torch.empty(width * height * 3, dtype=torch.uint8, device="cuda")
        kfp = package.kfp
        profile = kfp.recipe("seeded16")
        lut = torch.from_numpy(kfp.palette_lut(profile)).cuda()
        options = kfp.options(profile)
        for _ in range(2):
            if name.startswith("kfp"):
                status = library.fractal_gb300_colourise_kfp_device(
                    ctypes.c_void_p(field.data_ptr()), ctypes.c_void_p(rgb.data_ptr()), width, height,
                    keyframe.max_iter, ctypes.byref(options), ctypes.c_void_p(lut.data_ptr()), lut.shape[0],
                    ctypes.c_void_p(stream.cuda_stream))
            else:
                status = library.fractal_gb300_colourise_device(
                    ctypes.c_void_p(field.data_ptr()), ctypes.c_void_p(rgb.data_ptr()), width, height,
                    keyframe.max_iter, 0.3, 0.4, 0.7, 0.5, ctypes.c_void_p(stream.cuda_stream))
            assert status == 0, package.native.last_error(library)
        torch.cuda.synchronize()
        stack.close()
        print("ok", name)
        return 0
    width, height = (960, 540) if name.endswith("960x540") else (WIDTH, HEIGHT)
    levels, step = workload_levels("fhd_atlas_e100" if name.startswith("atlas_e100") else "fhd_keyframe_stack")
    x, y = centre()
    stack = package.atlas.KeyframeStack(library, x, y, levels, step=step)
    n = len(stack.keyframes)
    fields = torch.empty((n, width * height), dtype=torch.float32, device="cuda")
    counts = torch.empty((n, width * height), dtype=torch.int32, device="cuda")
    targets = [(fields[i].data_ptr(), counts[i].data_ptr()) for i in range(n)]
    direct = [i for i, k in enumerate(stack.keyframes) if k.reference is None]
    deep = [i for i, k in enumerate(stack.keyframes) if k.reference is not None][::-1]
    shallow = [i for i, k in enumerate(stack.keyframes) if k.shallow_reference is not None]
    subsets = {"direct_levels_4_13_960x540": direct[4:], "direct_levels_0_3_960x540": direct[:4],
               "deep_levels_12_960x540": deep[:12], "stack_step_fhd": direct + deep,
               "atlas_e100_step_fhd": direct + deep, "atlas_e100_deep_24_960x540": deep[:24],
               "atlas_e100_shallow_960x540": shallow}
    full = name in ("stack_step_fhd", "atlas_e100_step_fhd")
    for _ in range(2 if full else 1):
        stack.render_batch_device(targets, width, height, form=1, stream=stream.cuda_stream, order=subsets[name],
                                  graph=full)
    torch.cuda.synchronize()
    stack.close()
    print("ok", name)
    return 0


def run_frame_passes(args) -> int:
    """Per-video-frame passes at 3840x2160 (the song path: atlas keyframes at
    4K, factor 4): the atlas compositor (aurora RGB8, scalar frame, and the
    raw KFP frame: composed surface + KFP pass) from two 4K keyframe fields
    at parent zoom z / child fraction z/4 (the factor-4 ladder; z =
    --frame-zoom, default 1.7), and the aurora and KFP colour passes of one
    4K field.  Each pass: 3 warm-up runs,
    then `--steps` runs timed with CUDA events on the launching stream, an
    L2 flush (256 MiB write, untimed) before each.  Algorithmic bytes: the
    source samples the frame needs once (parent crop + child, 4 B each) plus
    the output (3 B RGB or 4 B float per pixel).  The oracle port times the
    same atlas frame on the host cores."""
    import torch

    package = __graft_entry__._package()
    library = package.load_library()
    native = package.native
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    width, height = 3840, 2160
    pixels = width * height
    levels, step = workload_levels()
    x, y = centre()
    pair = [levels[30], levels[31]]
    stack = package.atlas.KeyframeStack(library, x, y, pair, step=step)
    fields = torch.empty((2, pixels), dtype=torch.float32, device="cuda")
    counts = torch.empty((2, pixels), dtype=torch.int32, device="cuda")
    for i, keyframe in enumerate(stack.keyframes):
        stack.render_device(keyframe, fields[i].data_ptr(), counts[i].data_ptr(), width, height, form=1,
                            stream=stream.cuda_stream)
    torch.cuda.synchronize()
    caps = [k.max_iter for k in stack.keyframes]
    rgb = torch.empty(pixels * 3, dtype=torch.uint8, device="cuda")
    frame = torch.empty(pixels, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    interior = (ctypes.c_int * 3)(0, 0, 0)
    zoom, fraction = args.frame_zoom, args.frame_zoom / 4.0
    kfp = package.kfp
    profile = kfp.recipe("seeded16")
    lut = torch.from_numpy(kfp.palette_lut(profile)).cuda()
    options = kfp.options(profile)
    h = ctypes.c_void_p(stream.cuda_stream)
    packed = torch.empty(pixels * 4, dtype=torch.uint8, device="cuda")
    passes = {
        "atlas_colourise": (lambda: library.fractal_gb300_atlas_colourise_device(
            fields[0].data_ptr(), width, height, caps[0], fields[1].data_ptr(), width, height, caps[1],
            rgb.data_ptr(), width, height, zoom, fraction, 0, 0.3, 0.4, 0.7, 0.5, interior, None, h),
            pixels * 4 / zoom ** 2 + pixels * 4 + pixels * 3),
        "atlas_field": (lambda: library.fractal_gb300_atlas_field_device(
            fields[0].data_ptr(), width, height, caps[0], fields[1].data_ptr(), width, height, caps[1],
            frame.data_ptr(), width, height, zoom, fraction, 1.0, 0.0, 0.0, 0.0, caps[1], 48, h),
            pixels * 4 / zoom ** 2 + pixels * 4 + pixels * 4),
        "atlas_kfp_raw": (lambda: library.fractal_gb300_atlas_colourise_kfp_raw_device(
            fields[0].data_ptr(), width, height, caps[0], fields[1].data_ptr(), width, height, caps[1],
            rgb.data_ptr(), width, height, zoom, fraction, 1.0, caps[1], ctypes.byref(options),
            ctypes.c_void_p(lut.data_ptr()), lut.shape[0], h),
            pixels * 4 / zoom ** 2 + pixels * 4 + pixels * 3),
        "aurora_colour": (lambda: library.fractal_gb300_colourise_device(
            ctypes.c_void_p(fields[0].data_ptr()), ctypes.c_void_p(rgb.data_ptr()), width, height, caps[0], 0.3,
            0.4, 0.7, 0.5, h), pixels * 7),
        "kfp_colour": (lambda: library.fractal_gb300_colourise_kfp_device(
            ctypes.c_void_p(fields[0].data_ptr()), ctypes.c_void_p(rgb.data_ptr()), width, height, caps[0],
            ctypes.byref(options), ctypes.c_void_p(lut.data_ptr()), lut.shape[0], h), pixels * 7),
        # Frame packing for the encoder pipe: RGB8 in (3 B), NV12 out (1.5 B)
        # or RGBA out (4 B) per pixel.
        "pack_nv12": (lambda: library.fractal_gb300_pack_frame_device(
            ctypes.c_void_p(rgb.data_ptr()), width, height, 4, ctypes.c_void_p(packed.data_ptr()), h),
            pixels * 3 + pixels * 3 // 2),
        "pack_rgba": (lambda: library.fractal_gb300_pack_frame_device(
            ctypes.c_void_p(rgb.data_ptr()), width, height, 2, ctypes.c_void_p(packed.data_ptr()), h),
            pixels * 7),
    }
    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"), encoding="ascii"))["hbm_gbs"]
    results = []
    with torch.cuda.stream(stream):
        for name, (call, algorithmic) in passes.items():
            times = []
            for i in range(3 + args.steps):
                flush.fill_(i & 0xFF)
                start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                start.record(stream)
                status = call()
                stop.record(stream)
                assert status == 0, native.last_error(library)
                stream.synchronize()
                if i >= 3:
                    times.append(start.elapsed_time(stop))
            ms = statistics.median(times)
            achieved = algorithmic / (ms * 1e-3) / 1e9
            entry = {"pass": f"{name}_3840x2160", "ms": round(ms, 4), "algorithmic_bytes": int(algorithmic),
                     "achieved_gbs": round(achieved, 1), "frac_of_measured_hbm": round(achieved / peak, 4)}
            if name.startswith("atlas"):
                entry["exact_pass_pixels"] = int(library.fractal_gb300_atlas_last_exact_pixels())
            results.append(entry)
    # The same atlas frame on the host cores through the oracle port.
    port = native.load(os.path.join(ROOT, "oracle", "_ref", "liboracle.so"))
    host = [fields[i].cpu().numpy() for i in range(2)]
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    native.atlas_colourise(port, host[0], (width, height), caps[0], host[1], (width, height), caps[1],
                           (width, height), zoom, fraction, 0, 0.3, 0.4, 0.7, 0.5, interior=(0, 0, 0))
    cpu_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    native.atlas_colourise(library, host[0], (width, height), caps[0], host[1], (width, height), caps[1],
                           (width, height), zoom, fraction, 0, 0.3, 0.4, 0.7, 0.5, interior=(0, 0, 0))
    e2e_ms = (time.perf_counter() - t0) * 1e3
    entries = host_entry_passes(package, library, stack, fields, counts, caps, width, height, zoom, fraction,
                                args.steps)
    stack.close()
    print(json.dumps({"frame_passes": results, "host_entries": entries, "parent_zoom": zoom,
                      "child_fraction": fraction,
                      "atlas_colourise_cpu_port_ms": round(cpu_ms, 2),
                      "cpu_cores": cores, "atlas_colourise_e2e_host_buffers_ms": round(e2e_ms, 2),
                      "levels": [pair[0][0], pair[1][0]], "caps": caps}))
    return 0


def host_entry_passes(package, library, stack, fields, counts, caps, width, height, zoom, fraction, steps):
    """The renderer.h entries that take host buffers, at 3840x2160: wall time
    of the call (uploads and readback included) and the device time of its
    kernels (fractal_gb300_last_kernel_ms), medians of `steps` calls after
    one warm-up.  Inputs: the two 4K keyframe fields; seeded synthetic render
    planes (orbit_iteration from the counts, test1 / test2 / phase / DE
    drawn from fixed distributions); the plane atlas from 1920x1080 halves;
    the separate-tile child a 1920x1080 centre crop; 2^20 log-polar points
    around the first keyframe's reference."""
    import numpy as np

    native, kfp = package.native, package.kfp
    rng = np.random.default_rng(5)
    pixels = width * height
    host = [fields[i].cpu().numpy() for i in range(2)]
    orbit = [np.maximum(counts[i].cpu().numpy().astype(np.int64) - 1, 0) for i in range(2)]

    def planes_of(i):
        return {"orbit_iteration": orbit[i], "test1": rng.uniform(1.0e8, 1.0e12, pixels),
                "test2": rng.uniform(1.0e2, 1.0e6, pixels), "phase": rng.uniform(0.0, 1.0, pixels),
                "de_x": rng.normal(size=pixels), "de_y": rng.normal(size=pixels)}

    def half(a):
        return np.ascontiguousarray(a.reshape(height, width)[::2, ::2]).ravel()

    planes = [planes_of(0), planes_of(1)]
    small = [{k: half(v) for k, v in p.items()} for p in planes]
    crop = np.ascontiguousarray(host[1].reshape(height, width)[540:1620, 960:2880]).ravel()
    profile = kfp.recipe("differences7")
    lut, options = kfp.palette_lut(profile), kfp.options(profile)
    keyframe = stack.keyframes[0]
    count = 1 << 20
    u = rng.uniform(-1.5, 0.5, count)
    angle = rng.uniform(0.0, 2.0 * math.pi, count)
    log2_radius = (u - keyframe.log10_zoom) * math.log2(10.0)
    exponents = np.ceil(log2_radius).astype(np.int32)
    magnitude = np.exp2(log2_radius - exponents)
    real, imag = magnitude * np.cos(angle), magnitude * np.sin(angle)
    cap = max(caps)
    calls = {
        "kfp_planes_3840x2160": lambda: native.colourise_kfp_planes(library, host[0], width, height, cap, options,
                                                                    planes[0], lut),
        "atlas_kfp_tiles_3840x2160": lambda: native.atlas_colourise_kfp(
            library, host[0], (width, height), crop, (1920, 1080), (960, 540), 32, cap, options, lut),
        "atlas_kfp_planes_3840x2160": lambda: native.atlas_colourise_kfp_planes(
            library, half(host[0]), (1920, 1080), caps[0], small[0], half(host[1]), (1920, 1080), caps[1], small[1],
            (width, height), zoom, fraction, 1.0, cap, 0, options, lut),
        "points_1048576": lambda: native.render_points(
            library, keyframe.reference, package.atlas.zoom_text(keyframe.log10_zoom), real, imag, exponents,
            keyframe.max_iter),
    }
    results = []
    for name, call in calls.items():
        walls, kernels = [], []
        for i in range(1 + steps):
            t0 = time.perf_counter()
            call()
            wall = (time.perf_counter() - t0) * 1e3
            if i >= 1:
                walls.append(wall)
                kernels.append(library.fractal_gb300_last_kernel_ms())
        results.append({"entry": name, "wall_ms": round(statistics.median(walls), 3),
                        "device_ms": round(statistics.median(kernels), 4)})
    # The same point render on the host cores through the oracle port (its
    # own reference at the keyframe's zoom), on the first 2^14 points.
    port = native.load(os.path.join(ROOT, "oracle", "_ref", "liboracle.so"))
    zoom = package.atlas.zoom_text(keyframe.log10_zoom)
    bits = package.atlas.precision_bits(stack.x, stack.y, keyframe.log10_zoom)
    handle = native.create_reference(port, stack.x, stack.y, zoom, keyframe.max_iter, bits, 32)
    try:
        sample = 1 << 14
        t0 = time.perf_counter()
        native.render_points(port, handle, zoom, real[:sample], imag[:sample], exponents[:sample], keyframe.max_iter)
        cpu_ms = (time.perf_counter() - t0) * 1e3
    finally:
        port.fractal_destroy_reference(handle)
    results.append({"entry": "points_16384_cpu_port", "wall_ms": round(cpu_ms, 3), "cores": os.cpu_count() or 1,
                    "points_per_s": round(sample / (cpu_ms * 1e-3), 1)})
    return results


SONG_FACTOR = 4.0      # atlas keyframe factor of the song workload
SONG_OVERSCAN = 1.2    # KFP tiles are stored 1.2x wider than their view (ATLAS_TILE_OVERSCAN_FACTOR)
SONG_MAX_LOG = 100.0   # the camera path ends at zoom 1e100


def song_levels():
    """The 4K song atlas: levels 0..167 of factor 4 up to 1e100 (the
    reference's _atlas_geometry for a [0, 100] decade path), each tile stored
    at its level zoom / 1.2, caps max_iterations(log, 384, 500, 100000)."""
    step = math.log10(SONG_FACTOR)
    count = int(math.ceil(SONG_MAX_LOG / step - 1.0e-12))
    levels = []
    for i in range(count + 1):
        log_zoom = i * step - math.log10(SONG_OVERSCAN)
        cap = min(100_000, max(64, int(384 + 500 * max(0.0, log_zoom))))
        levels.append((i, log_zoom, cap))
    return levels, step


def song_frame(log_zoom: float, step: float, last_level: int):
    """Atlas parameters of a frame at log10 zoom `log_zoom`: (parent level,
    parent zoom, child fraction); child zoom is the overscan
    (visualizer.py:11959-11975, 666-696)."""
    level = max(0, min(int(math.floor(log_zoom / step + 1.0e-9)), last_level))
    parent_zoom = max(1.0, SONG_OVERSCAN * 10.0 ** (log_zoom - level * step))
    fraction = min(1.0, max(0.0, parent_zoom / (SONG_FACTOR * SONG_OVERSCAN))) if level < last_level else 0.0
    return level, parent_zoom, fraction


def run_song(args) -> int:
    """The song workload at 4K60: 180 s -> 10,800 frames over the 168-tile
    factor-4 atlas to 1e100 (seeded Misiurewicz centre).  Every tile is
    rendered once (batched keyframe call, chosen form), then every frame is
    one raw KFP atlas frame (parent + child composed into a 4K surface, one
    KFP pass: 16 seeded stops, ColorMethod 7, Differences 3, slopes, dither)
    into device RGB8.  The camera follows the song: a seeded synthetic track
    (sines 110-880 Hz, pink noise, a 120-BPM onset train, a slow envelope;
    song.synthesize) gives per-frame loudness and onsets (song.frame_controls)
    that drive the reference's zoom plan from 1e0 to 1e100 (song.zoom_plan,
    visualizer.py:6982; punch 3, quiet speed -0.04, the CLI defaults).
    Reports fps and the iteration / colour time shares; the reference
    creation (MPFR orbit, host) and the audio side are reported apart."""
    import torch

    package = __graft_entry__._package()
    library = package.load_library()
    native = package.native
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    width, height = 3840, 2160
    pixels = width * height
    t0 = time.perf_counter()
    audio = package.song.synthesize(seconds=args.song_seconds)
    loudness, onset = package.song.frame_controls(audio, fps=60.0)
    plan = package.song.zoom_plan(loudness, 0.0, SONG_MAX_LOG, 3.0, -0.04, onset, 0.0)
    audio_s = time.perf_counter() - t0
    frames = len(plan)
    levels, step = song_levels()
    last = len(levels) - 1
    x, y = centre()
    t0 = time.perf_counter()
    stack = package.atlas.KeyframeStack(library, x, y, levels, step=step)
    reference_s = time.perf_counter() - t0
    fields = torch.empty((len(levels), pixels), dtype=torch.float32, device="cuda")
    counts = torch.empty((len(levels), pixels), dtype=torch.int32, device="cuda")
    targets = [(fields[i].data_ptr(), counts[i].data_ptr()) for i in range(len(levels))]
    h = stream.cuda_stream
    # Warm-up (tables upload, graph/autotune state), then the timed tile pass.
    stack.render_batch_device(targets, width, height, form=1, stream=h)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    stack.render_batch_device(targets, width, height, form=1, stream=h)
    stop.record(stream)
    stop.synchronize()
    fields_ms = start.elapsed_time(stop)
    iterations = int(counts.to(torch.int64).sum().item())
    caps = [cap for _, _, cap in levels]
    kfp = package.kfp
    profile = kfp.recipe("seeded16")
    lut = torch.from_numpy(kfp.palette_lut(profile)).cuda()
    options = kfp.options(profile)
    rgb = torch.empty((2, pixels * 3), dtype=torch.uint8, device="cuda")

    def frame(t):
        level, parent_zoom, fraction = song_frame(float(plan[t]), step, last)
        child = level + 1 if fraction > 0.0 else None
        status = library.fractal_gb300_atlas_colourise_kfp_raw_device(
            fields[level].data_ptr(), width, height, caps[level],
            fields[child].data_ptr() if child is not None else None, width if child is not None else 0,
            height if child is not None else 0, caps[child] if child is not None else 0,
            rgb[t & 1].data_ptr(), width, height, parent_zoom, fraction, SONG_OVERSCAN if child else 1.0,
            max(caps[level], caps[child] if child is not None else 0), ctypes.byref(options),
            ctypes.c_void_p(lut.data_ptr()), lut.shape[0], ctypes.c_void_p(h))
        if status != 0:
            raise RuntimeError(native.last_error(library))

    for t in range(3):
        frame(t)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    start.record(stream)
    for t in range(frames):
        frame(t)
    stop.record(stream)
    stop.synchronize()
    frames_wall_ms = (time.perf_counter() - wall0) * 1e3
    frames_ms = start.elapsed_time(stop)
    total_ms = fields_ms + frames_ms
    # The same frames handed to an encoder pipe: packed to NV12 on the device
    # and copied into pinned host buffers (double-buffered), the pipe itself
    # replaced by a sink that discards the bytes.
    class Discard:
        def write(self, data):
            return len(data)

    writer = package.frames.FrameWriter(library, Discard(), width, height, "nv12")
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for t in range(frames):
        frame(t)
        writer.push(rgb[t & 1].data_ptr(), stream)
    writer.close()
    torch.cuda.synchronize()
    handoff_wall_ms = (time.perf_counter() - wall0) * 1e3
    stack.close()
    print(json.dumps({
        "workload": f"song 4K60: {frames} frames, {len(levels)} atlas tiles (factor 4, to 1e100), KFP raw atlas frames",
        "camera": "zoom plan of the synthetic song (loudness punch 3, quiet speed -0.04)",
        "plan_backward_frames": int(np.sum(np.diff(plan) < 0)),
        "plan_levels_visited": int(len({song_frame(float(z), step, last)[0] for z in plan})),
        "audio_side_s": round(audio_s, 2),
        "fps": round(frames / (total_ms / 1e3), 1),
        "fields_ms": round(fields_ms, 2), "frames_ms": round(frames_ms, 2),
        "frames_wall_ms": round(frames_wall_ms, 2),
        "per_frame_ms": round(frames_ms / frames, 4),
        "iteration_share": round(fields_ms / total_ms, 4), "colour_share": round(frames_ms / total_ms, 4),
        "tile_gpixel_iter_per_s": round(iterations / (fields_ms * 1e-3) / 1e9, 1),
        "tile_pixel_iterations": iterations, "reference_creation_s": round(reference_s, 2),
        "readback": "none (RGB8 stays in device memory)",
        "fps_with_nv12_handoff": round(frames / ((fields_ms + handoff_wall_ms) / 1e3), 1),
        "handoff_wall_ms": round(handoff_wall_ms, 2)}))
    return 0


def main() -> int:
    parser = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=4)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--form", choices=["chosen", "plain"], default="chosen")
    parser.add_argument("--workload", choices=sorted(WORKLOADS), default=HEADLINE)
    parser.add_argument("--headline-only", action="store_true",
                        help="skip the 55-keyframe stack measured beside the 1e100 atlas")
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--dry-run", action="store_true",
                        help="replica bookkeeping only: each rank joins the group (gloo), prints its rank and "
                             "the max over ranks, and exits")
    parser.add_argument("--frame-passes", action="store_true",
                        help="time the per-frame 4K passes (atlas compositor, colour) and exit")
    parser.add_argument("--song", action="store_true",
                        help="run the 4K60 song workload (all atlas tiles, then every frame) and exit")
    parser.add_argument("--song-seconds", type=float, default=180.0)
    parser.add_argument("--frame-zoom", type=float, default=1.7,
                        help="parent zoom of the timed atlas frame (child fraction = zoom / 4)")
    parser.add_argument("--case", default=None,
                        choices=["direct_levels_4_13_960x540", "direct_levels_0_3_960x540", "deep_levels_12_960x540",
                                 "stack_step_fhd", "atlas_e100_step_fhd", "atlas_e100_deep_24_960x540",
                                 "atlas_e100_shallow_960x540", "costnet_predict_20992", "kfp_colour_3840x2160",
                                 "aurora_colour_3840x2160", "atlas_colour_3840x2160"],
                        help="run one fixed piece of the workload for a profiler capture and exit")
    args = parser.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ and not (args.case or args.frame_passes or args.song):
        return launch_replicas(sys.argv[1:], args.gpus)
    if args.dry_run:
        return run_dry(args)
    if args.case:
        return run_case(args.case)
    if args.frame_passes:
        return run_frame_passes(args)
    if args.song:
        return run_song(args)
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
