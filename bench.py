"""Benchmark of the srp draw path on GB300.

Workload (one "step" = one frame): the ~2M-triangle soup of random geodesic
spheres at 1920x1080 (1024^2 random texture, scissor = central 80%, stencil
INCR on depth pass, depth LESS, mixed perspective/affine/flat varyings),
followed by 100k lines and 100k points -- three srp draw calls.

  value   Mfrag/s with vertex/index data already resident in HBM; the frame's
          draws are timed with CUDA events on the library's stream, the L2 is
          flushed and the framebuffer re-initialised between frames, outside
          the events.
  e2e     the same frame through the public API from host memory, frames
          back to back: each frame copies its vertex and index bytes in with
          srpGpuVertexBufferCopyDataAsync / srpGpuIndexBufferCopyDataAsync and
          reads its framebuffer planes back with srpGpuFramebufferSyncAsync,
          all inside the timed region, which ends with srpGpuSynchronize.
          Beside it: one wait per frame, and the reference's own copy calls
          (srpVertexBufferCopyData / srpIndexBufferCopyData).
A fragment is a pixel that passed coverage and the scissor test (before depth
and stencil), counted the same way by the CPU oracle.

  roofline  the frame's algorithmic bytes (vertex and index bytes, the three
            framebuffer planes read and written once, the texture once) over
            the frame time, against the measured HBM copy bandwidth;
            stage_roofline splits them by stage, with the resolve stage's
            intermediate bytes and measured DRAM traffic beside its share.

At N = 1 the line also carries the other configurations, each measured after
the frame on its own scenes (--frame-only leaves them out):
  batch          4096 independent scenes through srpGpuDrawBatch (scenes/s)
  learned        the frame shaded by the marble shader, plain against its
                 learned MLP stand-in, alone and with the 40 dB judge
  batch_learned  the batch with the marble shader and its stand-in

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's algorithm on the host cores: the CPU
oracle (a restatement of the reference, bit-identical to it) rendering the
same frame, one process per core. N > 1 runs independent replicas (the path
does not shard across GPUs within a frame).
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SCENE = "soup"
SEED = 1
WORKLOAD = "soup: 2.0M-triangle geodesic-sphere soup, 1920x1080, 100k lines, 100k points"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def replica_throughput(local_ms, local_units, world, device):
    """Whole-job throughput of independent replicas, one per rank: the units
    every rank processed over the slowest rank's time. Returns (units per
    second, that time in ms). With world > 1 it takes a process group; the
    reduction carries only the two numbers, never frame data."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
        u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        local_ms, local_units = float(t.item()), float(u.item())
    return local_units / (local_ms / 1000.0), local_ms


FRAME_TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "frame_traffic_soup.md")


def profile_figure(key, scale):
    """A per-frame DRAM byte count of the full-size frame from the committed
    ncu summary (cold-cache bytes of each kernel captured on the half-size
    frame, scaled); None for any other size or when it is missing."""
    if scale != 1.0:
        return None
    try:
        with open(FRAME_TRAFFIC_PROFILE) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


def frame_traffic(scale):
    """DRAM bytes (read + write) of all the frame's kernels per frame."""
    return profile_figure("traffic_bytes_per_frame", scale)


def resolve_traffic(scale):
    """DRAM bytes (read + write) of the resolve stage's kernels per frame."""
    return profile_figure("resolve_traffic_bytes_per_frame", scale)


# NVML clock-event reason bits (nvml.h, nvmlClocksEventReason*)
NVML_REASONS = [(0x8, "hw_slowdown"), (0x40, "hw_thermal_slowdown"), (0x20, "sw_thermal_slowdown"),
                (0x4, "sw_power_cap"), (0x80, "hw_power_brake_slowdown")]


def clock_sampler_main(argv):
    """The clock-sampling child process: reads the SM clock, its maximum and
    the clock-event reasons of one GPU through NVML (read-only queries) every
    `period` seconds and prints `monotonic_s,sm_mhz,max_mhz,reasons,power_mw`
    lines until killed. Exits 3 when NVML cannot be used."""
    bus, index, period = argv[0], int(argv[1]), float(argv[2])
    try:
        nvml = ctypes.CDLL("libnvidia-ml.so.1")
        if nvml.nvmlInit_v2() != 0:
            sys.exit(3)
        h = ctypes.c_void_p()
        if not bus or nvml.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(h)) != 0:
            if nvml.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(h)) != 0:
                sys.exit(3)
        reasons_fn = getattr(nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nvml.nvmlDeviceGetCurrentClocksThrottleReasons
    except (OSError, AttributeError):
        sys.exit(3)
    sm, mx, rs, pw = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong(), ctypes.c_uint()
    i = 0
    while True:
        t = time.monotonic()
        ok = nvml.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0  # NVML_CLOCK_SM
        ok = ok and nvml.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0
        ok = ok and reasons_fn(h, ctypes.byref(rs)) == 0
        if i % 20 == 0 and nvml.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw)) != 0:
            pw.value = 0
        if ok:
            sys.stdout.write(f"{t:.6f},{sm.value},{mx.value},{rs.value},{pw.value}\n")
            sys.stdout.flush()
        i += 1
        time.sleep(period)


class ClockSampler:
    """Samples the SM clock and the throttle reasons of the GPU while the
    bench runs: a child process polls NVML every millisecond (nvidia-smi's
    100 ms loop where NVML cannot be loaded). start() returns once the first
    sample is in; begin() and end() mark the timed region, and stop() reports
    the samples taken inside it."""

    def __init__(self, index):
        self.index, self.samples, self.proc = index, [], None
        self.t0 = self.t1 = None
        self.source = None
        self.first = threading.Event()

    def _bus_id(self):
        try:
            import torch
            p = torch.cuda.get_device_properties(self.index)
            return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
        except Exception:
            return ""

    def start(self):
        cmd = [sys.executable, os.path.abspath(__file__), "--clock-sampler", self._bus_id(), str(self.index), "0.001"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvml"
            self.thread = threading.Thread(target=self._read_nvml, daemon=True)
            self.thread.start()
            self.first.wait(timeout=10)
            if self.proc.poll() is not None:
                self._start_smi()
                self.first.wait(timeout=10)
        except Exception:
            self.proc, self.source = None, None

    def _start_smi(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.source = "nvidia-smi"
        self.thread = threading.Thread(target=self._read_smi, daemon=True)
        self.thread.start()

    @staticmethod
    def parse_nvml(line):
        """(time, sm_mhz, max_mhz, reasons, power_w) of a line of the NVML
        child, or None if it does not parse."""
        try:
            t, sm, mx, rs, pw = line.strip().split(",")
            bits = int(rs)
            return (float(t), float(sm), float(mx), [n for b, n in NVML_REASONS if bits & b], float(pw) / 1000.0)
        except ValueError:
            return None

    @staticmethod
    def parse_smi(line, t):
        """The same for a csv line of nvidia-smi, taken at time t."""
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        s = [x.strip() for x in line.split(",")]
        try:
            return (t, float(s[0]), float(s[1]), [n for n, v in zip(names, s[3:7]) if v.lower().startswith("active")],
                    float(s[2]))
        except (ValueError, IndexError):
            return None

    def _read_nvml(self):
        for line in self.proc.stdout:
            x = self.parse_nvml(line)
            if x:
                self.samples.append(x)
                self.first.set()

    def _read_smi(self):
        for line in self.proc.stdout:
            x = self.parse_smi(line, time.monotonic())
            if x:
                self.samples.append(x)
                self.first.set()

    def begin(self):
        self.t0 = time.monotonic()

    def end(self):
        self.t1 = time.monotonic()

    def stop(self):
        if self.t1 is None:
            self.end()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=5)
        t0 = self.t0 if self.t0 is not None else float("-inf")
        inside = [x for x in list(self.samples) if t0 <= x[0] <= self.t1]
        sm = sorted(x[1] for x in inside)
        power = sorted(x[4] for x in inside if x[4] > 0)
        reasons = sorted({r for x in inside for r in x[3]})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max((x[2] for x in inside), default=None),
                "sm_min_mhz": sm[0] if sm else None,
                "power_w": power[len(power) // 2] if power else None,
                "reasons": reasons, "samples": len(sm), "source": self.source,
                "window_ms": round((self.t1 - self.t0) * 1e3, 2) if self.t0 is not None else None}


def host_cpu():
    """The host CPU's model name (lscpu) and the number of cores the process sees."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return {"model": model or platform.machine(), "nproc": os.cpu_count()}


def cpu_frame(scale, frames, seed=SEED):
    exe = os.path.join(ROOT, "oracle", "_build", "port_scenes")
    out = subprocess.check_output([exe, "time", SCENE, str(seed), repr(float(scale)), str(frames)]).decode()
    return json.loads(out.strip().splitlines()[-1])


def run_reference(args):
    """The reference algorithm (CPU oracle) on all host cores, one frame per
    core per step."""
    import concurrent.futures as cf
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from srp_gb300.build import build_oracle
    build_oracle()
    cores = os.cpu_count() or 1
    frames = max(1, args.warmup + args.steps)
    t0 = time.perf_counter()
    # every core renders the same frame (seed and size of the GPU line)
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        res = list(ex.map(lambda i: cpu_frame(args.scale, frames, SEED), range(cores)))
    wall = time.perf_counter() - t0
    # throughput over the timed frames: each worker reports its mean frame time
    frags = res[0]["fragments"]
    per_core_fps = [1.0 / r["mean_s"] for r in res]
    value = frags * sum(per_core_fps) / 1e6
    mean_s = sum(r["mean_s"] for r in res) / cores
    line = {"impl": "reference", "metric": "Mfrag/s", "value": round(value, 3), "unit": "Mfrag/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000.0 * mean_s / cores, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "seed": SEED, "width": res[0]["width"], "height": res[0]["height"],
                       "triangles": res[0]["triangles"], "lines": res[0]["lines"], "points": res[0]["points"],
                       "fragments_per_frame": frags, "frames_per_s": round(sum(per_core_fps), 2),
                       "mtri_per_s": round(res[0]["triangles"] * sum(per_core_fps) / 1e6, 2)},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mfrag/s", "cores": cores, "kind": "port",
                             "host": host_cpu(),
                             "sample": f"{frames} full frames per core, {cores} processes, wall {wall:.1f}s"},
            "e2e": {"value": round(value, 3), "unit": "Mfrag/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


BATCH_BASE = 11
BATCH_SCENES = 4096
BATCH_WORKLOAD = ("batch: 4096 scenes, one textured Blinn-Phong mesh each (12-200k triangles, log-uniform), "
                  "framebuffers 64-1024 per side (log-uniform), one srpGpuDrawBatch call")


def cpu_batch_sample(scale, count, first=0):
    """The oracle rendering scenes first..first+count-1 of the batch, one at a
    time on one core: (seconds, fragments, scenes)."""
    from srp_gb300 import batch_seed
    exe = os.path.join(ROOT, "oracle", "_build", "port_scenes")
    secs, frags = 0.0, 0
    for i in range(first, first + count):
        out = subprocess.check_output([exe, "time", "bscene", str(batch_seed(BATCH_BASE, i)), repr(float(scale)), "1"])
        r = json.loads(out.decode().strip().splitlines()[-1])
        secs += r["mean_s"]
        frags += r["fragments"]
    return secs, frags, count


def run_reference_batch(args):
    """The reference algorithm (CPU oracle) on all host cores over a sample of
    the batch, one scene per task."""
    import concurrent.futures as cf
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from srp_gb300.build import build_oracle
    build_oracle()
    cores = os.cpu_count() or 1
    sample = min(args.scenes, 16 * cores)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        res = list(ex.map(lambda i: cpu_batch_sample(args.scale, 1, i), range(sample)))
    wall = time.perf_counter() - t0
    frags = sum(r[1] for r in res)
    value = sample / wall
    line = {"impl": "reference", "metric": "scenes/s", "value": round(value, 3), "unit": "scenes/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000.0 * wall * args.scenes / sample, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD, "scenes": args.scenes, "mfrag_per_s": round(frags / wall / 1e6, 3)},
            "cpu_baseline": {"value": round(value, 3), "unit": "scenes/s", "cores": cores, "kind": "port",
                             "sample": f"scenes 0..{sample - 1} of the batch, {cores} threads, wall {wall:.1f}s"},
            "e2e": {"value": round(value, 3), "unit": "scenes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_batch(args, emit=True):
    """The batched-scenes workload: all scenes drawn by one srpGpuDrawBatch
    call per step (multi-draw passes). Returns the line; prints it if emit."""
    import ctypes
    import torch
    import srp_gb300

    srp_gb300.build()
    L = srp_gb300.lib()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    stream = torch.cuda.Stream()
    L.srpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    t0 = time.perf_counter()
    batch = [srp_gb300.Scene("bscene", srp_gb300.batch_seed(BATCH_BASE, i), args.scale) for i in range(args.scenes)]
    gen_s = time.perf_counter() - t0
    fbs = [sc.fb for sc in batch]
    tris = sum(sc.info.inputTriangles for sc in batch)
    pixels = sum(sc.info.width * sc.info.height for sc in batch)
    h2d = sum(sc.info.vertexBytes + sc.info.indexBytes for sc in batch)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def prepare():
        srp_gb300.prepare_batch(batch, fbs)

    tuning = None
    if not args.no_autotune:
        with torch.cuda.stream(stream):
            prepare()
            t0 = time.perf_counter()
            best = srp_gb300.autotune_batch(batch, fbs, 1)
            tuning = {"heavy_items": best.heavyItems, "heavy_ctas_per_sm": best.heavyCtasPerSM,
                      "autotune_s": round(time.perf_counter() - t0, 2)}

    for _ in range(max(args.warmup, 1)):
        with torch.cuda.stream(stream):
            prepare()
            srp_gb300.render_batch(batch, fbs)
    torch.cuda.synchronize()
    L.srpGpuResetStats()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    times = []
    clocks.begin()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            prepare()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            srp_gb300.render_batch(batch, fbs)
            e1.record(stream)
        stream.synchronize()
        times.append(e0.elapsed_time(e1))
    clocks.end()
    st = srp_gb300.SRPGpuStats()
    L.srpGpuGetStats(ctypes.byref(st))
    frags = st.fragments / max(args.steps, 1)
    clk = clocks.stop()
    # end to end through the public API: every scene's geometry up from pinned
    # host memory and its three framebuffer planes back, with the
    # stream-ordered transfers and one wait per step: the Batch calls (gather
    # kernels), and one call per buffer beside them
    def e2e_steps(batch_calls):
        out = []
        for it in range(1 + max(3, args.steps)):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            if batch_calls:
                srp_gb300.upload_batch(batch)
            else:
                for sc in batch:
                    sc.upload_async()
            prepare()
            srp_gb300.render_batch(batch, fbs)
            if batch_calls:
                srp_gb300.sync_batch(fbs)
            else:
                for sc in batch:
                    sc.sync_async()
            if L.srpGpuSynchronize() != 0:
                raise RuntimeError("srpGpuSynchronize failed")
            if it:  # the first pass is an untimed warm-up
                out.append(time.perf_counter() - t1)
        return out

    e2e = e2e_steps(True)
    e2e_calls = e2e_steps(False)

    # Steps back to back with the Batch calls and one srpGpuSynchronize at
    # the end: with one copy of the batch (step n+1's uploads follow step n's
    # draws), and with two (a second batch of the same seeds; step n+1's
    # uploads are issued before step n's draws, and run beside them).
    def e2e_stream(batches, nsteps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if len(batches) > 1:
            srp_gb300.upload_batch(batches[0])
        for i in range(nsteps):
            cur = batches[i % len(batches)]
            if len(batches) == 1:
                srp_gb300.upload_batch(cur)
            elif i + 1 < nsteps:
                srp_gb300.upload_batch(batches[(i + 1) % len(batches)])
            cur_fbs = [sc.fb for sc in cur]
            srp_gb300.prepare_batch(cur, cur_fbs)
            srp_gb300.render_batch(cur, cur_fbs)
            srp_gb300.sync_batch(cur_fbs)
        if L.srpGpuSynchronize() != 0:
            raise RuntimeError("srpGpuSynchronize failed after the streamed steps")
        return (time.perf_counter() - t1) / nsteps

    n_stream = max(4, args.steps)
    e2e_stream((batch,), 2)  # untimed warm-up
    e2e_one_copy = e2e_stream((batch,), n_stream)
    batch_b = [srp_gb300.Scene("bscene", srp_gb300.batch_seed(BATCH_BASE, i), args.scale) for i in range(args.scenes)]
    e2e_stream((batch, batch_b), 2)  # untimed warm-up
    e2e_prefetch = e2e_stream((batch, batch_b), n_stream)
    # both copies hold the same scenes: spot-check that their images agree
    for i in list(range(32)) + list(range(args.scenes - 32, args.scenes)):
        for x, y in zip(srp_gb300.framebuffer_arrays(batch[i].fb), srp_gb300.framebuffer_arrays(batch_b[i].fb)):
            if x.tobytes() != y.tobytes():
                raise RuntimeError(f"the double-buffered batches differ at scene {i}")
    for sc in batch_b:
        sc.close()
    del batch_b
    L.srpGpuSetProfiling(1)
    L.srpGpuResetProfile()
    with torch.cuda.stream(stream):
        prepare()
        srp_gb300.render_batch(batch, fbs)
    prof = srp_gb300.SRPGpuProfile()
    L.srpGpuGetProfile(ctypes.byref(prof))
    L.srpGpuSetProfiling(0)
    stage_ms = {n: prof.ms[i] for i, n in enumerate(srp_gb300.STAGES)}
    total_ms = sum(times)
    step_s = total_ms / args.steps / 1000.0
    peak, peak_kind = peaks()
    tex = sum(sc.info.textureBytes for sc in batch)
    # algorithmic bytes of a step: every scene's vertex and index bytes, its
    # colour and depth planes read and written, its texture once
    algo_bytes = h2d + pixels * 8 * 2 + tex
    step_gbs = algo_bytes / step_s / 1e9
    e2e_s = sum(e2e) / len(e2e)
    line = {
        "metric": "scenes/s", "value": round(args.scenes / step_s, 2), "unit": "scenes/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "scenes": args.scenes, "scale": args.scale, "triangles": tris,
                   "pixels": pixels, "fragments_per_step": frags, "mfrag_per_s": round(frags / step_s / 1e6, 1),
                   "mtri_per_s": round(tris / step_s / 1e6, 1), "generation_s": round(gen_s, 1),
                   "l2": "flushed between steps (256 MB write)", "tuning": tuning},
        "clocks": clk,
        "e2e": {"value": round(args.scenes / e2e_prefetch, 2), "unit": "scenes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(pixels * 9), "steps": n_stream,
                "ms_per_step": round(e2e_prefetch * 1e3, 3),
                "transfers": "srpGpuVertexBufferCopyDataBatchAsync / srpGpuIndexBufferCopyDataBatchAsync / "
                             "srpGpuFramebufferSyncBatchAsync (gather kernels); one srpGpuSynchronize after all steps",
                "prefetch": "two copies of the batch (same seeds): step n+1's uploads are issued before step n's draws",
                "one_copy": round(args.scenes / e2e_one_copy, 2),
                "one_wait_per_step": round(args.scenes / e2e_s, 2),
                "one_wait_per_step_per_buffer_calls": round(args.scenes / (sum(e2e_calls) / len(e2e_calls)), 2)},
        "gpu_launches": int(st.kernelLaunches),
        "roofline": {"bound": "hbm", "achieved": round(step_gbs, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(step_gbs / peak, 5), "traffic": None,
                     "kernel": "the whole batch: every kernel of srpGpuDrawBatch, timed as one step",
                     "algorithmic_bytes_per_step": int(algo_bytes),
                     "basis": "vertex + index bytes + colour and depth planes read and written + textures",
                     "resolve_intermediate_bytes_per_step": int(prof.resolveItems * 68 + pixels * 14),
                     "note": f"peak {peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "stages_ms_per_step": {k: round(v, 3) for k, v in stage_ms.items()},
    }
    if not args.no_cpu_baseline:
        from srp_gb300.build import build_oracle
        build_oracle()
        secs, cfr, cnt = cpu_batch_sample(args.scale, 48)
        line["cpu_baseline"] = {"value": round(cnt / secs, 3), "unit": "scenes/s", "cores": 1, "kind": "port",
                                "sample": f"scenes 0..{cnt - 1} of the batch on 1 host core, "
                                          f"{round(cfr / secs / 1e6, 2)} Mfrag/s"}
    if emit:
        print(json.dumps(line))
    for sc in batch:
        sc.close()
    return line


LEARNED_WORKLOAD = ("learned: 2.0M-triangle geodesic-sphere soup at 1920x1080 shaded by 8-octave value-noise "
                    "marble with 16 point lights (srpFsMarble), against its learned MLP stand-in")
# the 32 training scenes' size: about 4M shaded fragments in all
LEARNED_CAPTURE_SCALE = 0.24


def capture(L, net, marble, scenes, scale):
    """Every pixel the marble shader shades in `scenes` training scenes
    (seeds 1000 on, none of them the held-out frame's) becomes a sample of
    `net`."""
    import srp_gb300
    L.srpGpuMlpCapture(net, marble, 1)
    for i in range(scenes):
        sc = srp_gb300.Scene("msoup", 1000 + i, scale)
        sc.prepare()
        sc.render()
        sc.close()
    L.srpGpuMlpCapture(None, None, 0)


def covered_psnr(img, ref, covered):
    """PSNR (dB) over the covered pixels of packed RGBA8 planes, channels in [0, 1]."""
    import numpy as np
    def rgb(c):
        c = c[covered].astype(np.int64)
        return np.stack([(c >> 24) & 255, (c >> 16) & 255, (c >> 8) & 255], -1) / 255.0
    mse = float(((rgb(img) - rgb(ref)) ** 2).mean())
    return round(10.0 * math.log10(1.0 / mse), 2) if mse > 0 else None


def learned_quality(L, marble, net, scale):
    """PSNR of the held-out frame over its covered pixels against the 8-octave
    marble shader's own image: for the trained network (no fallback), for no
    network (every pixel the reference's mean colour), for the one-octave
    level of detail of the shader (msoup_lod), and for networks trained on
    fewer steps or fewer fragments."""
    import numpy as np
    import srp_gb300

    def frame(name, learned_net):
        sc = srp_gb300.Scene(name, SEED, scale)
        try:
            if learned_net:
                L.srpGpuSetLearnedShading(marble, learned_net, 0.0, 64)
            sc.prepare()
            sc.render()
            return [a.copy() for a in sc.planes()]
        finally:
            L.srpGpuSetLearnedShading(None, None, 0.0, 0)
            sc.close()

    ref = frame("msoup", None)
    covered = ref[1] != ref[1][0]
    c = ref[0][covered].astype(np.int64)
    mean = [int(round(float(((c >> s) & 255).mean()))) for s in (24, 16, 8)]
    const = np.full_like(ref[0], (mean[0] << 24) | (mean[1] << 16) | (mean[2] << 8) | 255)
    out = {"covered_pixels": int(covered.sum()),
           "network": covered_psnr(frame("msoup", net)[0], ref[0], covered),
           "constant_colour": covered_psnr(const, ref[0], covered),
           "one_octave_shader": covered_psnr(frame("msoup_lod", None)[0], ref[0], covered)}
    sweep = []
    for scenes, steps in ((32, 500), (32, 1500), (32, 6000), (8, 3000), (16, 3000)):
        n2 = L.srpGpuMlpCreate(11, 4 << 20)
        try:
            capture(L, n2, marble, scenes, LEARNED_CAPTURE_SCALE)
            samples = L.srpGpuMlpSampleCount(n2)
            L.srpGpuMlpTrain(n2, steps, 16384, 2e-3)
            sweep.append({"scenes": scenes, "samples": samples, "steps": steps,
                          "psnr_db": covered_psnr(frame("msoup", n2)[0], ref[0], covered)})
        finally:
            L.srpGpuMlpFree(n2)
    out["network_sweep"] = sweep
    return out


class LearnedStats(ctypes.Structure):
    """SRPGpuLearnedStats of srp/gpu.h."""
    _fields_ = [("draws", ctypes.c_uint64), ("fallbacks", ctypes.c_uint64), ("judgedDraws", ctypes.c_uint64),
                ("judgedChannels", ctypes.c_uint64), ("squaredError", ctypes.c_double),
                ("lastPsnrDb", ctypes.c_double), ("minPsnrDb", ctypes.c_double), ("maxChannelError", ctypes.c_float),
                ("psnrHistogram", ctypes.c_uint64 * 6)]


MLP_FLOPS_PER_FRAGMENT = 2 * (108 * 64 + 64 * 64 + 64 * 64 + 64 * 3)


def tensor_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def run_learned(args, emit=True):
    """Train the learned stand-in of the marble shader on fragments of 32
    training scenes, then time a held-out full-size frame shaded by the
    shader, by the network alone, and by the network with the judge's
    40 dB fallback. Returns the line; prints it if emit."""
    import ctypes
    import torch
    import srp_gb300

    srp_gb300.build()
    L = srp_gb300.lib()
    vp = ctypes.c_void_p
    marble = learned_api(L)
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    stream = torch.cuda.Stream()
    L.srpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    net = L.srpGpuMlpCreate(7, 4 << 20)
    # training data: every shaded pixel of 32 smaller scenes (other seeds),
    # about 4M fragments
    t0 = time.perf_counter()
    capture(L, net, marble, 32, LEARNED_CAPTURE_SCALE)
    samples = L.srpGpuMlpSampleCount(net)
    capture_s = time.perf_counter() - t0
    steps, batch = args.train_steps, 16384
    t0 = time.perf_counter()
    final_mse = L.srpGpuMlpTrain(net, steps, batch, 2e-3)
    train_s = time.perf_counter() - t0
    sc = srp_gb300.Scene("msoup", SEED, args.scale)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(frames):
        ms, shade = [], []
        for _ in range(frames):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                sc.prepare()
                L.srpGpuSetProfiling(1)
                L.srpGpuResetProfile()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sc.render()
                e1.record(stream)
            stream.synchronize()
            prof = srp_gb300.SRPGpuProfile()
            L.srpGpuGetProfile(ctypes.byref(prof))
            L.srpGpuSetProfiling(0)
            ms.append(e0.elapsed_time(e1))
            shade.append(prof.ms[4])
        return sorted(ms)[len(ms) // 2], sorted(shade)[len(shade) // 2]

    L.srpGpuResetStats()
    for _ in range(max(args.warmup, 1)):
        sc.prepare()
        sc.render()
    torch.cuda.synchronize()
    L.srpGpuResetStats()
    sc.prepare()
    depth_before = sc.planes()[1]
    sc.render()
    st = srp_gb300.SRPGpuStats()
    L.srpGpuGetStats(ctypes.byref(st))
    frags = st.fragments
    # pixels the shading stage colours: those whose depth the draw wrote
    shaded = int((sc.planes()[1] != depth_before).sum())
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    clocks.begin()
    plain_ms, plain_shade = timed(args.steps)
    L.srpGpuSetLearnedShading(marble, net, 0.0, 64)
    for _ in range(2):
        sc.prepare()
        sc.render()
    L.srpGpuResetLearnedStats()
    mlp_ms, mlp_shade = timed(args.steps)
    ls = LearnedStats()
    L.srpGpuGetLearnedStats(ctypes.byref(ls))
    psnr = 10.0 * math.log10(ls.judgedChannels / ls.squaredError) if ls.squaredError > 0 else None
    L.srpGpuSetLearnedShading(marble, net, 40.0, 64)
    L.srpGpuResetLearnedStats()
    judged_ms, judged_shade = timed(args.steps)
    lj = LearnedStats()
    L.srpGpuGetLearnedStats(ctypes.byref(lj))
    L.srpGpuSetLearnedShading(None, None, 0.0, 0)
    clk = clocks.stop()
    mfr = lambda ms: round(frags / (ms / 1000.0) / 1e6, 1)
    line = {
        "metric": "Mfrag/s", "value": mfr(judged_ms), "unit": "Mfrag/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(judged_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (network), f32 (rest)", "data": "synthetic",
        "config": {"workload": LEARNED_WORKLOAD, "seed": SEED, "fragments_per_frame": frags,
                   "training": {"scenes": 32, "scene_scale": LEARNED_CAPTURE_SCALE, "samples": samples,
                                "capture_s": round(capture_s, 2),
                                "steps": steps, "batch": batch, "train_s": round(train_s, 2),
                                "final_batch_mse": round(final_mse, 6)}},
        "plain": {"ms_per_frame": round(plain_ms, 4), "Mfrag_per_s": mfr(plain_ms), "shade_ms": round(plain_shade, 4)},
        "learned_no_fallback": {"ms_per_frame": round(mlp_ms, 4), "Mfrag_per_s": mfr(mlp_ms),
                                "shade_ms": round(mlp_shade, 4),
                                "psnr_db": round(psnr, 2) if psnr else None,
                                "max_channel_error": round(float(ls.maxChannelError), 4)},
        "learned_with_judge_40db": {"ms_per_frame": round(judged_ms, 4), "Mfrag_per_s": mfr(judged_ms),
                                    "shade_ms": round(judged_shade, 4), "draws": lj.draws,
                                    "fallbacks": lj.fallbacks},
        "shade_speedup_no_fallback": round(plain_shade / mlp_shade, 3) if mlp_shade > 0 else None,
        "clocks": clk,
        "gpu_launches": int(st.kernelLaunches),
    }
    line["quality_psnr_db"] = learned_quality(L, marble, net, args.scale)
    if shaded and mlp_shade > 0:
        tpk, tkind = tensor_peak()
        tflops = shaded * MLP_FLOPS_PER_FRAGMENT / (mlp_shade / 1000.0) / 1e12
        line["roofline"] = {"bound": "tensor", "achieved": round(tflops, 2), "peak": tpk, "unit": "TFLOP/s",
                            "frac": round(tflops / tpk, 5), "traffic": None,
                            "kernel": "learned shading stage (k_shade_learned5), network alone",
                            "flops_per_frame": shaded * MLP_FLOPS_PER_FRAGMENT, "shaded_pixels": shaded,
                            "note": f"peak {tkind} (MEASURED_PEAKS.json bf16_tflops)"}
    if emit:
        print(json.dumps(line))
    sc.close()
    L.srpGpuMlpFree(net)
    return line


BATCH_LEARNED_WORKLOAD = ("batch-learned: the 4096-scene batch shaded by 8-octave value-noise marble with 16 point "
                          "lights (srpFsMarble), against its learned MLP stand-in with per-draw judging")


def learned_api(L):
    vp = ctypes.c_void_p
    L.srpGpuMlpCreate.restype = vp
    L.srpGpuMlpCreate.argtypes = [ctypes.c_uint64, ctypes.c_size_t]
    L.srpGpuMlpFree.argtypes = [vp]
    L.srpGpuMlpCapture.argtypes = [vp, vp, ctypes.c_uint32]
    L.srpGpuMlpSampleCount.restype = ctypes.c_size_t
    L.srpGpuMlpSampleCount.argtypes = [vp]
    L.srpGpuMlpTrain.restype = ctypes.c_float
    L.srpGpuMlpTrain.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    L.srpGpuSetLearnedShading.argtypes = [vp, vp, ctypes.c_float, ctypes.c_uint32]
    L.srpGpuGetLearnedStats.argtypes = [ctypes.POINTER(LearnedStats)]
    return ctypes.cast(L.srpFsMarble, vp)


def run_batch_learned(args, emit=True):
    """The batch of run_batch with the marble shader: trained on fragments of
    512 other scenes, then timed plain, learned, and learned with the 40 dB
    per-draw fallback. Returns the line; prints it if emit."""
    import torch
    import srp_gb300

    srp_gb300.build()
    L = srp_gb300.lib()
    marble = learned_api(L)
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    stream = torch.cuda.Stream()
    L.srpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    net = L.srpGpuMlpCreate(7, 4 << 20)
    t0 = time.perf_counter()
    train = [srp_gb300.Scene("bmscene", srp_gb300.batch_seed(31, i), args.scale) for i in range(512)]
    L.srpGpuMlpCapture(net, marble, 4)
    for sc in train:
        sc.prepare()
    srp_gb300.render_batch(train, [sc.fb for sc in train])
    L.srpGpuMlpCapture(None, None, 0)
    samples = L.srpGpuMlpSampleCount(net)
    for sc in train:
        sc.close()
    capture_s = time.perf_counter() - t0
    steps, batch = args.train_steps, 16384
    t0 = time.perf_counter()
    final_mse = L.srpGpuMlpTrain(net, steps, batch, 2e-3)
    train_s = time.perf_counter() - t0
    batchs = [srp_gb300.Scene("bmscene", srp_gb300.batch_seed(BATCH_BASE, i), args.scale) for i in range(args.scenes)]
    fbs = [sc.fb for sc in batchs]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed():
        ms = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                for sc in batchs:
                    sc.prepare()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                srp_gb300.render_batch(batchs, fbs)
                e1.record(stream)
            stream.synchronize()
            ms.append(e0.elapsed_time(e1))
        return sorted(ms)[len(ms) // 2]

    for _ in range(max(args.warmup, 1)):
        for sc in batchs:
            sc.prepare()
        srp_gb300.render_batch(batchs, fbs)
    torch.cuda.synchronize()
    L.srpGpuResetStats()
    for sc in batchs:
        sc.prepare()
    srp_gb300.render_batch(batchs, fbs)
    st = srp_gb300.SRPGpuStats()
    L.srpGpuGetStats(ctypes.byref(st))
    frags = st.fragments
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    clocks.begin()
    plain_ms = timed()
    L.srpGpuSetLearnedShading(marble, net, 0.0, 64)
    L.srpGpuResetLearnedStats()
    learned_ms = timed()
    ls = LearnedStats()
    L.srpGpuGetLearnedStats(ctypes.byref(ls))
    L.srpGpuSetLearnedShading(marble, net, 40.0, 64)
    L.srpGpuResetLearnedStats()
    judged_ms = timed()
    lj = LearnedStats()
    L.srpGpuGetLearnedStats(ctypes.byref(lj))
    L.srpGpuSetLearnedShading(None, None, 0.0, 0)
    clk = clocks.stop()
    n = args.scenes
    psnr = 10.0 * math.log10(ls.judgedChannels / ls.squaredError) if ls.squaredError > 0 else None
    rate = lambda ms: {"ms_per_batch": round(ms, 3), "scenes_per_s": round(n / (ms / 1000.0), 1),
                       "Mfrag_per_s": round(frags / (ms / 1000.0) / 1e6, 1)}
    line = {
        "metric": "scenes/s", "value": round(n / (judged_ms / 1000.0), 1), "unit": "scenes/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(judged_ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (network), f32 (rest)", "data": "synthetic",
        "config": {"workload": BATCH_LEARNED_WORKLOAD, "scenes": n, "fragments_per_step": frags,
                   "training": {"scenes": 512, "samples": samples, "capture_s": round(capture_s, 2), "steps": steps,
                                "batch": batch, "train_s": round(train_s, 2), "final_batch_mse": round(final_mse, 6)}},
        "plain": rate(plain_ms),
        "learned_no_fallback": dict(rate(learned_ms), psnr_db=round(psnr, 2) if psnr else None,
                                    psnr_histogram_lt20_20_25_30_35_40_ge40=list(ls.psnrHistogram)),
        "learned_with_judge_40db": dict(rate(judged_ms), draws=lj.draws, fallbacks=lj.fallbacks,
                                        fallback_rate=round(lj.fallbacks / max(lj.draws, 1), 4)),
        "clocks": clk,
    }
    if emit:
        print(json.dumps(line))
    for sc in batchs:
        sc.close()
    L.srpGpuMlpFree(net)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="frame", choices=["frame", "batch", "learned", "batch-learned"],
                    help="frame: the 2M-triangle 1080p frame (default); batch: the batched-scenes workload; "
                         "learned: the marble-shaded frame with its learned stand-in")
    ap.add_argument("--scenes", type=int, default=BATCH_SCENES, help="scenes per batch (--workload batch)")
    ap.add_argument("--train-steps", type=int, default=3000, help="training steps (--workload learned, batch-learned)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default resolve tuning (--workload frame, batch)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every kernel directly instead of replaying captured CUDA graphs (srpGpuSetDrawGraphs(0))")
    ap.add_argument("--tile-copies", type=int, default=None,
                    help="SRP_GPU_TILE_COPY_* bits for srpGpuSetTileCopies (default: the library's)")
    ap.add_argument("--frame-only", action="store_true",
                    help="--workload frame without the batch, learned and batch-learned summaries added to its line")
    args = ap.parse_args()
    if args.workload == "batch":
        return run_reference_batch(args) if args.impl == "reference" else run_batch(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "batch-learned":
        return run_batch_learned(args)
    if args.impl == "reference":
        return run_reference(args)

    import ctypes
    import torch
    import srp_gb300

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    srp_gb300.build()
    L = srp_gb300.lib()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    if args.no_graphs:
        L.srpGpuSetDrawGraphs(0)
    if args.tile_copies is not None:
        L.srpGpuSetTileCopies.argtypes = [ctypes.c_uint]
        L.srpGpuSetTileCopies(args.tile_copies)
    stream = torch.cuda.Stream()
    L.srpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    sc = srp_gb300.Scene(SCENE, SEED + rank, args.scale)
    info = sc.info
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def frame():
        sc.render()

    # warm-up, then the library's online autotuner over whole frames
    for _ in range(max(args.warmup, 1)):
        with torch.cuda.stream(stream):
            sc.prepare()
            frame()
    tuning = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            busy = 1
            while busy:
                # tuned under the conditions of the timed frames below
                flush.fill_(1.0)
                sc.prepare()
                stream.synchronize()
                frame()
                busy = L.srpGpuAutotuneFrame()
        best = srp_gb300.SRPGpuTuning()
        L.srpGpuGetTuning.argtypes = [ctypes.POINTER(srp_gb300.SRPGpuTuning)]
        L.srpGpuGetTuning(ctypes.byref(best))
        tuning = {"heavy_items": best.heavyItems, "heavy_ctas_per_sm": best.heavyCtasPerSM,
                  "autotune_s": round(time.perf_counter() - t0, 2)}
    torch.cuda.synchronize()
    L.srpGpuResetStats()
    st0 = srp_gb300.SRPGpuStats()
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    times = []
    clocks.begin()
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            sc.prepare()
            # the library's front stream (vertex, setup, binning) is not ordered
            # after this stream's earlier work: let the flush and the clear
            # finish first, so that every draw of the frame runs after e0
            stream.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            frame()
            e1.record(stream)
        stream.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clocks.end()
    L.srpGpuGetStats(ctypes.byref(st0))
    frags_per_frame = st0.fragments / max(args.steps, 1)
    launches = st0.kernelLaunches
    clk = clocks.stop()
    # end-to-end through the API from host memory (after the clock sampler has
    # stopped: its nvidia-smi queries stall the host's CUDA calls now and then)
    # Two ways through the API: the stream-ordered uploads (srpGpu*CopyDataAsync,
    # one wait per frame: the headline e2e) and the reference's own calls
    # (srpVertexBufferCopyData / srpIndexBufferCopyData, each waiting for its copy)
    def e2e_frames(upload):
        ts = []
        for it in range(1 + max(5, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            upload()
            sc.prepare()
            frame()
            sc.sync()
            if it:  # the first pass is an untimed warm-up
                ts.append(time.perf_counter() - t0)
        return ts
    e2e_times = e2e_frames(sc.upload_async)
    e2e_sync_times = e2e_frames(sc.upload)

    # Frames back to back through the same calls with one srpGpuSynchronize at
    # the end (the headline e2e): every frame still uploads its vertex and
    # index buffers from host memory and downloads its framebuffer, but frame
    # n+1's uploads and front stages run beside frame n's resolve, shading and
    # download.
    def e2e_stream(nframes):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(nframes):
            sc.upload_async()
            sc.prepare()
            frame()
            sc.sync_async()
        if L.srpGpuSynchronize() != 0:
            raise RuntimeError("srpGpuSynchronize failed after the streamed frames")
        return time.perf_counter() - t0
    e2e_stream(2)  # untimed warm-up
    n_stream = max(10, args.steps)
    e2e_stream_s = e2e_stream(n_stream) / n_stream

    # The same with the frame's buffers double-buffered (a second Scene of the
    # same seed): frame i+1's uploads are issued before frame i's draws, so
    # they run on the copy engine beside frame i instead of after it. Every
    # frame still uploads its 83.6 MB and downloads its planes inside the
    # timed region, which starts before the first upload.
    sc_b = srp_gb300.Scene(SCENE, SEED + rank, args.scale)

    def e2e_prefetch(nframes):
        pair = (sc, sc_b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pair[0].upload_async()
        for i in range(nframes):
            cur = pair[i % 2]
            if i + 1 < nframes:
                pair[(i + 1) % 2].upload_async()
            cur.prepare()
            cur.render()
            cur.sync_async()
        if L.srpGpuSynchronize() != 0:
            raise RuntimeError("srpGpuSynchronize failed after the prefetched frames")
        return time.perf_counter() - t0
    e2e_prefetch(4)  # untimed warm-up
    e2e_prefetch_s = e2e_prefetch(n_stream) / n_stream
    # both copies hold the same frame: their host planes must agree
    for x, y in zip(srp_gb300.framebuffer_arrays(sc.fb), srp_gb300.framebuffer_arrays(sc_b.fb)):
        if x.tobytes() != y.tobytes():
            raise RuntimeError("the double-buffered frames differ")
    sc_b.close()
    # per-stage device time (CUDA events inside the library) on separate frames
    L.srpGpuSetProfiling(1)
    L.srpGpuResetProfile()
    nprof = max(2, min(args.steps, 5))
    for _ in range(nprof):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            sc.prepare()
            frame()
    prof = srp_gb300.SRPGpuProfile()
    L.srpGpuGetProfile(ctypes.byref(prof))
    L.srpGpuSetProfiling(0)
    stage_ms = {n: prof.ms[i] / nprof for i, n in enumerate(srp_gb300.STAGES)}
    stage_launches = {n: prof.launches[i] / nprof for i, n in enumerate(srp_gb300.STAGES)}
    rate, total_ms = replica_throughput(sum(times), frags_per_frame * args.steps, world, "cuda")
    value = rate / 1e6
    e2e_s = sum(e2e_times) / len(e2e_times)
    h2d = info.vertexBytes + info.indexBytes
    d2h = info.width * info.height * 9
    peak, peak_kind = peaks()
    # algorithmic bytes of the frame: every vertex and index byte read once,
    # the colour, depth and stencil planes read and written once (the API
    # keeps them across draws), the texture read once
    px = info.width * info.height
    algo_bytes = info.vertexBytes + info.indexBytes + px * 9 * 2 + info.textureBytes
    frame_gbs = algo_bytes / (total_ms / args.steps / 1000.0) / 1e9
    # each stage's share of those bytes; binning moves only intermediate data
    share = {"vertex": info.vertexBytes, "setup": info.indexBytes, "bin": 0,
             "resolve": px * 5 * 2, "shade": px * 4 * 2 + info.textureBytes}
    dom = max(stage_ms, key=stage_ms.get)
    items = prof.resolveItems / nprof
    stage_roof = {}
    for k, ms in stage_ms.items():
        gbs = share[k] / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
        stage_roof[k] = {"ms": round(ms, 4), "algorithmic_bytes": int(share[k]), "achieved": round(gbs, 1),
                         "frac": round(gbs / peak, 5)}
    # what the resolve reads and writes beyond its share: a (tile, item)
    # pair's index and record (4 + 64 B), the winner plane
    stage_roof["resolve"]["intermediate_bytes"] = int(items * 68 + px * 4)
    stage_roof["resolve"]["traffic"] = resolve_traffic(args.scale)
    line = {
        "metric": "Mfrag/s", "value": round(value, 3), "unit": "Mfrag/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "seed": SEED, "width": info.width, "height": info.height,
                   "graphs": not args.no_graphs, "tile_copies": args.tile_copies,
                   "triangles": info.inputTriangles, "lines": info.inputLines, "points": info.inputPoints,
                   "fragments_per_frame": frags_per_frame, "l2": "flushed between frames (256 MB write)",
                   "tuning": tuning,
                   "frames_per_s": round(args.steps / (total_ms / 1000.0), 2),
                   "mtri_per_s": round(info.inputTriangles * args.steps / (total_ms / 1000.0) / 1e6, 2)},
        "clocks": clk,
        "e2e": {"value": round(frags_per_frame / e2e_prefetch_s / 1e6, 3), "unit": "Mfrag/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "frames": n_stream,
                "ms_per_frame": round(e2e_prefetch_s * 1e3, 4),
                "calls": "per frame srpGpuVertexBufferCopyDataAsync / srpGpuIndexBufferCopyDataAsync, "
                         "framebuffer fill, draws, srpGpuFramebufferSyncAsync; one srpGpuSynchronize after all frames",
                "prefetch": "two copies of the frame's buffers and framebuffer (same seed): frame i+1's uploads "
                            "are issued before frame i's draws",
                "one_copy": round(frags_per_frame / e2e_stream_s / 1e6, 3),
                "one_wait_per_frame": round(frags_per_frame / e2e_s / 1e6, 3),
                "one_wait_per_frame_ms": round(e2e_s * 1e3, 3),
                "with_reference_copy_calls": round(frags_per_frame / (sum(e2e_sync_times) / len(e2e_sync_times)) / 1e6, 3)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": round(frame_gbs, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(frame_gbs / peak, 5), "traffic": frame_traffic(args.scale),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the frame's "
                                       "kernels, " + os.path.relpath(FRAME_TRAFFIC_PROFILE, ROOT),
                     "kernel": "the frame's draw path: every kernel of its three draws, timed as one frame",
                     "algorithmic_bytes_per_frame": int(algo_bytes),
                     "basis": "vertex + index bytes + colour/depth/stencil planes read and written + texture",
                     "dominant_stage": dom,
                     "note": f"peak {peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "stage_roofline": stage_roof,
        "stages_ms_per_frame": {k: round(v, 4) for k, v in stage_ms.items()},
        "stage_launches_per_frame": stage_launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        from srp_gb300.build import build_oracle
        build_oracle()
        r = cpu_frame(1.0, 5)
        line["cpu_baseline"] = {"value": round(r["fragments"] / r["mean_s"] / 1e6, 3), "unit": "Mfrag/s",
                                "cores": 1, "kind": "port", "host": host_cpu(),
                                "sample": "5 full frames of the same workload on 1 host core (mean frame time)"}
    sc.close()
    if rank == 0 and world == 1 and not args.frame_only:
        # the other configurations, each on its own scenes, after the frame
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup, sub.scale = min(args.steps, 5), max(args.warmup, 3), 1.0
        for key, fn in (("batch", run_batch), ("learned", run_learned), ("batch_learned", run_batch_learned)):
            try:
                line[key] = fn(sub, emit=False)
            except Exception as e:  # a failed summary must not hide the frame's line
                line[key] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--clock-sampler":
        clock_sampler_main(sys.argv[2:])
    else:
        main()
