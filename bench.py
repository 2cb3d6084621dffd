"""Throughput benchmark of the GB300 cpSpaceStep drop-in.

Workload (default): 20,000 circles (r ~ U[0.5,2], density 1, u 0.7, e 0.1)
in a 1000x2000 box of 4 static segments, v ~ N(0,5) per axis, gravity
(0,-100), dt 1/60, 10 iterations, seed 1 -- the single-large-space
configuration of the reference's benchmark plan.  A step is one cpSpaceStep.

Metric: body-steps/s = dynamic bodies x timed steps / device seconds.

  value      device time of the timed steps (CUDA events on the library's
             stream), state resident in HBM.
  e2e        the same steps through the public C API as a program uses it:
             cpSpaceStep, then every body's position, velocity and angle read
             back through cpBodyGet* (device->host copy inside the timed
             region), host wall clock.
  roofline   the dominant phase's algorithmic bytes per launch / its mean
             event-timed duration, against the measured HBM copy bandwidth.
  cpu_baseline  the CPU restatement of the same path (oracle/cp_oracle.c,
             "port"), one core, on a bounded sample of the same workload.

--impl reference runs only that CPU implementation, on the same workload
and metric, and prints its own JSON line.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--mode ordered|colored]
                       [--impl ours|reference] [--workload circles|pyramid|mixed|batch|rollout]
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

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

# the configured run length of each single-space workload (steps)
RUN_STEPS = {"circles": 600, "pyramid": 1000, "mixed": 600}


_PINNED = []


def pinned_doubles(n):
    """A numpy view of n doubles of page-locked host memory (the tensor
    that owns it is kept for the life of the run)."""
    import torch
    t = torch.empty(max(n, 1), dtype=torch.float64, pin_memory=True)
    _PINNED.append(t)
    return t.numpy()


def window_start(workload, warmup, steps):
    """First timed step: a K-step sample of a longer configured run is taken
    from its middle (untimed lead-in steps, the W warm-up steps among them),
    so that it costs what the run costs on average rather than its free-fall
    start; a run of K >= the configured length starts after the warm-up."""
    total = RUN_STEPS.get(workload, steps)
    return warmup if steps >= total else max(warmup, (total - steps)//2)


def host_cpu():
    """The host CPU model (lscpu, else /proc/cpuinfo) and its usable threads."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith(("model name", "cpu model")):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"model": model, "threads": cpu_threads()}


WORKLOADS = {
    # name: (scene config, size, dt, description)
    "circles": (2, 20000, 1 / 60, "20000 circles r~U[0.5,2] in a 1000x2000 box, 10 it, dt 1/60, seed 1"),
    "pyramid": (1, 14, 1 / 60, "14-row pyramid of 105 30x30 boxes, 10 it, dt 1/60"),
    "mixed": (3, 30000, 1 / 60, "30000 circles/polys/segments + 500 pivot chains of 20, 15 it, dt 1/60, seed 2"),
}

# Algorithmic bytes per unit (FP64, compulsory traffic) per phase.
BYTES_PER_BODY_POS = 184      # integrate position: read p,v,vb,a,w,wb,cog; write p,a,transform,zeroed bias
BYTES_PER_CIRCLE_CACHE = 120  # shape cache + AABB of a circle
BYTES_PER_BODY_VEL = 104      # integrate velocity
BYTES_PER_CONTACT_PRESTEP = 208
BYTES_PER_CONTACT_ITER = 376  # one sequential-impulse application of one contact


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def oracle_lib():
    so = os.path.join(REPO, "oracle", "_build", "liboracle.so")
    if not os.path.exists(so):
        subprocess.check_call([os.path.join(REPO, "oracle", "build_oracle.sh")], stdout=subprocess.DEVNULL)
    from chipmunk2d_gb300 import bind
    return bind(so)


def cpu_sample(workload, budget_s=15.0, warm=5, hasty_s=0.0):
    """Times the CPU restatement on the workload: `warm` untimed lead-in
    steps, then steps on one thread until about budget_s seconds have been
    spent, then (hasty_s > 0) steps with the solver on two threads as
    cpHastySpace's for about hasty_s seconds.  Returns ((value, steps,
    seconds) one thread, (value, steps, seconds) two threads or None, bodies)."""
    from chipmunk2d_gb300 import Scene
    cfg, size, dt, _ = WORKLOADS[workload]
    lib = oracle_lib()
    sc = Scene(lib, cfg, size)
    sc.step(dt, warm)
    n = sc.nbodies

    def timed(budget):
        steps = 0
        t0 = time.perf_counter()
        while True:
            sc.step(dt, 1)
            steps += 1
            el = time.perf_counter() - t0
            if el >= budget or steps >= 2000:
                return n * steps / el, steps, el

    one = timed(budget_s)
    two = None
    if hasty_s > 0:
        lib.cpx_space_set_hasty(sc.space, 2)
        two = timed(hasty_s)
    sc.free()
    return one, two, n


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_step_worlds(scenes, dt, steps, threads):
    """Steps independent worlds of the CPU implementation on `threads` host
    threads (one world at a time per thread; the ctypes calls release the
    GIL).  Returns the wall seconds."""
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    if threads <= 1:
        for sc in scenes:
            sc.step(dt, steps)
    else:
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda sc: sc.step(dt, steps), scenes))
    return time.perf_counter() - t0


def run_reference_worlds(args):
    """The batch (or the rollout's forward) on the CPU implementation: every
    world of the workload, stepped on all host threads, one world per thread
    at a time."""
    from chipmunk2d_gb300 import Scene
    lib = oracle_lib()
    threads = cpu_threads()
    if args.workload == "batch":
        sizes = batch_sizes(lib, BATCH_WORLDS)
        scenes = [Scene(lib, 4, sizes[i], seed=1000 + i) for i in range(BATCH_WORLDS)]
        dt, steps = BATCH_DT, args.steps
        desc = "4096 tumble worlds, bodies log-uniform in [8,512], 10 it, dt 1/60, seed 3"
    else:
        scenes = _rollout_scenes(lib, range(ROLLOUT_WORLDS))
        dt, steps = ROLLOUT_DT, ROLLOUT_STEPS
        desc = "forward only (the CPU implementation has no adjoint): " + ROLLOUT_DESC
    cpu_step_worlds(scenes, dt, args.warmup, threads)
    secs = cpu_step_worlds(scenes, dt, steps, threads)
    nb = sum(sc.nbodies for sc in scenes)
    for sc in scenes:
        sc.free()
    value = len(scenes) * steps / secs
    line = {
        "impl": "reference", "metric": "world-steps/s", "value": value, "unit": "world-steps/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": args.workload, "description": desc, "worlds": len(scenes), "bodies": nb},
        "body_steps_per_s": nb * steps / secs,
        "cpu_baseline": {"value": value, "unit": "world-steps/s", "cores": threads, "kind": "port",
                         "sample": "every world, %d steps after %d warm-up steps, one world per thread" % (steps, args.warmup)},
        "e2e": {"value": value, "unit": "world-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload in ("batch", "rollout"):
        return run_reference_worlds(args)
    workload = args.workload
    cfg, size, dt, desc = WORKLOADS[workload]
    from chipmunk2d_gb300 import Scene
    lib = oracle_lib()
    sc = Scene(lib, cfg, size)
    n = sc.nbodies
    # the reference's threaded space (cpHastySpace) solves on at most two
    # threads; its restatement in the oracle does the same
    threads = lib.cpx_space_set_hasty(sc.space, 2)
    # the same timed window as the GPU arm: an untimed lead-in to the
    # middle of the configured run
    start = window_start(workload, args.warmup, args.steps)
    sc.step(dt, start)
    # each timed step is a bounded sample: the whole run stays within minutes
    per_step = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sc.step(dt, 1)
        per_step.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > 150.0:
            break
    sc.free()
    k = len(per_step)
    secs = sum(per_step)
    value = n * k / secs
    line = {
        "impl": "reference", "metric": "body-steps/s", "value": value, "unit": "body-steps/s",
        "n_gpus": args.gpus, "steps": k, "warmup": args.warmup, "ms_per_step": 1000 * secs / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": workload, "description": desc, "bodies": n,
                                        "timed_window": [start, start + k], "lead_in_untimed": start},
        "host_cpu": host_cpu(),
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port",
                         "sample": "steps %d-%d of the %s workload (untimed lead-in before), solver on %d threads as cpHastySpace's"
                                   % (start, start + k, workload, threads)},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batch_sizes(lib, count, seed=3):
    import ctypes
    arr = (ctypes.c_int * count)()
    lib.cpx_batch_sizes(count, seed, ctypes.cast(arr, ctypes.c_void_p))
    return list(arr)


BATCH_WORLDS = 4096
BATCH_DT = 1 / 60
BATCH_STEPS = 300     # the workload's run length; the worlds settle into piles, so later steps cost more


def run_batch(args, emit=True, sharded=True):
    """4096 tumble worlds with body counts log-uniform in [8, 512], stepped
    together (cpGpuBatchStep, reference sweep order in every world).  Under
    torchrun each rank steps its contiguous range of worlds (balanced on
    body count, chipmunk2d_gb300.shard) as one batch on its own GPU: no
    collective on the data path, a barrier around the timed steps and the
    maximum of the ranks' times."""
    import ctypes
    import torch
    from chipmunk2d_gb300 import load_gpu_library, Scene
    from chipmunk2d_gb300.shard import rank_range
    world_size = int(os.environ.get("WORLD_SIZE", "1")) if sharded else 1
    rank = int(os.environ.get("RANK", "0")) if sharded else 0
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if not dist.is_initialized():
            dist.init_process_group("nccl")
    lib = load_gpu_library()
    stream = torch.cuda.Stream()
    lib.cpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    sizes = batch_sizes(lib, BATCH_WORLDS)
    lo, hi = rank_range(sizes, rank, world_size)
    t0 = time.perf_counter()
    scenes = [Scene(lib, 4, sizes[i], seed=1000 + i) for i in range(lo, hi)]
    nb = sum(sc.nbodies for sc in scenes)
    batch = lib.cpGpuBatchNew()
    for sc in scenes:
        lib.cpGpuBatchAddSpace(batch, sc.space)
    assert lib.cpGpuBatchStep(batch, BATCH_DT, args.warmup, 0) == 0
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lib.cpGpuGetLaunchCount(1)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world_size > 1 else 0)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            ev[i][0].record(stream)
        lib.cpGpuBatchStep(batch, BATCH_DT, 1, 1)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = lib.cpGpuGetLaunchCount(1)
    clk = clocks.stop()
    if lib.cpGpuGetLastError():
        raise RuntimeError(lib.cpGpuGetLastErrorString().decode())
    tune = (ctypes.c_int * 2)()
    lib.cpGpuBatchGetTuning(batch, ctypes.cast(tune, ctypes.c_void_p))
    total_s = sum(a.elapsed_time(b) for a, b in ev) / 1000.0
    if dist:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
        dist.barrier()
    if getattr(args, "profile", False):
        # profiling runs (ncu) stop after the device-timed steps
        lib.cpGpuBatchFree(batch)
        for sc in scenes:
            sc.free()
        return None
    world_steps = BATCH_WORLDS * args.steps / total_s
    nb_total = nb
    if dist:
        t = torch.tensor([float(nb)], device="cuda")
        dist.all_reduce(t)
        nb_total = int(t.item())
    if rank != 0:
        lib.cpGpuBatchFree(batch)
        for sc in scenes:
            sc.free()
        return None
    lib.cpGpuSetTiming(1)
    phase = np.zeros(8)
    buf = np.zeros(8)
    for _ in range(5):
        lib.cpGpuBatchStep(batch, BATCH_DT, 1, 0)
        lib.cpGpuGetPhaseTimes(scenes[0].space, buf.ctypes.data, 8)
        phase += buf
    lib.cpGpuSetTiming(0)
    phase /= 5
    lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()

    # the same worlds stepped one cpSpaceStep at a time (plain GPU step), on a sample
    loop_n = 64
    loop = [Scene(lib, 4, sizes[i], seed=1000 + i) for i in range(loop_n)]
    for sc in loop:
        sc.step(BATCH_DT, args.warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loop_steps = 5
    for _ in range(loop_steps):
        for sc in loop:
            lib.cpSpaceStep(sc.space, BATCH_DT)
    torch.cuda.synchronize()
    loop_ws = loop_n * loop_steps / (time.perf_counter() - t0)
    for sc in loop:
        sc.free()

    # CPU restatement on a sample of worlds (every 16th), the same run
    # length: one thread, and all host threads (one world per thread)
    from chipmunk2d_gb300 import Scene as S2
    orc = oracle_lib()
    sample = list(range(0, BATCH_WORLDS, 16))
    cw = [S2(orc, 4, sizes[i], seed=1000 + i) for i in sample]
    threads = cpu_threads()
    cpu_step_worlds(cw, BATCH_DT, args.warmup, threads)
    cpu_all_s = cpu_step_worlds(cw, BATCH_DT, args.steps, threads)
    cpu_ws_all = len(cw) * args.steps / cpu_all_s
    for sc in cw:
        sc.free()
    c1 = [S2(orc, 4, sizes[i], seed=1000 + i) for i in sample[::8]]
    cpu_step_worlds(c1, BATCH_DT, args.warmup, 1)
    cpu_ws = len(c1) * args.steps / cpu_step_worlds(c1, BATCH_DT, args.steps, 1)
    for sc in c1:
        sc.free()

    names = PHASES
    line = {
        "metric": "world-steps/s", "value": world_steps, "unit": "world-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "batch", "worlds": BATCH_WORLDS, "bodies": nb_total,
                   "description": "4096 tumble worlds, bodies log-uniform in [8,512], 10 it, dt 1/60, seed 3",
                   "solver": "ordered (reference sweep order per world)", "build_s": build_s,
                   "parallelism": ("worlds sharded over %d GPUs (contiguous ranges balanced on body count)" % world_size
                                   if world_size > 1 else "single"),
                   "l2": "flushed between timed steps (256 MB fill, untimed)"},
        "body_steps_per_s": nb_total * args.steps / total_s,
        "launch": {"cuda_graph": True, "tuned_solve_threads": tune[0], "tuned_tree_staging": tune[1]},
        "looped_plain_gpu_world_steps_per_s": loop_ws,
        "batched_over_looped": world_steps / loop_ws,
        "phase_ms_after_run": dict(zip(names, [round(float(x), 4) for x in phase[:7]])),
        "gpu_launches": int(launches),
        "clocks": clk,
        "cpu_baseline": {"value": cpu_ws, "unit": "world-steps/s", "cores": 1, "kind": "port",
                         "sample": "%d worlds (every 128th) x %d steps" % (len(sample[::8]), args.steps)},
        "cpu_all_threads": {"value": cpu_ws_all, "unit": "world-steps/s", "cores": threads, "kind": "port",
                            "sample": "%d worlds (every 16th) x %d steps, one world per thread" % (len(sample), args.steps)},
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


ROLLOUT_WORLDS, ROLLOUT_SIZE, ROLLOUT_STEPS, ROLLOUT_K, ROLLOUT_DT = 1024, 64, 240, 16, 1 / 120
ROLLOUT_DESC = ("1024 worlds x (32 circles r~U[1,3] + 32 boxes sides U[2,6]) over a ground segment, "
                "240 steps, dt 1/120, 10 it, checkpoint every 16, world i seeded 4000+i; "
                "loss sum |p_final - target|^2, targets ~ N(0,10)")


def _rollout_scenes(lib, indices):
    from chipmunk2d_gb300 import Scene
    return [Scene(lib, 5, ROLLOUT_SIZE, seed=4000 + i) for i in indices]


def _positions(scenes):
    return np.concatenate([sc.bodies()[:, 0:2] for sc in scenes])


def _rollout_fd(lib, targets, n_params=64, seed=11):
    """Central differences of the GPU forward for sampled parameters.  The
    worlds are independent, so the loss terms of world i are the only ones
    a parameter of world i moves: each difference steps that world alone
    (cpGpuBatchStep on a one-world batch, bit-identical to its steps in the
    full batch).  Two step sizes screen out parameters where the loss is not
    smooth (a contact starting inside the step).  Each difference is formed
    from the final positions, L(+h) - L(-h) = sum (p+ - p-)(p+ + p- - 2t),
    so the rounding of the ~1e5 loss itself does not enter, at three step
    sizes whose spread bounds the differences' own error."""
    from chipmunk2d_gb300 import cpVect
    rng = np.random.default_rng(seed)
    kinds = ["v"] * 24 + ["w"] * 10 + ["m"] * 10 + ["e"] * 10 + ["u"] * 10
    params = []
    for k in kinds[:n_params]:
        w = int(rng.integers(ROLLOUT_WORLDS))
        idx = int(rng.integers(ROLLOUT_SIZE + (1 if k in "eu" else 0)))
        params.append((k, w, idx, int(rng.integers(2))))

    def world_final(p, h):
        k, w, idx, comp = p
        (sc,) = _rollout_scenes(lib, [w])
        if k in "vwm":
            body = lib.cpx_scene_body(sc.h, idx)
            if k == "v":
                v = lib.cpBodyGetVelocity(body)
                lib.cpBodySetVelocity(body, cpVect(v.x + (h if comp == 0 else 0.0), v.y + (h if comp == 1 else 0.0)))
            elif k == "w":
                lib.cpBodySetAngularVelocity(body, lib.cpBodyGetAngularVelocity(body) + h)
            else:
                lib.cpBodySetMass(body, lib.cpBodyGetMass(body) + h)
        else:
            shape = lib.cpx_scene_shape(sc.h, idx)
            if k == "e":
                lib.cpShapeSetElasticity(shape, lib.cpShapeGetElasticity(shape) + h)
            else:
                lib.cpShapeSetFriction(shape, lib.cpShapeGetFriction(shape) + h)
        b = lib.cpGpuBatchNew()
        lib.cpGpuBatchAddSpace(b, sc.space)
        assert lib.cpGpuBatchStep(b, ROLLOUT_DT, ROLLOUT_STEPS, 0) == 0
        p_ = sc.bodies()[:, 0:2]
        lib.cpGpuBatchFree(b)
        sc.free()
        return p_

    out = []
    for p in params:
        t = targets[p[1] * ROLLOUT_SIZE:(p[1] + 1) * ROLLOUT_SIZE]
        fd = []
        for h in ROLLOUT_FD_STEPS:
            pp, pm = world_final(p, h), world_final(p, -h)
            fd.append(float(np.sum((pp - pm) * (pp + pm - 2.0 * t))) / (2 * h))
        out.append((p, fd))
    return out


ROLLOUT_FD_STEPS = (1e-5, 1e-6, 1e-7)


def run_rollout(args, emit=True, sharded=True):
    """Differentiable rollout: 1024 worlds of 32 circles and 32 boxes over a
    ground segment, 240 steps at dt 1/120, 10 iterations, a checkpoint every
    16 steps; loss sum |p_final - target|^2, targets ~ N(0, 10).  Timed: the
    plain batched forward (cpGpuBatchStep, 240 steps) and the forward with
    checkpoints plus the reverse pass (cpGpuRolloutForward +
    cpGpuRolloutBackward, host gradient buffers), each from the same fresh
    worlds.  Under torchrun each rank takes its contiguous range of worlds;
    the gradients are per world, so nothing is exchanged."""
    import ctypes
    import torch
    from chipmunk2d_gb300 import load_gpu_library
    from chipmunk2d_gb300.shard import rank_range
    world_size = int(os.environ.get("WORLD_SIZE", "1")) if sharded else 1
    rank = int(os.environ.get("RANK", "0")) if sharded else 0
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if not dist.is_initialized():
            dist.init_process_group("nccl")
    lib = load_gpu_library()
    stream = torch.cuda.Stream()
    lib.cpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    lo, hi = rank_range([ROLLOUT_SIZE] * ROLLOUT_WORLDS, rank, world_size)
    targets = np.random.default_rng(4).normal(0.0, 10.0, size=(ROLLOUT_WORLDS * ROLLOUT_SIZE, 2))
    my_t = targets[lo * ROLLOUT_SIZE:hi * ROLLOUT_SIZE]

    def fresh():
        scenes = _rollout_scenes(lib, range(lo, hi))
        b = lib.cpGpuBatchNew()
        for sc in scenes:
            lib.cpGpuBatchAddSpace(b, sc.space)
        assert lib.cpGpuBatchStep(b, ROLLOUT_DT, 0, 0) == 0      # uploads the worlds
        torch.cuda.synchronize()
        return scenes, b

    def done(scenes, b):
        lib.cpGpuBatchFree(b)
        for sc in scenes:
            sc.free()

    def sync_all():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def plain():
        scenes, b = fresh()
        sync_all()
        t0 = time.perf_counter()
        assert lib.cpGpuBatchStep(b, ROLLOUT_DT, ROLLOUT_STEPS, 0) == 0
        torch.cuda.synchronize()
        dt_ = time.perf_counter() - t0
        done(scenes, b)
        return dt_

    def rollout(timing=False):
        scenes, b = fresh()
        nd = sum(sc.nbodies for sc in scenes)
        ns = sum(sc.nshapes for sc in scenes)
        g = {"v0": np.zeros(2 * nd), "w0": np.zeros(nd), "m": np.zeros(nd), "e": np.zeros(ns), "u": np.zeros(ns)}
        lib.cpGpuSetTiming(1 if timing else 0)
        sync_all()
        t0 = time.perf_counter()
        assert lib.cpGpuRolloutForward(b, ROLLOUT_DT, ROLLOUT_STEPS, ROLLOUT_K) == 0, lib.cpGpuGetLastErrorString()
        p = _positions(scenes)      # the final positions, read back through the C API
        dLdp = np.ascontiguousarray(2.0 * (p - my_t)).ravel()
        t1 = time.perf_counter()
        rc = lib.cpGpuRolloutBackward(b, dLdp.ctypes.data, g["v0"].ctypes.data, g["w0"].ctypes.data,
                                      g["m"].ctypes.data, g["e"].ctypes.data, g["u"].ctypes.data)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        assert rc == 0, lib.cpGpuGetLastErrorString()
        tt = np.zeros(4)
        lib.cpGpuDebugRolloutTimes(b, tt.ctypes.data)
        lib.cpGpuSetTiming(0)
        L = float(np.sum((p - my_t) ** 2))
        done(scenes, b)
        return t1 - t0, t2 - t1, g, L, tt, nd, ns

    if getattr(args, "profile", False):
        # profiling runs (ncu): one plain forward and one rollout
        plain()
        rollout()
        if dist:
            dist.destroy_process_group()
        return None
    # warm-up: one of each (allocations, tape sizing), the reverse pass with
    # per-phase timing
    plain()
    _, _, _, _, phase_tt, _, _ = rollout(timing=True)
    lib.cpGpuGetLaunchCount(1)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world_size > 1 else 0)
    clocks.start()
    plain_s = min(plain() for _ in range(2))
    runs = [rollout() for _ in range(2)]
    launches = lib.cpGpuGetLaunchCount(1)
    clk = clocks.stop()
    fwd_s, bwd_s, g, L, _, nd, ns = min(runs, key=lambda r: r[0] + r[1])
    if dist:
        t = torch.tensor([plain_s, fwd_s, bwd_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        plain_s, fwd_s, bwd_s = (float(x) for x in t.tolist())
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None
    deterministic = all(np.array_equal(runs[0][2][k], runs[1][2][k]) for k in g)

    fd_rows = _rollout_fd(lib, targets) if world_size == 1 else []
    # u = the spread of the differences at the three step sizes bounds
    # their own error.  Resolved: u <= 1e-6 |fd|; kinked: the two smaller
    # sizes differ by more than 1e-2 |fd| (a contact event within the step).
    resolved, kinked, within, outside = [], 0, 0, []
    for (k, w, idx, comp), (f5, f6, f7) in fd_rows:
        b0 = (w - lo) * ROLLOUT_SIZE + idx
        s0 = (w - lo) * (ROLLOUT_SIZE + 1) + idx
        adj = {"v": lambda: g["v0"][2 * b0 + comp], "w": lambda: g["w0"][b0], "m": lambda: g["m"][b0],
               "e": lambda: g["e"][s0], "u": lambda: g["u"][s0]}[k]()
        if abs(f6 - f7) > 1e-2 * abs(f6):
            kinked += 1
            continue
        u = max(abs(f5 - f6), abs(f6 - f7), abs(f5 - f7))
        if abs(adj - f6) <= max(1e-6 * abs(f6), u):
            within += 1
        else:
            outside.append({"param": "%s world %d index %d comp %d" % (k, w, idx, comp), "adjoint": float(adj),
                            "fd": [f5, f6, f7], "rel_err": abs(adj - f6) / max(abs(f6), 1e-300)})
        if f6 != 0.0 and u <= 1e-6 * abs(f6):
            resolved.append(abs(adj - f6) / abs(f6))

    # CPU restatement (the oracle): the plain forward, one thread on a
    # sample of worlds and all host threads on every world
    orc = oracle_lib()
    cpu_n = 16
    cw = _rollout_scenes(orc, range(cpu_n))
    cpu_s = cpu_step_worlds(cw, ROLLOUT_DT, ROLLOUT_STEPS, 1)
    for sc in cw:
        sc.free()
    threads = cpu_threads()
    cw = _rollout_scenes(orc, range(ROLLOUT_WORLDS))
    cpu_all_s = cpu_step_worlds(cw, ROLLOUT_DT, ROLLOUT_STEPS, threads)
    for sc in cw:
        sc.free()

    total = fwd_s + bwd_s
    worlds = ROLLOUT_WORLDS
    line = {
        "metric": "rollout steps/s (forward+adjoint)", "value": ROLLOUT_STEPS / total, "unit": "steps/s",
        "n_gpus": world_size, "steps": ROLLOUT_STEPS, "warmup": 1,
        "ms_per_step": 1000 * total / ROLLOUT_STEPS, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "rollout", "worlds": worlds, "bodies_per_world": ROLLOUT_SIZE,
                   "description": ROLLOUT_DESC,
                   "parallelism": ("worlds sharded over %d GPUs" % world_size if world_size > 1 else "single"),
                   "l2": "inputs larger than L2 (tape and checkpoints)"},
        "plain_forward_ms": 1000 * plain_s,
        "rollout_forward_ms": 1000 * fwd_s,
        "backward_ms": 1000 * bwd_s,
        "fwd_adj_over_forward": total / plain_s,
        "backward_phases_ms": {"replay_with_recording": float(phase_tt[0]), "reverse_steps": float(phase_tt[1])},
        "device_memory_gb": {"segment_tape": float(phase_tt[2]) / 1e9, "checkpoints": float(phase_tt[3]) / 1e9},
        "gradients_deterministic": bool(deterministic),
        "fd_check": {"params": len(fd_rows), "kinked": kinked,
                     "within_fd_uncertainty": within,
                     "outside": outside,
                     "resolved": len(resolved),
                     "resolved_max_rel_err": max(resolved) if resolved else None,
                     "resolved_median_rel_err": float(np.median(resolved)) if resolved else None,
                     "against": ("central differences of the GPU forward at h = 1e-5, 1e-6, 1e-7, formed from the "
                                 "final positions (sum (p+ - p-)(p+ + p- - 2t)), one world per difference; u = their "
                                 "spread; resolved: u <= 1e-6 |fd|; kinked: fd(1e-6), fd(1e-7) differ by > 1e-2; "
                                 "within: |adjoint - fd(1e-6)| <= max(1e-6 |fd|, u)")},
        "e2e": {"value": ROLLOUT_STEPS / total, "unit": "steps/s",
                "h2d_bytes_per_step": 72 * nd / ROLLOUT_STEPS,
                "d2h_bytes_per_step": (16 * nd + 8 * nd * 2 + 8 * ns * 2 + 18 * 8 * nd) / ROLLOUT_STEPS,
                "path": "cpGpuRolloutForward, final bodies read back, cpGpuRolloutBackward with host seed and gradient buffers"},
        "loss": L,
        "gpu_launches": int(launches),
        "clocks": clk,
        "cpu_baseline": {"value": cpu_n * ROLLOUT_STEPS * ROLLOUT_SIZE / cpu_s, "unit": "body-steps/s (forward only)",
                         "cores": 1, "kind": "port",
                         "sample": "%d worlds x %d steps of the forward (the reference has no adjoint)" % (cpu_n, ROLLOUT_STEPS)},
        "cpu_all_threads": {"value": ROLLOUT_WORLDS * ROLLOUT_STEPS * ROLLOUT_SIZE / cpu_all_s,
                            "unit": "body-steps/s (forward only)", "cores": threads, "kind": "port",
                            "sample": "all %d worlds x %d steps of the forward, one world per thread" % (ROLLOUT_WORLDS, ROLLOUT_STEPS)},
        "gpu_forward_body_steps_per_s": worlds * ROLLOUT_SIZE * ROLLOUT_STEPS / plain_s,
    }
    if dist:
        dist.destroy_process_group()
    if emit:
        print(json.dumps(line), flush=True)
    return line


PHASES = ["integrate+cache", "broadphase", "narrowphase", "arbiters", "schedule", "prestep+velocity", "solve"]


def mode_sample(lib, workload, steps, warmup, mode=0, phases=False, e2e=False):
    """Wall-timed steps of one workload in one solver mode (0: the exact
    reference-order mode, the drop-in's default; 1: coloured), closed by a
    device sync, for the JSON line's extra records; `warmup` untimed steps
    lead in.  With e2e, as many further steps are timed through the public
    API as a program uses it: cpSpaceStep, then every body's position,
    velocity and angle (cpBodyGet*)."""
    import torch
    from chipmunk2d_gb300 import Scene
    cfg, size, dt, desc = WORKLOADS[workload]
    sc = Scene(lib, cfg, size)
    lib.cpGpuSetSolverMode(sc.space, mode)
    for _ in range(warmup):
        lib.cpSpaceStep(sc.space, dt)
    lib.cpGpuSpaceSync(sc.space)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        lib.cpSpaceStep(sc.space, dt)
    lib.cpGpuSpaceSync(sc.space)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    err = lib.cpGpuGetLastError()
    rec = {"workload": workload, "solver": "colored" if mode else "ordered", "bodies": sc.nbodies,
           "shapes": sc.nshapes, "constraints": sc.nconstraints, "steps": steps, "warmup": warmup,
           "timed_window": [warmup, warmup + steps],
           "body_steps_per_s": sc.nbodies * steps / secs, "ms_per_step": 1000 * secs / steps,
           "description": desc}
    if e2e:
        out = pinned_doubles(8 * sc.nbodies)
        t0 = time.perf_counter()
        for _ in range(steps):
            lib.cpSpaceStep(sc.space, dt)
            assert lib.cpGpuSpaceGetBodyStates(sc.space, out.ctypes.data, sc.nbodies) == sc.nbodies
        es = time.perf_counter() - t0
        rec["e2e"] = {"value": sc.nbodies * steps / es, "unit": "body-steps/s", "timed_window": [warmup + steps, warmup + 2 * steps],
                      "d2h_bytes_per_step": 64 * sc.nbodies,
                      "path": "cpSpaceStep + cpGpuSpaceGetBodyStates (every body's position, velocity, angle, angular velocity, rotation)"}
    if err:
        rec["error"] = lib.cpGpuGetLastErrorString().decode()
    if phases:
        lib.cpGpuSetTiming(1)
        buf, acc = np.zeros(8), np.zeros(7)
        for _ in range(5):
            lib.cpSpaceStep(sc.space, dt)
            lib.cpGpuGetPhaseTimes(sc.space, buf.ctypes.data, 8)
            acc += buf[:7]
        lib.cpGpuSetTiming(0)
        rec["phase_ms"] = dict(zip(PHASES, [round(float(x) / 5, 4) for x in acc]))
    sc.free()
    return rec


def sleep_sample(lib, olib, workload="pyramid", threshold=0.5, n=300):
    """The exact-order mode with sleeping on (cpSpaceSetSleepTimeThreshold):
    each step wall-timed with a device sync, on the GPU and on the oracle
    (one core); the awake window before the pile settles and the window
    after it fell asleep."""
    import torch
    from chipmunk2d_gb300 import Scene
    cfg, size, dt, desc = WORKLOADS[workload]
    rec = {"workload": workload, "threshold_s": threshold, "steps": n,
           "windows": {"awake": [10, 100], "asleep": [n - 100, n]}}
    for name, L in (("gpu", lib), ("oracle_1core", olib)):
        sc = Scene(L, cfg, size)
        L.cpSpaceSetSleepTimeThreshold(sc.space, threshold)
        times = []
        for _ in range(n):
            t0 = time.perf_counter()
            L.cpSpaceStep(sc.space, dt)
            if name == "gpu":
                L.cpGpuSpaceSync(sc.space)
                torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        asleep = sum(L.cpBodyIsSleeping(L.cpx_scene_body(sc.h, i)) for i in range(sc.nbodies))
        rec[name] = {"ms_per_step_awake": 1000 * float(np.mean(times[10:100])),
                     "ms_per_step_asleep": 1000 * float(np.mean(times[-100:])),
                     "bodies": sc.nbodies, "asleep_at_end": int(asleep)}
        if name == "gpu" and L.cpGpuGetLastError():
            rec[name]["error"] = L.cpGpuGetLastErrorString().decode()
        sc.free()
    return rec


def variant_sample(lib, workload="pyramid", n=200, lead=300):
    """The exact-order step with the host-side parts of the reference on:
    the spatial hash as the broadphase, collision handlers (the default
    handler functions, registered for the type every shape has, so their
    host calls are all the bridge adds; then for types no shape has, so
    the arbiters stay on the device), and sleeping; each step wall-timed
    with a device sync, after `lead` untimed steps."""
    import ctypes
    import torch
    from chipmunk2d_gb300 import Scene
    cfg, size, dt, desc = WORKLOADS[workload]
    lib.cpSpaceUseSpatialHash.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
    lib.cpSpaceAddCollisionHandler.restype = ctypes.c_void_p
    lib.cpSpaceAddCollisionHandler.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
    rec = {"workload": workload, "steps": n, "timed_window": [lead, lead + n]}
    for name in ("plain", "spatial_hash", "handlers", "handlers_other_types", "sleeping"):
        sc = Scene(lib, cfg, size)
        if name == "spatial_hash":
            lib.cpSpaceUseSpatialHash(sc.space, 40.0, 1000)
        elif name == "handlers":
            lib.cpSpaceAddCollisionHandler(sc.space, 0, 0)
        elif name == "handlers_other_types":
            # a handler for types no shape has: every arbiter stays on the device
            lib.cpSpaceAddCollisionHandler(sc.space, 1, 2)
        elif name == "sleeping":
            lib.cpSpaceSetSleepTimeThreshold(sc.space, 1e9)   # the sleeping path, nothing falls asleep
        for _ in range(lead):
            lib.cpSpaceStep(sc.space, dt)
        lib.cpGpuSpaceSync(sc.space)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            lib.cpSpaceStep(sc.space, dt)
            lib.cpGpuSpaceSync(sc.space)
        torch.cuda.synchronize()
        rec[name + "_ms_per_step"] = 1000 * (time.perf_counter() - t0) / n
        if lib.cpGpuGetLastError():
            rec[name + "_error"] = lib.cpGpuGetLastErrorString().decode()
        sc.free()
    return rec


def parity_mode_sample(lib, workload, steps, warmup, e2e=False):
    """The exact reference-order mode, for the `ordered_mode` record."""
    rec = mode_sample(lib, workload, steps, warmup, mode=0, phases=True, e2e=e2e)
    return {k: rec[k] for k in ("workload", "bodies", "steps", "timed_window", "body_steps_per_s", "ms_per_step",
                                "phase_ms", "e2e") if k in rec}


def solver_quality(lib, sc, dt, iters):
    """cpGpuSolverQuality from the space's current state, both solver modes:
    per iteration the RMS normal and friction residuals and the largest
    penetration."""
    out = {}
    for mode, name in ((0, "ordered"), (1, "colored")):
        q = np.zeros(3 * iters)
        if lib.cpGpuSolverQuality(sc.space, mode, dt, iters, q.ctypes.data) != 0:
            out[name] = {"error": lib.cpGpuGetLastErrorString().decode()}
            continue
        q = q.reshape(iters, 3)
        out[name] = {"normal_residual_rms": [float(x) for x in q[:, 0]],
                     "friction_residual_rms": [float(x) for x in q[:, 1]],
                     "max_penetration": [float(x) for x in q[:, 2]]}
    return out


def run_ours(args):
    import ctypes
    import torch
    from chipmunk2d_gb300 import load_gpu_library, Scene

    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    lib = load_gpu_library()
    stream = torch.cuda.Stream()
    lib.cpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
    cfg, size, dt, desc = WORKLOADS[args.workload]
    mode = 1 if args.mode == "colored" else 0

    def make():
        sc = Scene(lib, cfg, size, seed=cfg + 1000 * rank if world_size > 1 else None)
        lib.cpGpuSetSolverMode(sc.space, mode)
        return sc

    # ---- device-timed run (state resident in HBM) ----
    start = window_start(args.workload, args.warmup, args.steps)
    sc = make()
    n = sc.nbodies
    for _ in range(start):
        lib.cpSpaceStep(sc.space, dt)
    torch.cuda.synchronize()
    arbs0 = sc.arbiters()
    contacts0 = int(arbs0[:, 2].sum()) if len(arbs0) else 0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lib.cpGpuGetLaunchCount(1)
    clocks = ClockSampler(local_rank)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))          # L2 flush between timed steps (not timed)
            ev[i][0].record(stream)
        lib.cpSpaceStep(sc.space, dt)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = lib.cpGpuGetLaunchCount(1)
    if args.profile:
        # profiling runs (ncu) stop after the device-timed steps
        clocks.stop()
        sc.free()
        return
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1000.0
    if dist:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
        dist.barrier()
    clk = clocks.stop()
    err = lib.cpGpuGetLastError()
    if err:
        raise RuntimeError("GPU step failed: %s" % lib.cpGpuGetLastErrorString().decode())
    arbs = sc.arbiters()
    contacts = int(arbs[:, 2].sum()) if len(arbs) else 0
    # solver quality at the end of the window, both modes from this state
    quality = solver_quality(lib, sc, dt, 15 if cfg == 3 else 10) if rank == 0 and args.extras else None

    # ---- per-phase timing pass (phase events, separate run) ----
    lib.cpGpuSetTiming(1)
    phase = np.zeros(7)
    nph = min(10, args.steps)
    buf = np.zeros(8)
    for _ in range(nph):
        lib.cpSpaceStep(sc.space, dt)
        lib.cpGpuGetPhaseTimes(sc.space, buf.ctypes.data, 8)
        phase += buf[:7]
    lib.cpGpuSetTiming(0)
    phase /= nph
    st = np.zeros(8, dtype=np.int32)
    lib.cpGpuGetStepStats(sc.space, st.ctypes.data, 8)
    sweep_levels = int(st[6])
    sc.free()

    # ---- end-to-end run through the public C API, same window ----
    sc = make()
    for _ in range(start):
        lib.cpSpaceStep(sc.space, dt)
    out = pinned_doubles(8 * n)
    sc.public()
    torch.cuda.synchronize()
    e2e_steps = min(args.steps, 200)
    e2e_s = 0.0
    arb_per_step = []
    stats = np.zeros(8, dtype=np.int32)
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        lib.cpSpaceStep(sc.space, dt)
        got = lib.cpGpuSpaceGetBodyStates(sc.space, out.ctypes.data, n)
        e2e_s += time.perf_counter() - t0
        assert got == n, got
        lib.cpGpuGetStepStats(sc.space, stats.ctypes.data, 8)      # untimed: arbiters solved this step
        arb_per_step.append(int(stats[5]))
    # the same window read through one getter call per value instead
    getter_s = 0.0
    for _ in range(min(e2e_steps, 20)):
        t0 = time.perf_counter()
        lib.cpSpaceStep(sc.space, dt)
        lib.cpx_scene_dump_public(sc.h, out.ctypes.data)
        getter_s += time.perf_counter() - t0
    getter_value = n * min(e2e_steps, 20) * world_size / getter_s
    sc.free()

    value = n * args.steps * world_size / total_s
    e2e_value = n * e2e_steps * world_size / e2e_s

    # ---- roofline of the dominant phase ----
    names = PHASES
    dom = int(np.argmax(phase))
    iters = 10 if cfg != 3 else 15
    algo_all = {
        0: n * (BYTES_PER_BODY_POS + BYTES_PER_CIRCLE_CACHE),
        1: 32 * sc.nshapes + 8 * contacts,
        2: contacts * (24 * 2 + 4 + 16 + 40 + 8),
        3: contacts * 104,
        4: 16 * len(arbs),
        5: contacts * BYTES_PER_CONTACT_PRESTEP + n * BYTES_PER_BODY_VEL,
        6: contacts * BYTES_PER_CONTACT_ITER * (iters + 1),
    }
    algo = algo_all[dom]
    # achieved HBM GB/s of every phase (algorithmic bytes / event-timed duration)
    phase_gbs = {names[i]: round(algo_all[i] / (phase[i] / 1000.0) / 1e9, 2) if phase[i] > 0 else None
                 for i in range(len(names))}
    peak, peak_kind = measured_peaks()
    achieved = algo / (phase[dom] / 1000.0) / 1e9 if phase[dom] > 0 else 0.0
    # DRAM bytes of one launch of the dominant kernel, from an ncu capture
    # of the same timed window (profiles/traffic.json records each window)
    traffic, traffic_note = None, "no capture of this window"
    tpath = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            recs = json.load(f).get(args.workload, [])
        for rec in (recs if isinstance(recs, list) else [recs]):
            if rec.get("window") == [start, start + args.steps] and names[dom] in rec:
                traffic = rec[names[dom]]
                traffic_note = rec.get("how", "")

    if rank == 0:
        (cpu_v, cpu_steps, cpu_s), (hv, h_steps, h_s), _ = cpu_sample(
            args.workload, budget_s=args.cpu_seconds, warm=start, hasty_s=min(args.cpu_seconds, 8.0))
    else:
        cpu_v, cpu_steps, cpu_s, hv, h_steps, h_s = None, 0, 0, None, 0, 0

    extras = {}
    if args.extras and rank == 0 and args.workload == "circles":
        # the exact-order mode (bit-compatible with cpSpaceStep) on the
        # pyramid and on this workload, and the batched-world throughput
        lib.cpGpuSetStream(ctypes.c_void_p(stream.cuda_stream))
        extras["ordered_mode"] = [parity_mode_sample(lib, "pyramid", 300, window_start("pyramid", 5, 300)),
                                  parity_mode_sample(lib, "circles", 10, window_start("circles", 5, 10), e2e=True)]
        extras["sleeping"] = sleep_sample(lib, oracle_lib())
        extras["host_parts"] = variant_sample(lib)
        # mixed shapes and pivot chains at full size (40,000 bodies)
        extras["mixed"] = [mode_sample(lib, "mixed", 150, 150, mode=1, phases=True),
                           mode_sample(lib, "mixed", 3, 2, mode=0)]
        b = run_batch(argparse.Namespace(steps=BATCH_STEPS, warmup=3), emit=False, sharded=False)
        extras["batch"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "body_steps_per_s",
                                             "looped_plain_gpu_world_steps_per_s", "batched_over_looped", "launch",
                                             "cpu_baseline", "cpu_all_threads", "phase_ms_after_run")}
        extras["batch"]["config"] = b["config"]
        r = run_rollout(args, emit=False, sharded=False)
        extras["rollout"] = {k: r[k] for k in ("value", "unit", "plain_forward_ms", "rollout_forward_ms", "backward_ms",
                                               "fwd_adj_over_forward", "backward_phases_ms", "device_memory_gb",
                                               "gradients_deterministic",
                                               "fd_check", "cpu_baseline", "cpu_all_threads")}
        extras["rollout"]["config"] = r["config"]

    line = {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": args.workload, "description": desc, "bodies": n, "solver": args.mode,
                   "timed_window": [start, start + args.steps], "lead_in_untimed": start,
                   "run_length": RUN_STEPS.get(args.workload),
                   "contacts_window_start": contacts0, "contacts_window_end": contacts,
                   "arbiters_per_timed_step": arb_per_step,
                   "l2": "flushed between timed steps (256 MB fill, untimed)",
                   "parallelism": "replicas" if world_size > 1 else "single"},
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": 88,
                "d2h_bytes_per_step": 64 * n + 64, "steps": e2e_steps,
                "l2": "not flushed: consecutive steps as a program runs them (the device-timed value flushes L2 before every step)",
                "path": "cpSpaceStep + cpGpuSpaceGetBodyStates (every body's position, velocity, angle, angular velocity, rotation into pinned host memory)",
                "per_body_getters": {"value": getter_value, "steps": min(e2e_steps, 20),
                                     "path": "cpSpaceStep + cpBodyGetPosition/Velocity/Angle/AngularVelocity/Rotation for every body (one C call each)"}},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "traffic_capture": traffic_note, "algorithmic_bytes_per_launch": algo,
                     "limiter": ("latency: one grid barrier, one round of L2 body loads and the dependent FP64 "
                                 "chain per colour level; rows and bodies stay L2-resident" if names[dom] == "solve"
                                 else "latency-bound gather")},
        "phase_ms": dict(zip(names, [round(float(x), 4) for x in phase])),
        "phase_achieved_gbs": phase_gbs,
        "sweep_levels_final": sweep_levels,
        "gpu_launches": int(launches),
        "clocks": clk,
        "cpu_baseline": {"value": cpu_v, "unit": "body-steps/s", "cores": 1, "kind": "port",
                         "sample": "%d steps (%.1f s) of the %s workload from step %d (the timed window's start)" % (cpu_steps, cpu_s, args.workload, start)},
        "cpu_hasty": {"value": hv, "unit": "body-steps/s", "cores": 2, "kind": "port",
                      "sample": ("cpHastySpace's two-thread solver restated in the oracle, %d steps (%.1f s) following those"
                                 % (h_steps, h_s))},
        "host_cpu": host_cpu(),
        "solver_quality": ({"state": "after step %d, both solvers from the same state" % (start + args.steps), **quality}
                           if quality else None),
    }
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 600; the batch workload's own 300; the rollout's 240)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="colored", choices=["ordered", "colored"])
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the ordered-mode and batched-world records of the default line")
    ap.add_argument("--workload", default="circles", choices=sorted(WORKLOADS) + ["batch", "rollout"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--profile", action="store_true",
                    help="run only the warm-up and device-timed steps (for ncu captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        args.steps = BATCH_STEPS if args.workload == "batch" else 600
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "rollout":
        run_rollout(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
