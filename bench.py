"""Benchmark of the batched arena tick: 2v2 arena-ticks/s on one GB300.

Workload (the batched, uniform 2v2 configuration): 4096 independent arenas on
the seeded procedural soccar mesh, each with 4 Octane cars (2v2) and a ball.
Per-arena seeded starting states: car positions uniform in the field,
velocities of uniform direction with |v| <= 2300 uu/s, a quarter of the cars
airborne with uniformly random orientation; ball |v| <= 6000 uu/s.  Controls
follow the 2v2 input process (analog inputs uniform in [-1, 1], jump / boost /
handbrake Bernoulli(0.3), each car re-drawing after a hold of 2..60 ticks).

A step is 8 ticks of every arena.  ``value`` runs each step as one
rsg_step_async launch whose per-tick controls are already in device memory;
``e2e`` runs it through the synchronous host API: the step's per-tick controls
from pinned host memory (rsg_step_controls, 8 ticks), and every car, ball and
pad state read back to host memory (rsg_get_all_states).  The L2 cache is flushed
(a 256 MiB device write) between timed steps.

The same line carries ``adjoint``: gradient steps (forward with checkpoints,
loss, hand-written adjoint backward) of 60-tick air-control rollouts over
8192 instances, replayed as one captured CUDA graph (and eagerly), their
relative error against FP64 central finite differences on a few instances,
and the backward / forward cost ratio of the C-ABI calls; and ``ground_adjoint``:
the same for 120-tick ground-driving rollouts over 65536 instances (eager
steps), checked on 256 of them.

``--impl reference`` times the CPU implementation of the same tick on the
host cores instead: the reference library built from its sources when it is
loadable on this machine, else the CPU restatement of it (oracle/).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

TICKS_PER_STEP = 8
CARS = 4
WORKLOAD = "batched uniform 2v2: 4096 arenas x (4 Octane + ball), procedural soccar mesh seed 0, 8 ticks/step"


# ---------------------------------------------------------------- workload
def initial_states(n_arenas: int, seed: int, car_dt, ball_dt, cars_per_arena: int = CARS):
    rng = np.random.default_rng(seed)
    A = n_arenas
    cars = np.zeros(A * cars_per_arena, car_dt)
    n = A * cars_per_arena
    air = rng.random(n) < 0.25
    x, y = rng.uniform(-3500, 3500, n), rng.uniform(-4500, 4500, n)
    z = np.where(air, rng.uniform(200, 1800, n), 17.0)
    # orientation: yaw only on the ground, a uniformly random quaternion in the air
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    yaw = rng.uniform(0, 2 * np.pi, n)
    q[~air] = np.stack([np.cos(yaw / 2), np.zeros(n), np.zeros(n), np.sin(yaw / 2)], 1)[~air]
    w, qx, qy, qz = q.T
    R = np.stack([
        np.stack([1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - w * qz), 2 * (qx * qz + w * qy)], 1),
        np.stack([2 * (qx * qy + w * qz), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - w * qx)], 1),
        np.stack([2 * (qx * qz - w * qy), 2 * (qy * qz + w * qx), 1 - 2 * (qx * qx + qy * qy)], 1),
    ], 1)  # [n, row, col]
    d = rng.normal(size=(n, 3))
    d[~air, 2] = 0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    v = d * rng.uniform(0, 2300, (n, 1))
    for k, c in enumerate("xyz"):
        cars["pos"][c] = (x, y, z)[k]
        cars["vel"][c] = v[:, k]
        cars["ang_vel"][c] = np.where(air, rng.uniform(-3, 3, n), 0.0)
        for j, col in enumerate(("forward", "right", "up")):
            cars["rot_mat"][col][c] = R[:, k, j]
    cars["is_on_ground"] = (~air).astype(np.uint8)
    cars["boost"] = rng.uniform(0, 100, n)
    cars["ball_hit_info"]["tick_count_when_hit"] = np.uint64(2 ** 64 - 1)
    cars["ball_hit_info"]["tick_count_when_extra_impulse_applied"] = np.uint64(2 ** 64 - 1)
    balls = np.zeros(A, ball_dt)
    d = rng.normal(size=(A, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    bv = d * rng.uniform(0, 6000, (A, 1))
    for k, c in enumerate("xyz"):
        balls["pos"][c] = (rng.uniform(-3000, 3000, A), rng.uniform(-4000, 4000, A), rng.uniform(93.15, 1800, A))[k]
        balls["vel"][c] = bv[:, k]
        balls["ang_vel"][c] = rng.uniform(-2, 2, A)
    for j, col in enumerate(("forward", "right", "up")):
        for k, c in enumerate("xyz"):
            balls["rot_mat"][col][c] = 1.0 if j == k else 0.0
    return cars, balls


class ControlProcess:
    """Per-car hold-and-redraw input process, vectorised over all cars."""

    def __init__(self, n_cars: int, seed: int, ctl_dt):
        self.rng = np.random.default_rng(seed)
        self.n = n_cars
        self.dt = ctl_dt
        self.cur = np.zeros(n_cars, ctl_dt)
        self.hold = np.zeros(n_cars, np.int64)

    def tick(self) -> np.ndarray:
        redraw = self.hold <= 0
        m = int(redraw.sum())
        if m:
            for name in ("throttle", "steer", "pitch", "yaw", "roll"):
                self.cur[name][redraw] = self.rng.uniform(-1, 1, m)
            for name in ("jump", "boost", "handbrake"):
                self.cur[name][redraw] = (self.rng.random(m) < 0.3).astype(np.uint8)
            self.hold[redraw] = self.rng.integers(2, 61, m)
        self.hold -= 1
        return self.cur.copy()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

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
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU timing
def cpu_kind() -> str:
    """'ref' when the reference library built from its sources loads here, else 'oracle'."""
    from oracle.pyoracle import REF_SO, load
    if os.path.exists(REF_SO):
        try:
            load("ref")
            return "ref"
        except OSError:
            pass
    return "oracle"


def cpu_ticks_per_second(threads: int, seconds: float, seed: int = 7, kind: str | None = None):
    """Arena-ticks/s of the CPU implementation: `threads` threads, each stepping its
    own 2v2 arena with the same input process for about `seconds`.  Controls are
    generated before the timed region and fed 240 ticks per native call, which
    releases the GIL, so the threads run in parallel."""
    from oracle.pyoracle import SimArena, CarState as OCarState, BallState as OBallState, CarControls as OCtl
    from rocketsim_gb300.arena_mesh import arena_cmf
    kind = kind or cpu_kind()
    cmf = arena_cmf(0)
    cars, balls = initial_states(max(threads, 1), seed, np.dtype(OCarState), np.dtype(OBallState))
    ctl_dt = np.dtype(OCtl)
    chunk, nchunks = 240, 8
    counts = [0] * threads
    stop = threading.Event()
    arenas, buffers = [], []
    for t in range(threads):
        a = SimArena(kind, cmf)
        ids = [a.add_car(i % 2, 0) for i in range(CARS)]
        for i, cid in enumerate(ids):
            a.set_car(cid, OCarState.from_buffer_copy(cars[t * CARS + i].tobytes()))
        a.set_ball(OBallState.from_buffer_copy(balls[t].tobytes()))
        proc = ControlProcess(CARS, seed + 100 + t, ctl_dt)
        buffers.append(np.ascontiguousarray(np.stack([proc.tick() for _ in range(chunk * nchunks)])))
        arenas.append(a)
    a.run(buffers[0].ctypes.data, CARS, 1)  # load / first-tick work outside the timed region
    for a, buf in zip(arenas[1:], buffers[1:]):
        a.run(buf.ctypes.data, CARS, 1)

    def worker(t):
        a, buf = arenas[t], buffers[t]
        n, k = 0, 0
        while not stop.is_set():
            a.run(buf[k * chunk:(k + 1) * chunk].ctypes.data, CARS, chunk)
            n += chunk
            k = (k + 1) % nchunks
        counts[t] = n

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    time.sleep(seconds)
    stop.set()
    for th in ths:
        th.join()
    el = time.perf_counter() - t0
    for a in arenas:
        a.close()
    return sum(counts) / el, sum(counts), el, kind


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def reference_kind_note(kind: str) -> str:
    if kind == "ref":
        return "the reference RocketSim built from its own sources (oracle/_ref)"
    return ("CPU restatement of the reference tick (oracle/; its SSE build reproduces the reference bit for bit "
            "on x86, the reference library itself is not built on this host)")


# ---------------------------------------------------------------- GPU arm
HITBOXES = 6  # Octane, Dominus, Plank, Breakout, Hybrid, Merc


def uneven_layout(n_arenas: int, seed: int):
    """Car counts 2, 4 or 6 drawn 1:1:1 per arena and a hitbox preset drawn uniformly per car."""
    rng = np.random.default_rng(seed)
    counts = rng.choice([2, 4, 6], n_arenas)
    presets = [rng.integers(0, HITBOXES, int(c)) for c in counts]
    return counts, presets


def make_batch(rsg, abi, A: int, mc: int, counts=None, presets=None):
    batch = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, A, mc, 120.0)
    for a in range(A):
        n = mc if counts is None else int(counts[a])
        for i in range(n):
            batch.add_car(a, i % 2, abi.CAR_OCTANE if presets is None else int(presets[a][i]), 0)
    return batch


def place_states(batch, rsg, A: int, mc: int, seed: int):
    """Seeded starting states of the batched workloads (slots without a car are ignored on set)."""
    cars, balls = initial_states(A, seed, rsg.CAR_STATE_DTYPE, rsg.BALL_STATE_DTYPE, cars_per_arena=mc)
    batch.set_all_states(cars, balls, None)


def run_arena_leg(args, dev: int, A: int, mc: int, steps: int, warmup: int, settle: int, counts=None,
                  presets=None, reset_every: int = 0, reset_frac: float = 0.0, rank: int = 0, world: int = 1,
                  e2e: bool = True, flush_l2: bool = True, curve: bool = True, tps: int = TICKS_PER_STEP):
    """One batched workload: `settle` ticks to leave the start transient, `warmup` untimed steps,
    then `steps` timed steps of `tps` ticks, each one rsg_step_async launch with its
    controls already in device memory (L2 flushed before each).  Optionally the end-to-end leg
    through the synchronous host API with pinned host buffers."""
    import torch
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi

    batch = make_batch(rsg, abi, A, mc, counts, presets)
    place_states(batch, rsg, A, mc, 1234 + rank)
    n_ctl = A * mc
    proc = ControlProcess(n_ctl, 99 + rank, rsg.CONTROLS_DTYPE)
    rng = np.random.default_rng(555 + rank)
    d = f"cuda:{dev}"
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=d) if flush_l2 else None
    stream = torch.cuda.ExternalStream(batch.stream(), device=d)
    ticks_done = 0
    resets = 0

    def maybe_reset(t0: int, t1: int):
        # a goal or reset re-randomises reset_frac of the arenas once per reset_every ticks
        nonlocal resets
        if not reset_every or t1 // reset_every == t0 // reset_every:
            return
        k = max(1, int(round(A * reset_frac)))
        which = rng.choice(A, k, replace=False).astype(np.uint32)
        batch.reset_to_random_kickoff_many(which, rng.integers(0, 2 ** 31 - 1, k).astype(np.int32))
        resets += k

    def chunk(nticks: int) -> torch.Tensor:
        seq = np.stack([proc.tick() for _ in range(nticks)])
        t = torch.from_numpy(seq.view(np.uint8).reshape(-1).copy()).to(d)
        torch.cuda.current_stream().synchronize()  # the batch's stream reads it next
        return t

    # ---- settle: leave the start transient (cars land, drive on walls, collide); ticks/s against
    # game time on the way
    settle_curve = []
    win = 120
    while ticks_done < settle:
        n = min(win, settle - ticks_done)
        dc = chunk(n)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for k in range(0, n, tps):
                m = min(tps, n - k)
                batch.step_async(dc[k * n_ctl * 24:(k + m) * n_ctl * 24].data_ptr(), m)
            e1.record(stream)
        batch.sync()
        maybe_reset(ticks_done, ticks_done + n)
        ticks_done += n
        if curve:
            settle_curve.append([ticks_done, A * n / (e0.elapsed_time(e1) / 1e3)])
    # ---- warm-up and timed steps
    nsteps = warmup + steps
    d_seq = chunk(nsteps * tps).view(nsteps, -1)
    for s in range(warmup):
        batch.step_async(d_seq[s].data_ptr(), tps)
        batch.sync()
        maybe_reset(ticks_done, ticks_done + tps)
        ticks_done += tps
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    clocks = ClockSampler(dev)
    clocks.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    first_tick = ticks_done
    with torch.cuda.stream(stream):
        for k in range(steps):
            if flush is not None:
                flush.fill_(k & 0xff)
            ev[k][0].record(stream)
            batch.step_async(d_seq[warmup + k].data_ptr(), tps)
            ev[k][1].record(stream)
            if reset_every and (ticks_done + tps) // reset_every != ticks_done // reset_every:
                batch.sync()  # the reset is a host call between launches; it stays outside the events
                maybe_reset(ticks_done, ticks_done + tps)
            ticks_done += tps
    batch.sync()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clk = clocks.stop()
    times_ms = [a.elapsed_time(b) for a, b in ev]
    value, total_ms = replica_rate(A * tps * steps, sum(times_ms), world, d)
    flags = batch.device_flags()
    shape = batch.tick_shape()
    out = {"value": value, "ms_per_step": total_ms / steps, "times_ms": times_ms, "clocks": clk,
           "tick_shape": {"arenas_per_block": shape[0], "lanes_per_car": shape[1], "header_cache": shape[2],
                          "leaf_grid": shape[3], "collide_sync": shape[4], "persistent": shape[5],
                          "tuner": batch.tuning_log()},
           "game_tick_first_timed": first_tick, "game_tick_last_timed": ticks_done,
           "ticks_per_s_vs_game_tick": [[t, round(v)] for t, v in settle_curve],
           "warn_flags_any": int(np.bitwise_or.reduce(flags)) if flags.size else 0, "arenas_reset": resets,
           "gpu_launches": 2 * steps}  # per step: the tick kernel and the arena placement kernel
    if e2e:
        # ---- e2e: host buffers (pinned) through the synchronous API: controls in, every car, ball and
        # pad state out, each step
        pin = lambda dt, n: torch.empty(n * dt.itemsize, dtype=torch.uint8).pin_memory().numpy().view(dt)  # noqa
        ctl_np = pin(rsg.CONTROLS_DTYPE, n_ctl * tps).reshape(tps, n_ctl)
        out_cars = pin(rsg.CAR_STATE_DTYPE, A * mc)
        out_balls = pin(rsg.BALL_STATE_DTYPE, A)
        out_pads = pin(rsg.PAD_STATE_DTYPE, A * batch.num_pads)
        e2e_steps = max(3, min(steps, 20))
        seq_h = np.stack([proc.tick() for _ in range((e2e_steps + 2) * tps)]).reshape(e2e_steps + 2, tps, n_ctl)
        for s in range(2):
            ctl_np[:] = seq_h[s]
            batch.step_controls(ctl_np, tps)
            batch.get_all_states(out_cars, out_balls, out_pads)
        e2e_time = 0.0
        for s in range(e2e_steps):
            ctl_np[:] = seq_h[s + 2]
            if flush is not None:
                flush.fill_(s & 0xff)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            batch.step_controls(ctl_np, tps)
            batch.get_all_states(out_cars, out_balls, out_pads)
            e2e_time += time.perf_counter() - t0
        out["e2e"] = {"value": A * tps * e2e_steps * world / e2e_time, "unit": "arena-ticks/s",
                      "h2d_bytes_per_step": int(ctl_np.nbytes),
                      "d2h_bytes_per_step": int(out_cars.nbytes + out_balls.nbytes + out_pads.nbytes),
                      "host_buffers": "pinned",
                      "controls": "a control per car and tick from the same input process as the device-resident steps "
                                  "(rsg_step_controls)"}
    batch.close()
    return out


def replica_rate(units_per_rank: float, rank_ms: float, world: int, device) -> tuple[float, float]:
    """Whole-job rate of `world` independent replicas: every rank's units over the slowest rank's time
    (the maximum over the ranks, one all_reduce on the initialised process group).  Returns the rate
    per second and that time in ms."""
    total_ms = rank_ms
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([rank_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return units_per_rank * world / (total_ms / 1e3), total_ms


def load_counters() -> dict:
    """Per-launch figures of the tick kernels from the committed ncu summary (profiles/)."""
    p = os.path.join(REPO, "profiles", "tick_counters.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def sm_count(dev: int) -> int:
    import torch
    return torch.cuda.get_device_properties(dev).multi_processor_count


def run_gpu(args, rank: int, world: int):
    """The headline workload (4096 uniform 2v2 arenas) with its roofline and issue-slot figures."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300.arena_mesh import arena_cmf

    dev = int(os.environ.get("LOCAL_RANK", 0))
    import torch
    torch.cuda.set_device(dev)
    rsg.init_from_mem([arena_cmf(0)])
    A = args.arenas
    r = run_arena_leg(args, dev, A, CARS, args.steps, args.warmup, args.settle_ticks, rank=rank, world=world)
    # roofline of the tick: algorithmic bytes per launch (minimal 2v2 state read + written once per
    # launch, controls read every tick)
    state_rt = 1548
    ctl_per_tick = CARS * 24
    alg_bytes = A * (state_rt + ctl_per_tick * TICKS_PER_STEP)
    avg_launch_s = (sum(r["times_ms"]) / len(r["times_ms"])) / 1e3
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / avg_launch_s / 1e9
    cnt = load_counters()
    traffic = None
    if cnt.get("dram_bytes_per_arena_launch") is not None:
        traffic = {"per_launch": cnt["dram_bytes_per_arena_launch"] * A + cnt.get("dram_bytes_fixed_per_launch", 0),
                   "per_arena_records": cnt["dram_bytes_per_arena_launch"],
                   "fixed_mesh_per_launch": cnt.get("dram_bytes_fixed_per_launch", 0),
                   "source": cnt.get("source", "")}
    issue = None
    wi = cnt.get("warp_instructions_per_arena_tick")
    clk_mhz = r["clocks"].get("sm_mhz") or 2070.0
    if wi:
        slots = sm_count(dev) * 4 * clk_mhz * 1e6
        issue = {"warp_instructions_per_arena_tick": wi, "issue_slots_per_s": slots,
                 "frac": wi * r["value"] / world / slots,
                 "note": "warp instructions per arena-tick (ncu) x arena-ticks/s / (SMs x 4 schedulers x SM clock)"}
    r["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic["per_launch"] if traffic else None, "traffic_split": traffic,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "issue_slots": issue}
    return r


def run_config0(args, dev: int):
    """One arena, 2v2 Octane: the reference's own benchmark shape, a bounded sample of its 1M ticks."""
    return run_arena_leg(args, dev, 1, CARS, args.c0_steps, 3, args.settle_ticks, e2e=False, flush_l2=False,
                         curve=False, tps=120)


def run_config2(args, dev: int):
    """16384 arenas with 2, 4 or 6 cars (1:1:1) of all six hitboxes, 34 pads, 1 % of the arenas reset
    to a random kickoff every 300 ticks."""
    import rocketsim_gb300 as rsg  # noqa: F401
    counts, presets = uneven_layout(args.c2_arenas, 77)
    r = run_arena_leg(args, dev, args.c2_arenas, 6, args.c2_steps, args.warmup, args.settle_ticks, counts=counts,
                      presets=presets, reset_every=300, reset_frac=0.01, e2e=False)
    r["cars"] = int(np.sum(counts))
    return r


# ---------------------------------------------------------------- adjoint (air phase)
ADJ_TICKS = 60
ADJ_WORKLOAD = ("air-phase adjoint: 8192 instances x (1 airborne Octane + ball), 60 ticks, controls "
                "pitch/yaw/roll in [-1, 1] and relaxed boost in [0, 1], checkpoints every 16 ticks")


def adjoint_case(n: int, seed: int):
    """Air-phase differentiation workload: car at 400..1600 uu, |v| <= 1500 uu/s of uniform
    direction, uniformly random orientation, at rest rotationally; the ball point 300..1500 uu away
    with |v| <= 500 uu/s; controls uniform (|u| >= 1e-3 so no input sits on the |u| kink of the
    damping); a seeded target orientation per instance.  Bullet units (1 BT = 50 uu)."""
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 24), np.float32)
    s[:, 0:2] = rng.uniform(-3000, 3000, (n, 2)) / 50.0
    s[:, 2] = rng.uniform(400, 1600, n) / 50.0
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    s[:, 3:6] = d * rng.uniform(0, 1500, (n, 1)) / 50.0

    def rot(k):
        q = rng.normal(size=(k, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        x, y, z, w = q.T
        return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)
    s[:, 9:18] = rot(n)
    off = rng.normal(size=(n, 3))
    off *= (rng.uniform(300, 1500, n) / np.linalg.norm(off, axis=1))[:, None]
    s[:, 18:21] = s[:, 0:3] + off / 50.0
    bd = rng.normal(size=(n, 3))
    bd /= np.linalg.norm(bd, axis=1, keepdims=True)
    s[:, 21:24] = bd * rng.uniform(0, 500, (n, 1)) / 50.0
    u = rng.uniform(1e-3, 1.0, (ADJ_TICKS, n, 4)) * rng.choice([-1.0, 1.0], (ADJ_TICKS, n, 4))
    u[..., 3] = rng.uniform(1e-3, 1.0 - 1e-3, (ADJ_TICKS, n))
    return s, u.astype(np.float32), rot(n).reshape(n, 3, 3).astype(np.float32)


def _captured_grad_steps(args, adjoint, ds, du_g, tgt):
    """Times args.steps replays of one captured gradient step; returns the per-replay ms and the graph."""
    import torch
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            du_g.grad = None
            adjoint.aim_loss(adjoint.air_rollout(ds, du_g, ckpt_every=16), tgt).sum().backward()
    torch.cuda.current_stream().wait_stream(side)
    du_g.grad = None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        fin_g = adjoint.air_rollout(ds, du_g, ckpt_every=16)
        adjoint.aim_loss(fin_g, tgt).sum().backward()
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    gev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        gev[k][0].record()
        graph.replay()
        gev[k][1].record()
    torch.cuda.synchronize()
    graph_ms = [a.elapsed_time(b) for a, b in gev]
    return graph_ms, graph  # the graph owns the pool that holds du_g.grad


def run_adjoint(args, dev: int):
    """Gradient steps of the air-phase workload: forward with checkpoints, loss, adjoint backward."""
    import torch
    from rocketsim_gb300 import adjoint

    n = args.adj_instances
    s, u, target = adjoint_case(n, 4321)
    ds = torch.from_numpy(s).to(f"cuda:{dev}")
    du = torch.from_numpy(u).to(f"cuda:{dev}").requires_grad_(True)
    tgt = torch.from_numpy(target).to(f"cuda:{dev}")

    def grad_step():
        du.grad = None
        fin = adjoint.air_rollout(ds, du, ckpt_every=16)
        adjoint.aim_loss(fin, tgt).sum().backward()

    for _ in range(args.warmup):
        grad_step()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for k in range(args.steps):
        du.grad = None
        ev[k][0].record()
        fin = adjoint.air_rollout(ds, du, ckpt_every=16)
        ev[k][1].record()
        adjoint.aim_loss(fin, tgt).sum().backward()
        ev[k][2].record()
    torch.cuda.synchronize()
    fwd = [a.elapsed_time(b) for a, b, _ in ev]
    bwd = [b.elapsed_time(c) for _, b, c in ev]
    total_ms = sum(a.elapsed_time(c) for a, _, c in ev)
    grads_per_s = n * args.steps / (total_ms / 1e3)
    # plain forward (no checkpoints) for the cost ratio
    with torch.no_grad():
        adjoint.air_rollout(ds, du.detach())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            adjoint.air_rollout(ds, du.detach())
        e1.record()
        torch.cuda.synchronize()
        plain_fwd_ms = e0.elapsed_time(e1) / args.steps
    eager_grads_per_s = grads_per_s
    del fin
    # the same gradient step captured once as a CUDA graph and replayed (a training loop's form:
    # the controls and the gradient are static tensors updated in place).  The captured leaf is a
    # fresh tensor: autograd keeps a leaf's gradient accumulator, and with it the stream of its
    # first use, for as long as any graph refers to it.
    du_g = du.detach().clone().requires_grad_(True)
    try:
        graph_ms, graph = _captured_grad_steps(args, adjoint, ds, du_g, tgt)
        grads_per_s = n * args.steps / (sum(graph_ms) / 1e3)
        step_kind = "forward + loss + backward captured as one CUDA graph"
    except RuntimeError as e:  # capture refused: report the eager steps
        graph_ms, graph = [total_ms / args.steps] * args.steps, None
        step_kind = "eager (CUDA graph capture failed: " + str(e).splitlines()[0] + ")"
        du_g.grad = None
        adjoint.aim_loss(adjoint.air_rollout(ds, du_g, ckpt_every=16), tgt).sum().backward()
    g_gpu = du_g.grad[:, :args.adj_check].detach().cpu().numpy().astype(np.float64)
    del graph
    # the two C-ABI calls alone
    import ctypes as C
    from rocketsim_gb300 import abi
    from rocketsim_gb300.arena import car_config
    lib = abi.load(build_if_missing=False)
    cfg = car_config(abi.CAR_OCTANE)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    ck = torch.empty(((ADJ_TICKS + 15) // 16, n, 24), device=ds.device)
    fin = torch.empty_like(ds)
    gfin = torch.randn_like(ds)
    gu = torch.empty_like(du)
    nb = C.c_size_t()
    abi.check(lib.rsg_air_backward_workspace_size(n, ADJ_TICKS, C.byref(nb)), "workspace size")
    work = torch.empty(nb.value, dtype=torch.uint8, device=ds.device)
    strm = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    kf, kb = [], []
    for k in range(args.warmup + args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        abi.check(lib.rsg_air_forward(C.byref(cfg), 120.0, n, ADJ_TICKS, P(ds), P(du), P(fin), P(ck), 16, strm),
                  "rsg_air_forward")
        e[1].record()
        abi.check(lib.rsg_air_backward(C.byref(cfg), 120.0, n, ADJ_TICKS, P(du), P(ck), 16, P(gfin), P(gu), None,
                                       P(work), nb.value, strm), "rsg_air_backward")
        e[2].record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            kf.append(e[0].elapsed_time(e[1]))
            kb.append(e[1].elapsed_time(e[2]))
    return {"value": grads_per_s, "ms_per_step": sum(graph_ms) / args.steps, "step_kind": step_kind,
            "eager_value": eager_grads_per_s, "eager_ms_per_step": total_ms / args.steps,
            "ms_forward_ckpt": statistics.median(fwd), "ms_forward_plain": plain_fwd_ms,
            "ms_backward": statistics.median(bwd),
            "backward_over_forward": statistics.median(bwd) / plain_fwd_ms,
            "kernel_ms_forward_ckpt": statistics.median(kf), "kernel_ms_backward": statistics.median(kb),
            "kernel_backward_over_forward": statistics.median(kb) / plain_fwd_ms,
            "workspace_bytes": nb.value,
            "case": (s, u, target), "g_gpu": g_gpu}


def adjoint_cpu_check(case, g_gpu: np.ndarray, k: int):
    """FP64 central finite differences (step 1e-4) on the host for the first k instances: the
    gradient reference (relative error of the GPU adjoint) and the CPU way to the same gradients."""
    from oracle import air_fp64 as F
    s, u, target = case
    s64 = s[:k].astype(np.float64)
    u64 = u[:, :k].astype(np.float64)
    t64 = target[:k].astype(np.float64)
    iinv = F.car_inv_inertia((120.507, 86.6994, 38.6591))
    t0 = time.perf_counter()
    gfd = F.fd_grad(s64, u64, iinv, 1.0 / 120.0, lambda f: F.aim_loss(f, t64), h=1e-4)
    el = time.perf_counter() - t0
    num = np.linalg.norm((g_gpu - gfd).transpose(1, 0, 2).reshape(k, -1), axis=1)
    den = np.linalg.norm(gfd.transpose(1, 0, 2).reshape(k, -1), axis=1)
    return float((num / den).max()), k / el, el


# ---------------------------------------------------------------- adjoint (ground driving)
GROUND_TICKS = 120
GROUND_SETTLE = 24
GROUND_WORKLOAD = ("ground-driving adjoint: 65536 instances x (1 Octane on the procedural mesh floor + ball), 120 "
                   "ticks, throttle/steer in [-1, 1] and relaxed boost in [0, 1], loss on the car's nose point and "
                   "velocity at tick 120, checkpoints every 16 ticks")


def _smooth_controls(rng, ticks: int, n: int, lo: float, hi: float, knots: int = 4) -> np.ndarray:
    """[ticks, n] piecewise-linear signals through `knots` uniform values in [lo, hi] per instance."""
    vals = rng.uniform(lo, hi, (knots, n))
    pos = np.arange(ticks) / max(ticks - 1, 1) * (knots - 1)
    k = np.minimum(pos.astype(int), knots - 2)
    f = (pos - k)[:, None]
    return vals[k] * (1 - f) + vals[k + 1] * f


def ground_adjoint_case(n: int, seed: int, dev: str):
    """Ground-driving workload: an Octane on the floor within 800 uu of the centre, random heading,
    forward speed 0..1200 uu/s, settled for 24 ticks at throttle 0.5 by the rollout itself; the ball
    in the air far away; smooth random controls inside the ranges; a nose-point target 50..150 uu
    from where the car would be after 1 s at its start velocity, at nose height, and a random
    horizontal target velocity of up to 1500 uu/s.  Bullet units."""
    import torch
    from rocketsim_gb300 import adjoint
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 39), np.float32)
    yaw = rng.uniform(0, 2 * np.pi, n)
    c, si = np.cos(yaw), np.sin(yaw)
    s[:, 0:2] = rng.uniform(-800, 800, (n, 2)) / 50.0
    s[:, 2] = 17.0 / 50.0
    speed = rng.uniform(0, 1200, n) / 50.0
    s[:, 3], s[:, 4] = speed * c, speed * si
    s[:, 9:18] = np.stack([c, -si, np.zeros(n), si, c, np.zeros(n), np.zeros(n), np.zeros(n), np.ones(n)], 1)
    s[:, 33:36] = np.array([2500.0, -3500.0, 1200.0]) / 50.0
    s[:, 36:39] = rng.uniform(-300, 300, (n, 3)) / 50.0
    settle = np.zeros((GROUND_SETTLE, n, 4), np.float32)
    settle[..., 0] = 0.5
    with torch.no_grad():
        s = adjoint.ground_rollout(torch.from_numpy(s).to(dev), torch.from_numpy(settle).to(dev)).cpu().numpy()
    u = np.zeros((GROUND_TICKS, n, 4), np.float32)
    u[..., 0] = _smooth_controls(rng, GROUND_TICKS, n, 0.3, 0.9)
    u[..., 1] = _smooth_controls(rng, GROUND_TICKS, n, -0.6, 0.6)
    u[..., 2] = _smooth_controls(rng, GROUND_TICKS, n, 0.2, 0.8)
    ang = rng.uniform(0, 2 * np.pi, n)
    tp = np.zeros((n, 3), np.float32)
    tp[:, 0:2] = s[:, 0:2] + s[:, 3:5] * (GROUND_TICKS / 120.0) + \
        np.stack([np.cos(ang), np.sin(ang)], 1) * rng.uniform(1, 3, (n, 1))
    tp[:, 2] = (17.0 + 20.755) / 50.0
    ang = rng.uniform(0, 2 * np.pi, n)
    tv = np.zeros((n, 3), np.float32)
    tv[:, 0:2] = np.stack([np.cos(ang), np.sin(ang)], 1) * rng.uniform(0, 1500, (n, 1)) / 50.0
    return s, u, tp, tv


def run_ground_adjoint(args, dev: int):
    """Gradient steps of the ground-driving workload, eager: forward with checkpoints, loss, backward."""
    import ctypes as C
    import torch
    from rocketsim_gb300 import abi, adjoint
    from rocketsim_gb300.arena import car_config
    n = args.ground_instances
    d = f"cuda:{dev}"
    s, u, tp, tv = ground_adjoint_case(n, 2468, d)
    ds = torch.from_numpy(s).to(d)
    du = torch.from_numpy(u).to(d).requires_grad_(True)
    t_p, t_v = torch.from_numpy(tp).to(d), torch.from_numpy(tv).to(d)

    for _ in range(args.warmup):
        du.grad = None
        fin, flags = adjoint.ground_rollout(ds, du, ckpt_every=16, return_flags=True)
        adjoint.contact_loss(fin, t_p, t_v).sum().backward()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for k in range(args.steps):
        du.grad = None
        ev[k][0].record()
        fin = adjoint.ground_rollout(ds, du, ckpt_every=16)
        ev[k][1].record()
        adjoint.contact_loss(fin, t_p, t_v).sum().backward()
        ev[k][2].record()
    torch.cuda.synchronize()
    fwd = [a.elapsed_time(b) for a, b, _ in ev]
    bwd = [b.elapsed_time(c) for _, b, c in ev]
    total_ms = sum(a.elapsed_time(c) for a, _, c in ev)
    g_gpu = du.grad[:, :args.ground_check].detach().cpu().numpy().astype(np.float64)
    with torch.no_grad():
        adjoint.ground_rollout(ds, du.detach())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            adjoint.ground_rollout(ds, du.detach())
        e1.record()
        torch.cuda.synchronize()
        plain_fwd_ms = e0.elapsed_time(e1) / args.steps
    # the C-ABI calls alone
    lib = abi.load(build_if_missing=False)
    cfg = car_config(abi.CAR_OCTANE)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    ck = torch.empty(((GROUND_TICKS + 15) // 16, n, 39), device=d)
    fin = torch.empty_like(ds)
    gfin = torch.randn_like(ds)
    gu = torch.empty_like(du)
    nb = C.c_size_t()
    abi.check(lib.rsg_ground_backward_workspace_size(n, GROUND_TICKS, C.byref(nb)), "workspace size")
    work = torch.empty(nb.value, dtype=torch.uint8, device=d)
    strm = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    kf, kb = [], []
    for k in range(args.warmup + args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        abi.check(lib.rsg_ground_forward(C.byref(cfg), 120.0, n, GROUND_TICKS, P(ds), P(du), P(fin), P(ck), 16, None,
                                         strm), "rsg_ground_forward")
        e[1].record()
        abi.check(lib.rsg_ground_backward(C.byref(cfg), 120.0, n, GROUND_TICKS, P(du), P(ck), 16, P(gfin), P(gu),
                                          None, P(work), nb.value, strm), "rsg_ground_backward")
        e[2].record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            kf.append(e[0].elapsed_time(e[1]))
            kb.append(e[1].elapsed_time(e[2]))
    return {"value": n * args.steps / (total_ms / 1e3), "ms_per_step": total_ms / args.steps,
            "ms_forward_ckpt": statistics.median(fwd), "ms_forward_plain": plain_fwd_ms,
            "ms_backward": statistics.median(bwd), "backward_over_forward": statistics.median(bwd) / plain_fwd_ms,
            "kernel_ms_forward_ckpt": statistics.median(kf), "kernel_ms_backward": statistics.median(kb),
            "workspace_bytes": nb.value, "flagged_instances": int((flags != 0).sum()),
            "case": (s, u, tp, tv), "g_gpu": g_gpu}


GROUND_FD_TICKS = (0, 30, 60, 90, 110, 119)


def ground_cpu_check(case, g_gpu: np.ndarray):
    """FP64 central finite differences (step 1e-4) of the ground restatement for the instances of
    g_gpu at six ticks x three controls: the relative error of the GPU adjoint per instance (the
    maximum over them) and the CPU's rate of such gradient entries."""
    from oracle import ground_fp64 as Gr
    s, u, tp, tv = case
    k = g_gpu.shape[1]
    s64, u64 = s[:k].astype(np.float64), u[:, :k].astype(np.float64)
    which = [(t, c) for t in GROUND_FD_TICKS for c in range(3)]
    loss = lambda f: Gr.contact_loss(f, tp[:k].astype(np.float64), tv[:k].astype(np.float64))  # noqa: E731
    t0 = time.perf_counter()
    gfd = Gr.fd_grad(s64, u64, Gr.car_geometry(), 1.0 / 120.0, loss, h=1e-4, which=which)
    el = time.perf_counter() - t0
    gfd2 = Gr.fd_grad(s64, u64, Gr.car_geometry(), 1.0 / 120.0, loss, h=5e-5, which=which)
    a = np.stack([g_gpu[t, :, c] for t, c in which], 1)
    b = np.stack([gfd[t, :, c] for t, c in which], 1)
    b2 = np.stack([gfd2[t, :, c] for t, c in which], 1)
    rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    # instances whose two central differences disagree have a jump of the tick inside the
    # stencil (the lateral-friction input switching on at 5 uu/s of side slip, a push-back
    # starting): the difference quotient is no derivative there
    smooth = np.linalg.norm(b - b2, axis=1) <= 1e-5 * np.linalg.norm(b, axis=1)
    return {"max": float(rel[smooth].max()), "median": float(np.median(rel[smooth])),
            "nonsmooth": int((~smooth).sum()), "max_all": float(rel.max()),
            "rate": k * len(which) / el, "seconds": el, "entries": len(which)}


def _pred_balls(n: int, seed: int, dt) -> np.ndarray:
    """Balls in flight anywhere over the field: position, speed up to 3000 uu/s, spin up to 3 rad/s."""
    rng = np.random.default_rng(seed)
    b = np.zeros(n, dt)
    for f, (lo, hi) in zip("xyz", ((-3000, 3000), (-4000, 4000), (100, 1800))):
        b["pos"][f] = rng.uniform(lo, hi, n)
    d = rng.normal(size=(n, 3))
    d *= (rng.uniform(0, 3000, n) / np.linalg.norm(d, axis=1))[:, None]
    for i, f in enumerate("xyz"):
        b["vel"][f] = d[:, i]
        b["ang_vel"][f] = rng.uniform(-3, 3, n)
    b["rot_mat"]["forward"]["x"] = b["rot_mat"]["right"]["y"] = b["rot_mat"]["up"]["z"] = 1
    return b


def run_ball_pred(args):
    """Batched BallPredTracker: full predictions (ForceUpdateAllPred of every arena from host states)
    and the incremental update after one tick of the source batch (UpdatePredFromArena: one new
    tick per arena), both through the C ABI, timed on the host around the synchronous calls."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import BALL_STATE_DTYPE, abi
    A, T = args.pred_arenas, args.pred_ticks
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, A, 1, 120.0)
    balls = _pred_balls(A, 4321, BALL_STATE_DTYPE)
    b.set_all_states(None, balls)
    tr = rsg.BallPredTracker(b, T)
    for _ in range(args.warmup):
        tr.force_update_all(balls)
    full = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tr.force_update_all(balls)
        full.append(time.perf_counter() - t0)
    tr.update_from_batch(b)
    inc = []
    for k in range(args.warmup + args.steps):
        b.step(1)
        t0 = time.perf_counter()
        tr.update_from_batch(b)
        if k >= args.warmup:
            inc.append(time.perf_counter() - t0)
    flags = int(np.count_nonzero(tr.device_flags()))
    tr.close()
    b.close()
    ms_full = statistics.median(full) * 1e3
    return {"value": A * (T - 1) / (ms_full / 1e3), "ms_full_prediction": ms_full,
            "ms_incremental_update": statistics.median(inc) * 1e3, "flagged_arenas": flags,
            "h2d_bytes_per_full_prediction": A * BALL_STATE_DTYPE.itemsize}


def ball_pred_cpu(seconds: float, T: int):
    """Ball-ticks/s of one CPU thread predicting: the reference's own BallPredTracker::ForceUpdateAllPred
    when the reference library is built here, else the CPU restatement stepping a ball-only arena
    T - 1 ticks per prediction in one native call (the per-tick state copy left out)."""
    from oracle.pyoracle import SimArena, BallState as OBallState
    from rocketsim_gb300.arena_mesh import arena_cmf
    kind = cpu_kind()
    a = SimArena(kind, arena_cmf(0))
    balls = [OBallState.from_buffer_copy(x.tobytes()) for x in _pred_balls(64, 4321, np.dtype(OBallState))]
    tr = a.ball_pred_tracker(T) if kind == "ref" else None
    n, i = 0, 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        if tr is not None:
            tr.force_update_all(balls[i % len(balls)])
        else:
            a.set_ball(balls[i % len(balls)])
            a.step(T - 1)
        n += T - 1
        i += 1
    el = time.perf_counter() - t0
    if tr is not None:
        tr.close()
    a.close()
    return n / el, n, el, kind


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arenas", type=int, default=4096)
    ap.add_argument("--cpu-seconds", type=float, default=1.5)
    ap.add_argument("--adj-instances", type=int, default=8192)
    ap.add_argument("--adj-check", type=int, default=4, help="instances checked against FP64 finite differences")
    ap.add_argument("--ground-instances", type=int, default=65536)
    ap.add_argument("--ground-check", type=int, default=256,
                    help="ground instances checked against FP64 finite differences")
    ap.add_argument("--pred-arenas", type=int, default=4096, help="arenas of the ball-prediction leg")
    ap.add_argument("--pred-ticks", type=int, default=360, help="predicted ticks per arena (BallPredTracker numPredTicks)")
    ap.add_argument("--settle-ticks", type=int, default=1200,
                    help="game ticks run before the warm-up steps, to time the steady state rather than the start")
    ap.add_argument("--c0-steps", type=int, default=10, help="timed 120-tick launches of the one-arena workload")
    ap.add_argument("--c2-arenas", type=int, default=16384, help="arenas of the uneven workload")
    ap.add_argument("--c2-steps", type=int, default=40, help="timed 8-tick steps of the uneven workload")
    ap.add_argument("--legs", default="all", help="comma list of extra legs: c0,c2,adjoint,ground,pred (or all / none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    # the launch-shape tuner's second round runs on a batch's first launch after 1024 ticks: keep it
    # in the settle ticks, out of the timed steps
    args.settle_ticks = max(args.settle_ticks, 1080)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    threads = os.cpu_count() or 1
    config = {"workload": WORKLOAD, "arenas": args.arenas, "cars_per_arena": CARS, "ticks_per_step": TICKS_PER_STEP,
              "tick_rate": 120, "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas{world}",
              "settle_ticks": args.settle_ticks}

    if args.impl == "reference":
        if rank != 0:
            return
        # each step: every host thread steps its own 2v2 arena for a bounded time
        vals, els = [], []
        kind = cpu_kind()
        for s in range(args.warmup + args.steps):
            v, n, el, kind = cpu_ticks_per_second(threads, 0.25 if s < args.warmup else 0.5, kind=kind)
            if s >= args.warmup:
                vals.append(v)
                els.append(el)
        value = statistics.mean(vals)
        line = {"impl": "reference", "metric": "2v2 arena-ticks/s", "value": value, "unit": "arena-ticks/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": statistics.mean(els) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": "arena-ticks/s", "cores": threads,
                                 "cpu_model": cpu_model(), "kind": "reference" if kind == "ref" else "port",
                                 "sample": f"{threads} threads x one 2v2 arena each, 0.5 s per step; "
                                           + reference_kind_note(kind)},
                "e2e": {"value": value, "unit": "arena-ticks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{int(os.environ.get('LOCAL_RANK', 0))}"))
    r = run_gpu(args, rank, world)
    if rank != 0:
        return
    dev = int(os.environ.get("LOCAL_RANK", 0))
    legs = set(["c0", "c2", "adjoint", "ground", "pred"] if args.legs == "all" else
               ([] if args.legs == "none" else args.legs.split(",")))
    single, _, _, kind = cpu_ticks_per_second(1, args.cpu_seconds)
    allc, n, el, _ = cpu_ticks_per_second(threads, args.cpu_seconds)
    line = {
        "metric": "2v2 arena-ticks/s", "value": r["value"], "unit": "arena-ticks/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
        "e2e": r["e2e"], "roofline": r["roofline"],
        "cpu_baseline": {"value": allc, "unit": "arena-ticks/s", "cores": threads, "cpu_model": cpu_model(),
                         "kind": "reference" if kind == "ref" else "port", "single_thread": single,
                         "sample": f"{threads} threads x one 2v2 arena each for {args.cpu_seconds:.1f} s "
                                   f"({n} arena-ticks) plus 1 thread for {args.cpu_seconds:.1f} s; "
                                   + reference_kind_note(kind)},
        "clocks": r["clocks"], "gpu_launches": r["gpu_launches"], "device_warn_flags": r["warn_flags_any"],
        "host": platform.machine(), "tick_shape": r["tick_shape"],
        "steady_state": {"game_tick_first_timed": r["game_tick_first_timed"],
                         "game_tick_last_timed": r["game_tick_last_timed"],
                         "ticks_per_s_vs_game_tick": r["ticks_per_s_vs_game_tick"]},
    }
    if "c0" in legs:
        c0 = run_config0(args, dev)
        line["config0_one_arena"] = {
            "metric": "2v2 ticks/s of one arena", "value": c0["value"], "unit": "ticks/s",
            "workload": "1 arena x (4 Octane + ball), procedural soccar mesh, the same input process; "
                        f"{args.c0_steps} timed launches of 120 ticks after {args.settle_ticks} + 360 ticks (a bounded "
                        "sample of the 1M-tick run)",
            "ms_per_launch": c0["ms_per_step"], "cpu_single_thread": single, "tick_shape": c0["tick_shape"]}
    if "c2" in legs:
        c2 = run_config2(args, dev)
        line["config2_uneven"] = {
            "metric": "arena-ticks/s", "value": c2["value"], "unit": "arena-ticks/s",
            "workload": f"{args.c2_arenas} arenas with 2/4/6 cars drawn 1:1:1 ({c2['cars']} cars), hitboxes drawn "
                        "uniformly from the six presets, 34 pads, 1% of the arenas reset to a random kickoff "
                        "every 300 ticks; 8 ticks per launch, L2 flushed between timed steps",
            "ms_per_step": c2["ms_per_step"], "steps": args.c2_steps,
            "game_tick_first_timed": c2["game_tick_first_timed"], "arenas_reset": c2["arenas_reset"],
            "ticks_per_s_vs_game_tick": c2["ticks_per_s_vs_game_tick"], "device_warn_flags": c2["warn_flags_any"],
            "clocks": c2["clocks"], "tick_shape": c2["tick_shape"]}
    if "adjoint" in legs:
        adj = run_adjoint(args, dev)
        adj_err, cpu_grads, cpu_el = adjoint_cpu_check(adj["case"], adj["g_gpu"], args.adj_check)
        line["adjoint"] = {
            "metric": "adjoint grads/s", "value": adj["value"], "unit": "grads/s (60-tick air rollouts)",
            "workload": ADJ_WORKLOAD, "rel_err_max_vs_fp64_fd": adj_err, "rel_err_instances": args.adj_check,
            "ms_per_step": adj["ms_per_step"], "step": adj["step_kind"],
            "eager_value": adj["eager_value"], "eager_ms_per_step": adj["eager_ms_per_step"],
            "ms_forward_with_checkpoints": adj["ms_forward_ckpt"],
            "ms_forward_plain": adj["ms_forward_plain"], "ms_backward": adj["ms_backward"],
            "backward_over_forward": adj["backward_over_forward"],
            "c_abi_ms_forward_with_checkpoints": adj["kernel_ms_forward_ckpt"],
            "c_abi_ms_backward": adj["kernel_ms_backward"],
            "c_abi_backward_over_forward": adj["kernel_backward_over_forward"],
            "workspace_bytes": adj["workspace_bytes"], "steps": args.steps, "warmup": args.warmup,
            "gpu_launches_per_step": 3,
            "cpu_baseline": {"value": cpu_grads, "unit": "grads/s", "cores": 1, "kind": "port",
                             "sample": f"FP64 central differences of the numpy restatement, "
                                       f"{args.adj_check} instances x 240 inputs x 2 rollouts ({cpu_el:.1f} s)"}}
    if "ground" in legs:
        gadj = run_ground_adjoint(args, dev)
        gchk = ground_cpu_check(gadj["case"], gadj["g_gpu"])
        line["ground_adjoint"] = {
            "metric": "adjoint grads/s", "value": gadj["value"], "unit": "grads/s (120-tick ground rollouts)",
            "workload": GROUND_WORKLOAD, "rel_err_max_vs_fp64_fd": gchk["max"], "rel_err_median": gchk["median"],
            "rel_err_sample": f"{args.ground_check} instances x {gchk['entries']} control entries; "
                              f"{gchk['nonsmooth']} instances left out whose central differences at steps 1e-4 "
                              f"and 5e-5 disagree (a jump inside the stencil; max over all {gchk['max_all']:.2e})",
            "ms_per_step": gadj["ms_per_step"], "step": "eager: forward + loss + backward",
            "ms_forward_with_checkpoints": gadj["ms_forward_ckpt"], "ms_forward_plain": gadj["ms_forward_plain"],
            "ms_backward": gadj["ms_backward"], "backward_over_forward": gadj["backward_over_forward"],
            "c_abi_ms_forward_with_checkpoints": gadj["kernel_ms_forward_ckpt"],
            "c_abi_ms_backward": gadj["kernel_ms_backward"], "workspace_bytes": gadj["workspace_bytes"],
            "c_abi_backward_over_forward": gadj["kernel_ms_backward"] / gadj["ms_forward_plain"],
            "flagged_instances": gadj["flagged_instances"], "gpu_launches_per_step": 3,
            "cpu_baseline": {"value": gchk["rate"], "unit": "gradient entries/s", "cores": 1, "kind": "port",
                             "sample": f"FP64 central differences of the numpy restatement, "
                                       f"{args.ground_check} instances x {gchk['entries']} entries x 2 rollouts "
                                       f"({gchk['seconds']:.1f} s)"}}
    if "pred" in legs:
        bp = run_ball_pred(args)
        bp_cpu, bp_n, bp_el, bp_kind = ball_pred_cpu(args.cpu_seconds, args.pred_ticks)
        line["ball_pred"] = {
            "metric": "predicted ball-ticks/s", "value": bp["value"], "unit": "ball-ticks/s",
            "workload": f"BallPredTracker over {args.pred_arenas} arenas x {args.pred_ticks} ticks, balls in flight "
                        f"(procedural soccar mesh seed 0); full prediction = ForceUpdateAllPred of every arena from "
                        f"host states",
            "ms_full_prediction": bp["ms_full_prediction"], "ms_incremental_update": bp["ms_incremental_update"],
            "h2d_bytes_per_full_prediction": bp["h2d_bytes_per_full_prediction"],
            "flagged_arenas": bp["flagged_arenas"], "gpu_launches_per_update": 2,
            "cpu_baseline": {"value": bp_cpu, "unit": "ball-ticks/s", "cores": 1,
                             "kind": "reference" if bp_kind == "ref" else "port",
                             "sample": f"one thread, {bp_n} predicted ticks in {bp_el:.1f} s: "
                                       + ("BallPredTracker::ForceUpdateAllPred of the reference built from its "
                                          "own sources (oracle/_ref)" if bp_kind == "ref" else
                                          "the CPU restatement (oracle/) stepping a ball-only arena, the per-tick "
                                          "state copy left out")}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
