"""Aggregate kMC steps/s of the GB300 engine on one benchmark configuration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config C] [--impl ours|reference]

One bench *step* = one persistent launch in which every trajectory of the batch
advances ``--chunk`` kMC steps (do_kmc_steps on every trajectory).  The default
workload is configuration 3, the one the 100x target is quoted on: 2048 lat_int
trajectories of uneven square lattices (side 16..256, P=21, 6 lateral-interaction
groups).  ``--config 2`` is the 4096-trajectory 64x64 ZGB-type batch; its CO-rich
trajectories (y above ~0.525) reach the absorbing CO-poisoned state, where the
reference stops ("can't find available process") and the engine retires the
trajectory with a dead-lock status, so steps are always counted from the trajectories'
own kmc_step counters.  The resident state (about 6 GB for configuration 3) is far
larger than the 129 MB L2, so no explicit L2 flush is needed between steps.

``value`` is device-timed (CUDA events on the engine's stream around the K launches,
max over ranks); ``e2e`` is the same metric through the public pool API with the
per-step host->device run list and a device->host read of every trajectory's
procstat, integ_rates and clock.  ``--impl reference`` times the CPU restatement of the
reference step loop (the reference's Fortran build needs a Fortran compiler that this
machine does not have) on all host cores, on a bounded sample of the same workload.
Under torchrun each rank runs its own batch (trajectory ids offset by rank): weak
scaling, no collective on the data path.

After the timed region rank 0 adds the two other parts of the metric: ``plain_dropin``,
the steps/s of one trajectory of the workload through the handle API (the plain
one-trajectory drop-in the batched rate is compared with; ``--plain 0`` skips it), and
``serving``, p50 / p99 request latency and served steps/s of a short run of the serving
loop on the configuration-5 request stream (one GPU only; ``--serving 0`` skips it).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "aggregate kMC steps/s"
UNIT = "steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3, 4])
    ap.add_argument("--chunk", type=int, default=0, help="kMC steps per trajectory per bench step")
    ap.add_argument("--ntraj", type=int, default=0, help="override the trajectory count")
    ap.add_argument("--graph", type=int, default=1, help="replay the launch from a CUDA graph")
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--warps", type=int, default=-1,
                    help="warps per block (0: balanced, one block per SM); default: autotune or the pool's")
    ap.add_argument("--bps", type=int, default=0)
    ap.add_argument("--sides", default="", help="config 3: comma-separated lattice sides to draw from")
    ap.add_argument("--fast", type=int, default=1, help="gather / replay step path (0: serial interpreter)")
    ap.add_argument("--autotune", type=int, default=1, help="pick the launch shape on scratch trajectories first")
    ap.add_argument("--cpu-steps", type=int, default=0,
                    help="kMC steps per trajectory of the CPU sample (default: a 10-30 s sample per config)")
    ap.add_argument("--plain", type=int, default=1,
                    help="also time the plain drop-in: one trajectory of the workload through the handle API")
    ap.add_argument("--otf", type=int, default=1,
                    help="after the timed region: the otf backend on intZGB (kmc_otf_*)")
    ap.add_argument("--otf-only", type=int, default=0,
                    help="run only the otf sample (--otf-ntraj trajectories, --otf-steps timed steps) and print it")
    ap.add_argument("--otf-ntraj", type=int, default=2048)
    ap.add_argument("--otf-steps", type=int, default=0, help="timed otf steps per trajectory (0: OTF_TIMED)")
    ap.add_argument("--otf-phases", type=int, default=0,
                    help="with --otf-only: run the phase-timing build and add the step loop's cycles per step "
                         "by phase (that build's timing is not a bench figure)")
    ap.add_argument("--serving", type=int, default=1,
                    help="also run a short serving sample (configuration 5 stream, 1 s of arrivals, steps x 0.05)")
    return ap.parse_args()


# kMC steps per trajectory per bench step.  Config 3's 40 000 make the default
# --steps 20 --warmup 5 run (25 bench steps) the configuration's 1e6 steps per trajectory.
DEFAULT_CHUNK = {1: 100000, 2: 20000, 3: 40000, 4: 10000}


# ------------------------------------------------------------------ distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks sampler
class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.first = threading.Event()
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        # the first query of a fresh nvidia-smi can hold the driver for seconds, and a
        # launch made meanwhile waits for it: the timed region starts after the first
        # sample has arrived
        self.first.wait(timeout=30.0)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()
        self.first.set()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def stratified(wl, k: int):
    """k trajectory indices spread over the workload's parameters: the trajectories
    sorted by (lattice side, T) for config 3, by y for config 2 and by T for config 4,
    then taken at evenly spaced ranks (config 1 has one trajectory)."""
    n = wl.n
    notes = wl.notes
    if "side" in notes:
        key = lambda i: (int(notes["side"][i]), float(notes["T"][i]))  # noqa: E731
    elif "y" in notes:
        key = lambda i: float(notes["y"][i])  # noqa: E731
    elif "T" in notes:
        key = lambda i: float(notes["T"][i])  # noqa: E731
    else:
        key = lambda i: i  # noqa: E731
    order = sorted(range(n), key=key)
    return [order[min(n - 1, int((j + 0.5) * n / k))] for j in range(k)]


def _cpu_worker(args):
    """One trajectory of the workload on the oracle: `start` untimed steps (the part of
    the run before the GPU's timed region), then `steps` timed ones with the book-keeping
    access counters on.  Returns (steps done, seconds, int32 table accesses, occupation
    accesses) of the timed part."""
    config, ntraj, sides, idx, start, steps = args
    from kmos_gb300 import configs
    from oracle import oracle as O
    wl = configs.build(config, n=ntraj, sides=sides)
    o = O.Oracle(wl.program, wl.sizes[idx], seed=wl.seeds[idx], rng=O.RNG_PHILOX, traj=wl.trajs[idx])
    o.set_rates(wl.rates[idx])
    o.update_accum_rate()
    try:
        o.do_kmc_steps(start)
    except O.OracleError:
        return 0, 0.0, 0, 0  # absorbing state reached before the sample: nothing to time
    k0 = o.kmc_step
    o.reset_counters()
    t0 = time.perf_counter()
    try:
        o.do_kmc_steps(steps)
    except O.OracleError:
        pass  # absorbing state reached: the trajectory ends, as in the reference
    dt = time.perf_counter() - t0
    n_as, n_occ = o.counters()
    return o.kmc_step - k0, dt, n_as, n_occ


CPU_STEPS = {1: 2_000_000, 2: 1_000_000, 3: 800_000, 4: 1_000_000}
AUTOTUNE_PROBE_STEPS = 11 * 500   # steps the default autotune run advances every trajectory


def cpu_sample(config: int, start: int, steps: int, ntraj=None, sides=None):
    """The oracle (the CPU restatement of the reference loop) on all host cores, one
    process per core, on a stratified sample of the workload's trajectories (at least 16),
    each run through the same phase as the GPU's timed region: `start` untimed steps, then
    `steps` timed ones.  Returns (aggregate steps/s, cores, sample text, B_step, N_as, N_occ)
    with the per-step bytes averaged over the sampled trajectories."""
    from kmos_gb300 import configs
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    wl = configs.build(config, n=ntraj, sides=sides)
    k = max(16, cores)
    idxs = stratified(wl, k)
    ctx = mp.get_context("spawn")
    total, wall, per_step = 0, 0.0, []
    sum_as = sum_occ = 0.0
    with ctx.Pool(cores) as pool:
        for r in range(0, k, cores):
            # all workers of a round run at once; the slowest one's own timer bounds it
            res = pool.map(_cpu_worker, [(config, ntraj, sides, i, start, steps) for i in idxs[r:r + cores]])
            wall += max(t for _, t, _a, _o in res)
            total += sum(s for s, _t, _a, _o in res)
            for s_, _t, a_, o_ in res:
                if s_ > 0:
                    per_step.append((a_ / s_, o_ / s_))
    P = wl.program.nproc
    n_as = sum(a for a, _ in per_step) / max(1, len(per_step))
    n_occ = sum(o for _, o in per_step) / max(1, len(per_step))
    bstep = 20 * P + 28 * P + 28 + 4 * n_as + wl.occupation_bytes * n_occ
    sample = ("%d trajectories of config %d (stratified over the workload's parameters), each %d untimed then "
              "%d timed kMC steps, one process per core" % (k, config, start, steps))
    return total / wall, cores, sample, bstep, n_as, n_occ


OTF_RATES = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
OTF_PARAMS = [1.3, 0.7, 1.9, 1e-10, 0.5]   # J_CO_CO, J_O_CO, J_O_O, kDes, yCO


def _otf_model_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "models", "intZGB_otf.json")


OTF_WARM = 5000     # untimed otf steps per trajectory (the lattice fills from empty)
OTF_TIMED = 20000   # timed otf steps per trajectory, GPU and CPU alike
OTF_CPU_PER_CORE = 24


def _otf_cpu_worker(args):
    trajs, warm, steps = args
    from kmos_gb300 import model as M, program as PG
    from oracle import oracle as O
    prog = PG.compile_model(M.load_json(_otf_model_path()), "otf")
    busy = 0.0
    for traj in trajs:
        o = O.Oracle(prog, (32, 32), seed=11, rng=O.RNG_PHILOX, traj=traj)
        o.set_rates(OTF_RATES)
        o.set_user_parameters(OTF_PARAMS)
        o.recalculate_rates_matrix()
        o.update_accum_rate()
        o.do_kmc_steps(warm)
        t0 = time.perf_counter()
        o.do_kmc_steps(steps)
        busy += time.perf_counter() - t0
    return steps * len(trajs), busy


def otf_cpu_sample(warm: int = OTF_WARM, steps: int = OTF_TIMED, per_core: int = OTF_CPU_PER_CORE):
    """The oracle's otf backend on all host cores over the GPU sample's window: trajectories
    0 .. cores*per_core-1 of the GPU batch (same seed and Philox ids), each ``warm``
    untimed then ``steps`` timed steps, ``per_core`` trajectories in turn per core
    process: (aggregate steps/s, cores, sample)."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    work = [(list(range(c * per_core, (c + 1) * per_core)), warm, steps) for c in range(cores)]
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_otf_cpu_worker, work)
    busy = max(t for _, t in res)
    sample = ("%d trajectories (intZGB 32x32, ids 0-%d of the GPU batch), each %d untimed then %d timed otf steps, "
              "%d in turn per core process" % (cores * per_core, cores * per_core - 1, warm, steps, per_core))
    return sum(s for s, _ in res) / busy, cores, sample


def replica_trajs(trajs, rank: int):
    """Philox trajectory ids of one rank's replica batch: the same workload with ids
    offset by rank * batch size, so ranks run disjoint, reproducible trajectories."""
    n = len(trajs)
    return [int(t) + rank * n for t in trajs]


def timed_phase(args):
    """(untimed steps before the GPU's timed region, timed steps) per trajectory for
    the arguments given, with the default autotune run."""
    chunk = args.chunk or DEFAULT_CHUNK[args.config]
    return AUTOTUNE_PROBE_STEPS + args.warmup * chunk, args.steps * chunk


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        dist.close()
        return
    start, length = timed_phase(args)
    # K timed samples that tile the GPU's timed window of the same trajectories (sample j
    # runs its part of the window after the steps before it, untimed), the value the
    # aggregate rate over all of them -- the CPU's rate over the GPU's window; W warm-up
    # samples before them
    full = args.cpu_steps or min(length, CPU_STEPS[args.config])
    k = max(1, args.steps)
    per = max(1000, full // k)
    sides = [int(x) for x in args.sides.split(",")] if args.sides else None
    ntraj = args.ntraj or None
    warm = [cpu_sample(args.config, start, max(1000, per // 10), ntraj, sides) for _ in range(args.warmup)]
    vals, parts = [], []
    for j in range(k):
        n = per if j < k - 1 else max(1000, full - per * (k - 1))
        vals.append(cpu_sample(args.config, start + j * per, n, ntraj, sides))
        parts.append(n)
    value = sum(parts) / sum(n / v[0] for n, v in zip(parts, vals))
    cores = vals[0][1]
    sample = ("%s, one process per core; %d samples tiling steps %d-%d of each trajectory (%d warm-up "
              "samples first)" % (vals[0][2].split(", each")[0], k, start, start + sum(parts), len(warm)))
    from kmos_gb300 import configs
    wl = configs.build(args.config, n=1, steps=1)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(vals), "warmup": len(warm), "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "parallelism": "%d host processes" % cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference step loop (oracle/kmc_oracle.c); the reference's "
                "Fortran build is unavailable here (no Fortran compiler on this machine)",
    }
    print(json.dumps(line))
    dist.close()


# ------------------------------------------------------------------ GPU run
def run_ours(args, dist: Dist):
    from kmos_gb300 import configs, engine as E

    chunk = args.chunk or DEFAULT_CHUNK[args.config]
    sides = [int(x) for x in args.sides.split(",")] if args.sides else None
    wl = configs.build(args.config, n=args.ntraj or None, sides=sides)
    n = wl.n
    dev = dist.local
    E.load()
    # size the arena from the per-slot byte counts
    pool = E.Pool(arena_bytes=1 << 20, max_slots=1, device=dev)
    mid = pool.add_model(wl.program)
    per = sorted((pool.slot_bytes(mid, s) for s in wl.sizes), reverse=True)
    need = sum(per)
    pool.close()
    pool = E.Pool(arena_bytes=need + (64 << 20), max_slots=n, device=dev)
    if args.warps >= 0:
        pool.set_launch(args.warps, args.bps)
    if not args.fast:
        pool.set_fast_path(False)
    mid = pool.add_model(wl.program)
    trajs = replica_trajs(wl.trajs, dist.rank)
    slots = []
    B = 1024
    for i in range(0, n, B):
        slots += pool.admit_many([mid] * len(wl.sizes[i:i + B]), wl.sizes[i:i + B], wl.rates[i:i + B],
                                 seeds=wl.seeds[i:i + B], rng=E.RNG_PHILOX, trajs=trajs[i:i + B])
    # longest lattices first so uneven work balances across warps
    order = sorted(range(n), key=lambda i: -wl.sizes[i][0] * wl.sizes[i][1])
    slots = [slots[i] for i in order]
    P = wl.program.nproc

    spl = chunk  # kMC steps per launch; a bench step is chunk / spl launches

    def launch():
        for _ in range(chunk // spl):
            if args.graph:
                pool.run_graph(slots, spl, sync=False)
            else:
                pool.run(slots, spl, sync=False)

    tuned = None
    nwarm = args.warmup
    if args.autotune and not (args.warps >= 0 or args.bps or not args.fast):
        # part of the warm-up: probes advance the real trajectories (results do not
        # depend on the launch shape)
        from kmos_gb300 import autotune
        tuned = autotune.tune(pool, slots)
        tuned["trials"] = [{k: r[k] for k in ("fast", "warps", "tables", "tpw", "steps_per_s") if k in r}
                           for r in tuned["trials"]]
        if args.graph and args.warmup >= 1:
            # the first warm-up bench steps are the steps-per-launch trials: each runs
            # one bench step's chunk as 1, 2 or 4 launches
            t2 = autotune.tune_steps_per_launch(pool, slots, chunk, splits=(1, 2, 4)[:args.warmup])
            spl = t2["steps_per_launch"]
            nwarm -= len(t2["trials"])
            tuned["steps_per_launch"] = spl
            tuned["steps_per_launch_trials"] = [{k: r[k] for k in ("launches", "steps_per_s")} for r in t2["trials"]]
    for _ in range(max(0, nwarm)):
        launch()
    pool.sync()
    _ps, _ig, _t, ksteps0, _st = pool.results(slots, P)

    clocks = Clocks(dev)
    dist.barrier()
    pool.sync()
    launches0 = pool.launch_count()
    clocks.start()
    pool.timer_start()
    for _ in range(args.steps):
        launch()
    ms = pool.timer_stop()
    clk = clocks.stop()
    launches = pool.launch_count() - launches0
    dist.barrier()
    ms = dist.max(ms)
    _ps, _ig, _t, ksteps, status = pool.results(slots, P)
    bad = set(status.tolist()) - {0, 3}
    if bad:
        raise SystemExit("trajectories ended with status %s" % sorted(bad))
    if not (ksteps - ksteps0 <= args.steps * chunk).all() or not ((ksteps - ksteps0 == args.steps * chunk) | (status == 3)).all():
        raise SystemExit("step counters disagree with the launches")
    kmc_steps_rank = int((ksteps - ksteps0).sum())
    active = int((status == 0).sum())
    total_steps = dist.sum(kmc_steps_rank)
    value = total_steps / (ms / 1e3)

    # end to end through the public API: host run list in, every trajectory's
    # procstat / integ_rates / clock out, each step
    e2e_steps = max(2, min(args.steps, 5))
    dist.barrier()
    k_before = ksteps
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for _l in range(chunk // spl):
            pool.run(slots, spl, sync=False)
        res = pool.results(slots, P)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = dist.sum(int((res[3] - k_before).sum())) / e2e_s
    h2d = n * 4 + n * 8
    d2h = n * P * 16 + n * (8 + 8 + 4)

    line = None
    if dist.rank == 0:
        import json as _json
        peaks = {}
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            peaks = _json.load(open(pk))
        peak = peaks.get("hbm_gbs", 6800.0)
        # the oracle on a stratified sample of the workload, through the same phase of the
        # run as the timed region: B_step (mean over the sample) and the CPU baseline
        import numpy as _np
        start = int(_np.median(ksteps0))
        cpu_steps = args.cpu_steps or min(args.steps * chunk, CPU_STEPS[args.config])
        v, cores, sample, bstep, n_as, n_occ = cpu_sample(args.config, start, cpu_steps, args.ntraj or None, sides)
        # per launch: the kernel's bytes over its average duration
        launches_timed = args.steps * (chunk // spl)
        per_launch_s = (ms / 1e3) / launches_timed
        achieved = bstep * (kmc_steps_rank / launches_timed) / per_launch_s / 1e9
        traffic = None
        prof = os.path.join(ROOT, "profiles", "traffic_config%d.json" % args.config)
        if os.path.exists(prof):
            tr = _json.load(open(prof))
            traffic = tr.get("bytes_per_kmc_step", 0) * kmc_steps_rank / launches_timed
        cpu = None
        if args.cpu_baseline:
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "trajectories_per_gpu": n, "kmc_steps_per_traj_per_step": chunk,
                       "timed_kmc_steps_per_traj": [start, start + args.steps * chunk],
                       "active_at_end": active,
                       "lattice": "x".join(str(v) for v in wl.sizes[0][:2]) if args.config != 3 else "uneven 16..256",
                       "nproc": P, "backend": wl.backend, "rng": "philox4x32-10",
                       "parallelism": "replicas%d" % dist.world, "graph": bool(args.graph), "autotune": tuned,
                       "l2": "resident state %.2f GB > L2, no flush" % (need / 1e9)},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "bytes_per_kmc_step": bstep, "n_as": n_as, "n_occ": n_occ,
                         "bytes_sample": "mean over the cpu_baseline sample's trajectories",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
    pool.close()
    # samples measured after the timed region; a failure in one is recorded in its key
    # and never costs the line itself
    extras = []
    if line is not None and args.plain:
        extras.append(("plain_dropin", lambda: plain_dropin(wl)))
        if args.config != 1:
            extras.append(("plain_dropin_config1", lambda: plain_dropin(configs.build(1), steps=200000)))
    if line is not None and args.serving and dist.world == 1:
        extras.append(("serving", serving_sample))
    if line is not None and args.otf and dist.world == 1:
        extras.append(("otf", lambda: otf_sample(args.cpu_baseline, args.otf_ntraj, args.otf_steps)))
    for key, fn in extras:
        try:
            line[key] = fn()
        except Exception as e:  # noqa: BLE001
            line[key] = {"error": "%s: %s" % (type(e).__name__, e)}
    if line is not None:
        print(json.dumps(line))
    dist.close()


def plain_dropin(wl, steps: int = 20000):
    """The plain method: one trajectory of the workload (its first) stepped through the
    handle API (kmc_create / kmc_do_steps, what the f2py module calls), after the timed
    region; wall time of the do_kmc_steps call, as `kmos benchmark` times it
    (kmos/cli.py:293-312)."""
    from kmos_gb300 import engine as E
    with E.Trajectory(wl.program, wl.sizes[0], seed=wl.seeds[0], rng=E.RNG_PHILOX, traj=wl.trajs[0]) as g:
        g.set_rates(wl.rates[0])
        g.update_accum_rate()
        g.do_kmc_steps(2000)
        t0 = time.perf_counter()
        g.do_kmc_steps(steps)
        dt = time.perf_counter() - t0
    size = "x".join(str(v) for v in wl.sizes[0][:2])
    return {"value": steps / dt, "unit": UNIT, "trajectory": "%s, lattice %s, trajectory 0" % (wl.name, size),
            "steps": steps}


def serving_sample():
    """A short run of the serving loop on the configuration-5 request stream (1 s of
    Poisson arrivals at 500/s, steps x 0.05), after the timed region: p50 / p99 request
    latency and served steps/s."""
    from kmos_gb300 import configs, serving
    reqs, progs = configs.serving_requests(rate=500.0, duration=1.0, steps_scale=0.05)
    srv = serving.Server(arena_bytes=16 << 30, max_slots=4096, quantum=20000, policy="fifo")
    for k, p in progs.items():
        srv.add_model(k, p)
    t0 = time.perf_counter()
    done = srv.serve(reqs)
    wall = time.perf_counter() - t0
    stats = serving.latency_stats(done)
    out = {"requests": len(reqs), "rate_per_s": 500.0, "duration_s": 1.0, "steps_scale": 0.05,
           "served_steps_per_s": srv.kmc_steps / wall, "wall_s": wall, **stats}
    srv.close()
    return out


OTF_PHASES = ["draws", "running sums and accum_rates", "clock and integ_rates", "pick", "event op list",
              "event evaluation", "event replay"]


def otf_sample(cpu: int = 1, ntraj: int = 2048, fixed_steps: int = 0, phases: bool = False):
    """The otf backend (per-entry rates from bystanders) after the timed region: intZGB
    (tests/golden/models/intZGB_otf.json, the reference's tests/export_test/intZGB_otf.xml)
    on a 32 x 32 lattice, 2048 Philox trajectories from an empty lattice: OTF_WARM
    untimed steps, then steps/s over every trajectory from CUDA events around one
    do_kmc_steps launch of OTF_TIMED steps (inputs resident), beside the oracle's otf
    backend on every host core over the same window of the same trajectories."""
    from kmos_gb300 import engine as E, model as M, otf as OTF, program as PG
    m = M.load_json(_otf_model_path())
    prog = PG.compile_model(m, "otf")
    rates, params = OTF_RATES, OTF_PARAMS
    size = (32, 32)
    b = E.OtfBatch(prog, size, ntraj=ntraj, seed=11, rng=E.RNG_PHILOX)
    b.set_rates(rates)
    b.set_user_parameters(params)
    b.recalculate_rates_matrix()
    b.update_accum_rate()
    b.do_kmc_steps(OTF_WARM)                  # untimed: the lattice fills from empty
    steps = fixed_steps or OTF_TIMED
    if phases:
        b.phase_cycles(reset=True)
    b.do_kmc_steps(steps)
    ms = b.last_kernel_ms()
    out = {"workload": "intZGB otf, 32x32, %d trajectories" % ntraj, "window": [OTF_WARM, OTF_WARM + steps],
           "steps_per_traj": steps, "kernel_ms": ms, "steps_per_s": ntraj * steps / (ms * 1e-3), "gpu_launches": 1,
           "rate_table_entries": b.rate_table_entries()}
    if phases:  # cycles of one trajectory's step, by phase (clock64 on lane 0, summed over warps)
        cyc = b.phase_cycles(reset=True)[:len(OTF_PHASES)].astype(float) / (ntraj * steps)
        out["build"] = "phase timing (KMC_PHASE_TIMING): slower than the product build"
        out["cycles_per_step"] = {n: round(float(c), 1) for n, c in zip(OTF_PHASES, cyc)}
        out["cycles_per_step_total"] = round(float(cyc.sum()), 1)
    b.close()
    if cpu:
        value, cores, sample = otf_cpu_sample(OTF_WARM, steps)
        out["cpu_baseline"] = {"value": value, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample}
        out["speedup_vs_cpu"] = out["steps_per_s"] / value
    return out


def main():
    args = parse()
    if args.otf_phases and not args.otf_only:
        raise SystemExit("--otf-phases needs --otf-only 1")
    if args.otf_only:
        if args.otf_phases:
            from kmos_gb300 import build as _build
            os.environ["KMC_GB300_LIB"] = _build.build(phase_timing=True)
        print(json.dumps(otf_sample(args.cpu_baseline, args.otf_ntraj, args.otf_steps, bool(args.otf_phases))))
        return
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
