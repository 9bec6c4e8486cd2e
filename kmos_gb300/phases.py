"""Per-phase cycle accounting of the step kernels on one benchmark workload.

    python -m kmos_gb300.phases [--config C] [--ntraj N] [--steps S] [--solo 0|1] [--fast 0|1]

Builds the library with KMC_PHASE_TIMING (libkmcgb300_timing.so, a separate file; the
product library is untouched), runs the workload's trajectories for S steps after a
warm-up and prints one JSON line: steps/s of the timing build and the cycles per kMC step
each phase took, summed over the launch's groups and divided by the steps.  The phase
marks themselves cost a few cycles each.  Phases of the solo kernel (lane 0): draws and
the batch's clock and integ, accum, bisection and site, trace, site coordinates,
run_proc_nr, term refresh.  Phases of the group kernel: the 16 marks listed at
kmc_pool_phase_cycles in include/kmc_gb300.h.
"""
from __future__ import annotations

import argparse
import json
import os


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=1, choices=[1, 2, 3, 4])
    ap.add_argument("--ntraj", type=int, default=1)
    ap.add_argument("--sides", default="", help="config 3: comma-separated lattice sides")
    ap.add_argument("--steps", type=int, default=200000)
    ap.add_argument("--warmup", type=int, default=20000)
    ap.add_argument("--solo", type=int, default=1)
    ap.add_argument("--fast", type=int, default=1)
    ap.add_argument("--otf", type=int, default=0,
                    help="the otf backend instead: intZGB (tests/golden/models/intZGB_otf.json), 32 x 32, --ntraj")
    a = ap.parse_args(argv)
    from . import build
    os.environ["KMC_GB300_LIB"] = build.build(phase_timing=True)
    if a.otf:
        return otf_phases(a)
    from . import configs, engine as E
    sides = [int(x) for x in a.sides.split(",")] if a.sides else None
    wl = configs.build(a.config, n=a.ntraj, steps=0, sides=sides)
    probe = E.Pool(arena_bytes=1 << 20, max_slots=1)
    pmid = probe.add_model(wl.program)
    need = sum(probe.slot_bytes(pmid, sz) for sz in wl.sizes)
    probe.close()
    pool = E.Pool(arena_bytes=need + (64 << 20), max_slots=max(4, wl.n))
    pool.set_solo(bool(a.solo))
    pool.set_fast_path(bool(a.fast))
    mid = pool.add_model(wl.program)
    slots = pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
    pool.run(slots, a.warmup)
    pool.phase_cycles(reset=True)
    pool.timer_start()
    pool.run(slots, a.steps, sync=False)
    ms = pool.timer_stop()
    total = wl.n * a.steps
    ph = pool.phase_cycles(reset=True).astype(float) / total
    line = {"workload": wl.name, "trajectories": wl.n, "steps_per_traj": a.steps, "solo": a.solo, "fast": a.fast,
            "steps_per_s_timing_build": total / ms * 1e3,
            "cycles_per_step_by_phase": [round(float(x), 1) for x in ph]}
    pool.close()
    print(json.dumps(line))
    return line


def otf_phases(a):
    """The otf step loop's phases on intZGB (the bench's otf sample model and rates)."""
    from . import engine as E, model as M, program as PG
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    m = M.load_json(os.path.join(root, "tests", "golden", "models", "intZGB_otf.json"))
    prog = PG.compile_model(m, "otf")
    b = E.OtfBatch(prog, (32, 32), ntraj=a.ntraj, seed=11, rng=E.RNG_PHILOX)
    b.set_rates([0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3])
    b.set_user_parameters([1.3, 0.7, 1.9, 1e-10, 0.5])
    b.recalculate_rates_matrix()
    b.update_accum_rate()
    b.do_kmc_steps(a.warmup)
    b.phase_cycles(reset=True)
    b.do_kmc_steps(a.steps)
    ms = b.last_kernel_ms()
    total = a.ntraj * a.steps
    ph = b.phase_cycles(reset=True).astype(float) / total
    line = {"workload": "intZGB otf 32x32", "trajectories": a.ntraj, "steps_per_traj": a.steps,
            "steps_per_s_timing_build": total / ms * 1e3,
            "cycles_per_step_by_phase": [round(float(x), 1) for x in ph]}
    b.close()
    print(json.dumps(line))
    return line


if __name__ == "__main__":
    main()
