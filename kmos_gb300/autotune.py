"""Launch-shape autotuner for the step kernel.

The step results do not depend on the launch shape (each trajectory's steps are the
same whatever warp runs them), so tuning runs short launches on the *real* trajectories:
each probe advances them by ``probe_steps`` steps, which the caller counts as warm-up or
as part of the requested steps.  It picks the launch shape (the balanced one-block-per-SM
shape, or 2, 4 or 8 warps per block with as many blocks as fit), the step path (gather /
replay or serial interpreter), the table placement (the model's hot section in shared
memory or read from global memory) and the trajectories per warp (one on 32 lanes, or two
on 16 lanes each) with the highest measured steps/s and sets them on the pool (``tune``,
11 probes); then, for runs of a given length, how many steps each launch takes
(``tune_steps_per_launch``).
"""
from __future__ import annotations

from typing import Dict, List, Sequence

from . import engine as E


def tune(pool: E.Pool, slots: Sequence[int], probe_steps: int = 500,
         warps=(0, 2, 4, 8), paths=(True, False)) -> Dict:
    results: List[Dict] = []
    for fast in paths:
        for w in warps:
            pool.set_fast_path(fast)
            pool.set_launch(w, 0)
            pool.timer_start()
            pool.run(slots, probe_steps, sync=False)
            ms = pool.timer_stop()
            results.append({"fast": fast, "warps": w, "ms": ms,
                            "steps_per_s": len(slots) * probe_steps / ms * 1e3})
    best = max(results, key=lambda r: r["steps_per_s"])
    pool.set_fast_path(best["fast"])
    pool.set_launch(best["warps"], 0)
    # table placement: the hot section read from global memory instead of shared
    pool.set_table_placement(False)
    pool.timer_start()
    pool.run(slots, probe_steps, sync=False)
    ms = pool.timer_stop()
    trial = {"fast": best["fast"], "warps": best["warps"], "tables": "global", "ms": ms,
             "steps_per_s": len(slots) * probe_steps / ms * 1e3}
    results.append(trial)
    if trial["steps_per_s"] > best["steps_per_s"]:
        best = trial
    else:
        pool.set_table_placement(True)
    # trajectories per warp: two half-warp groups per warp, with the best shape and with
    # the balanced one (or 4 warps per block when the balanced one was the best)
    best.setdefault("tables", "shared")
    best["tpw"] = 1
    for w in (best["warps"], 0 if best["warps"] else 4):
        pool.set_trajectories_per_warp(2)
        pool.set_launch(w, 0)
        pool.timer_start()
        pool.run(slots, probe_steps, sync=False)
        ms = pool.timer_stop()
        trial = {"fast": best["fast"], "warps": w, "tables": best["tables"], "tpw": 2, "ms": ms,
                 "steps_per_s": len(slots) * probe_steps / ms * 1e3}
        results.append(trial)
        if trial["steps_per_s"] > best["steps_per_s"]:
            best = trial
    pool.set_trajectories_per_warp(best["tpw"])
    pool.set_launch(best["warps"], 0)
    return {"warps_per_block": best["warps"], "fast_path": best["fast"], "tables": best["tables"],
            "trajectories_per_warp": best["tpw"],
            "probe_steps_per_trajectory": probe_steps * len(results), "trials": results}


def tune_steps_per_launch(pool: E.Pool, slots: Sequence[int], total: int, splits=(1, 2, 4)) -> Dict:
    """Steps per launch for runs of ``total`` kMC steps per trajectory.  Candidate ``s``
    runs the ``total`` steps as ``s`` replays of a captured launch of ``total / s`` steps
    on the real trajectories (which the caller counts as warm-up); the candidate with the
    least device time (CUDA events around each replay, capture excluded) wins.  A launch
    ends when its slowest trajectory has done its steps, so fewer, longer launches pay
    that tail less often; shorter ones hand control back to the host sooner."""
    trials = []
    for s in splits:
        if total % s:
            continue
        spl = total // s
        ms = 0.0
        for _ in range(s):
            pool.run_graph(slots, spl, sync=True)
            ms += pool.last_kernel_ms()
        trials.append({"launches": s, "steps_per_launch": spl, "ms": ms,
                       "steps_per_s": len(slots) * total / ms * 1e3})
    best = max(trials, key=lambda r: r["steps_per_s"])
    return {"steps_per_launch": best["steps_per_launch"], "launches_per_run": best["launches"],
            "probe_steps_per_trajectory": total * len(trials), "trials": trials}
