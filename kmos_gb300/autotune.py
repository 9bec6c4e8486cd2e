"""Launch-shape autotuner for the step kernel.

The step results do not depend on the launch shape (each trajectory's steps are the
same whatever warp runs them), so tuning runs short launches on the *real* trajectories:
each probe advances them by ``probe_steps`` steps, which the caller counts as warm-up or
as part of the requested steps.  It picks the launch shape (the balanced one-block-per-SM
shape, or 2, 4 or 8 warps per block with as many blocks as fit), the step path (gather /
replay or serial interpreter) and the table placement (the model's hot section in shared
memory or read from global memory) with the highest measured steps/s, sets them on the
pool, and returns steps per launch for about ``target_ms`` per launch.
"""
from __future__ import annotations

from typing import Dict, List, Sequence

from . import engine as E


def tune(pool: E.Pool, slots: Sequence[int], probe_steps: int = 500, target_ms: float = 100.0,
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
    per_traj_rate = best["steps_per_s"] / len(slots)
    steps = int(max(1000, min(1_000_000, per_traj_rate * target_ms / 1e3)))
    return {"warps_per_block": best["warps"], "fast_path": best["fast"], "tables": best.get("tables", "shared"),
            "steps_per_launch": steps,
            "probe_steps_per_trajectory": probe_steps * len(results), "trials": results}
