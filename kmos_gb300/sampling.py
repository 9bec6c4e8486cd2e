"""Standardised sampled output for a batch of resident trajectories.

kmos.run.KMC_Model.get_std_sampled_data (mhoffman/kmos, kmos/run/__init__.py:865-966)
runs one model for ``samples`` batches of ``sample_size / samples`` kMC steps, reads the
counters and the occupation after each batch through the f2py getters, and returns
``[parameters] [TOFs] [occupations] kmc_time simulated_time kmc_steps`` with the
occupations averaged with weights kmc_time_step and the TOFs with weights delta_t.

Here every listed trajectory of a pool is sampled at once: the batches, the occupation
reductions and the weighted sums stay on the device (``kmc_pool_sample_run``), and one
transfer at the end brings back per trajectory the mean occupation and the counter
differences.  The TOFs follow from those: the delta_t-weighted mean of the per-batch
``tof_matrix . (dX / delta_t / size)`` is ``tof_matrix . (dX_total / total_time / size)``
(equal up to rounding, about 1e-15 relative).  Where a trajectory's sampled time or every
weight is zero the values are NaN (the reference divides by zero there).
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from . import engine as E


def tof_matrix(model):
    """TOF names (sorted) and the [ntof, nproc] matrix of tof_count factors
    (run/__init__.py:261-267, get_tof_names run:2452-2459)."""
    names = model.tof_names()
    pid = model.process_ids()
    mat = np.zeros((len(names), len(model.processes)))
    for p in sorted(model.processes, key=lambda q: q.name):
        for tof, factor in (p.tof_count or {}).items():
            mat[names.index(tof), pid[p.name] - 1] += factor
    return names, mat


def param_names(model) -> List[str]:
    """Adjustable parameters in sorted order (get_param_header, run:351-360)."""
    return sorted(p.name for p in model.parameters if p.adjustable)


def occupation_names(model) -> List[str]:
    """``<species>_<layer>_<site>`` for sorted species x sites (get_occupation_header,
    run:362-373, with settings.site_names as the export writes it, io:3813-3814)."""
    sites = ["%s_%s" % (layer, site.name) for layer, site in model.site_list()]
    return ["%s_%s" % (sp, st) for sp in sorted(model.species) for st in sites]


def _float(text) -> float:
    try:
        return float(text)
    except (TypeError, ValueError):
        return float("nan")


def std_header(model) -> str:
    """get_std_header (run/__init__.py:841-852)."""
    return "#%s %s %s kmc_time simulated_time kmc_steps\n" % (
        " ".join(param_names(model)), " ".join(tof_matrix(model)[0]), " ".join(occupation_names(model)))


def get_std_sampled_data(pool: E.Pool, slots: Sequence[int], model, samples: int, sample_size: int,
                         tof_method: str = "integ", output: str = "array", params=None):
    """Samples every slot (all of ``model``) as get_std_sampled_data does.

    ``params``: the adjustable parameter values per slot ([n, k] or one row for all),
    which lead each output row as ``atoms.params`` does (default: the model's values).  ``output``: "array" (an
    [n, k + ntof + nocc + 3] float64 array), "str" (one "%.5e" line per slot) or "dict"
    (one header -> value dict per slot)."""
    if tof_method not in ("procrates", "integ"):
        raise NotImplementedError('tof_method="%s" not supported. Can be either procrates or integ.' % tof_method)
    slots = [int(s) for s in slots]
    n = len(slots)
    names, mat = tof_matrix(model)
    nocc = len(model.species) * model.spuck
    steps = int(sample_size / samples)
    out = pool.sample_run(slots, samples, steps)
    P = len(model.processes)
    cells = np.array([pool.volume(s) // model.spuck for s in slots], dtype=np.float64)
    total_time = out["times"][:, 0]
    if tof_method == "procrates":
        dx = out["dprocstat"][:, :P].astype(np.float64)
    else:
        dx = out["dinteg"][:, :P]
    with np.errstate(divide="ignore", invalid="ignore"):
        tofs = (dx / total_time[:, None] / cells[:, None]) @ mat.T
    if params is None:  # the model's own values, as atoms.params reads settings.parameters
        vals = {p.name: p.value for p in model.parameters}
        prm = np.array([[_float(vals[k]) for k in param_names(model)]] * n, dtype=np.float64).reshape(n, -1)
    else:
        prm = np.asarray(params, dtype=np.float64)
        prm = np.broadcast_to(prm.reshape(1, -1) if prm.ndim == 1 else prm, (n, prm.shape[-1]))
    data = np.concatenate([prm, tofs, out["occ"][:, :nocc], total_time[:, None], out["times"][:, 1:2],
                           out["steps"][:, None].astype(np.float64)], axis=1)
    if output == "array":
        return data
    if output == "str":
        return [(" ".join(["%.5e"] * data.shape[1]) + "\n") % tuple(row) for row in data]
    if output == "dict":
        header = std_header(model)[1:].split()
        return [dict(zip(header, row)) for row in data]
    raise UserWarning("Output format %s not defined. I only know 'str' and 'dict'" % output)
