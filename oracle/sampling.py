"""get_std_sampled_data restated on one oracle trajectory.

TEST INFRASTRUCTURE ONLY: tests/ compare the engine's on-device sampling
(kmc_pool_sample_* and kmos_gb300.sampling) with this restatement.  The product never
imports it.

It follows kmos.run.KMC_Model (mhoffman/kmos, kmos/run/__init__.py):
  __init__ / reset  run:261-273  tof_matrix from tof_count; procstat, integ_rates, time
                    and steps trackers start at zero
  get_atoms         run:779-848  TOF since the previous call:
                    tof = tof_matrix . ((X - X_prev) / delta_t / size), with
                    delta_steps = kmc_step - self.steps (self.steps is never updated:
                    the method stores self.step), so the "no steps" branch only fires
                    while kmc_step is 0
  get_std_sampled_data run:865-966  reset call, ``samples`` x (do_steps(sample_size /
                    samples), get_atoms), occupation averaged with weights
                    kmc_time_step, TOFs with weights delta_t, then
                    params + tofs + occupations + [total_time, simulated_time, total_steps]
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np


def tof_matrix(model):
    """run:261-267: rows are the sorted TOF names, columns the processes (file order)."""
    tofs = model.tof_names()
    pid = model.process_ids()
    mat = np.zeros((len(tofs), len(model.processes)))
    for p in sorted(model.processes, key=lambda q: q.name):
        for tof, factor in (p.tof_count or {}).items():
            mat[tofs.index(tof), pid[p.name] - 1] += factor
    return tofs, mat


class Trackers:
    """The KMC_Model attributes get_atoms reads and writes (run:269-273)."""

    def __init__(self, nproc: int, ntof: int):
        self.procstat = np.zeros(nproc, dtype=np.int64)
        self.integ_rates = np.zeros(nproc)
        self.time = 0.0
        self.steps = 0
        self.ntof = ntof


def get_atoms(o, trk: Trackers, tof_mat, size: int, nspecies: int):
    """run:779-848 with geometry=False, reset_time_overrun=False."""
    atoms = SimpleNamespace()
    atoms.kmc_time = o.kmc_time
    atoms.kmc_step = o.kmc_step
    atoms.procstat = np.zeros((o.P,))
    atoms.occupation = o.occupation(nspecies)
    atoms.procstat[:] = o.procstat()
    atoms.integ_rates = np.zeros((o.P,))
    atoms.integ_rates[:] = o.integ_rates()
    delta_t = atoms.kmc_time - trk.time
    delta_steps = atoms.kmc_step - trk.steps
    atoms.delta_t = delta_t
    if delta_steps == 0:
        atoms.tof_data = trk.tof_data if hasattr(trk, "tof_data") else np.zeros_like(tof_mat[:, 0])
        atoms.tof_integ = trk.tof_integ if hasattr(trk, "tof_integ") else np.zeros_like(tof_mat[:, 0])
    else:
        atoms.tof_data = np.dot(tof_mat, (atoms.procstat - trk.procstat) / delta_t / size)
        atoms.tof_integ = np.dot(tof_mat, (atoms.integ_rates - trk.integ_rates) / delta_t / size)
    trk.procstat[:] = atoms.procstat
    trk.integ_rates[:] = atoms.integ_rates
    trk.time = atoms.kmc_time
    trk.step = atoms.kmc_step
    trk.tof_data = atoms.tof_data
    trk.tof_integ = atoms.tof_integ
    return atoms


def std_sampled_data(o, trk: Trackers, tof_mat, size: int, nspecies: int, samples: int, sample_size: int,
                     tof_method: str = "integ", params=()):
    """run:865-966 with output="array": the outdata tuple as a numpy vector."""
    occs, tofs, delta_ts, step_ts = [], [], [], []
    t0 = o.kmc_time
    step0 = o.kmc_step
    get_atoms(o, trk, tof_mat, size, nspecies)
    for _ in range(samples):
        o.do_kmc_steps(int(sample_size / samples))
        atoms = get_atoms(o, trk, tof_mat, size, nspecies)
        delta_ts.append(atoms.delta_t)
        step_ts.append(o.kmc_time_step)
        occs.append(list(atoms.occupation.flatten()))
        if tof_method == "procrates":
            tofs.append(atoms.tof_data.flatten())
        elif tof_method == "integ":
            tofs.append(atoms.tof_integ.flatten())
        else:
            raise NotImplementedError(tof_method)
    occs_mean = np.average(occs, axis=0, weights=step_ts)
    tof_mean = np.average(tofs, axis=0, weights=delta_ts)
    total_time = o.kmc_time - t0
    simulated_time = o.kmc_time
    total_steps = o.kmc_step - step0
    return np.array(list(params) + list(tof_mean.flatten()) + list(occs_mean.flatten())
                    + [total_time, simulated_time, total_steps], dtype=np.float64)
