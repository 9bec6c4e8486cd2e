"""Drop-in for kmos's f2py module ``kmc_model``: ``base``, ``lattice`` and ``proclist``
with the names, argument conventions and return values of the generated Fortran
modules, running on the GB300 engine.

kmos builds ``kmc_model`` per model with f2py (kmos/utils/__init__.py:406-521) and
``kmos.run`` imports ``base, lattice, proclist`` from it (kmos/run/__init__.py:86-114).
Here one call configures the three namespaces for a model::

    from kmos_gb300 import kmc_model
    base, lattice, proclist = kmc_model.configure("model.ini", backend="local_smart")

(``kmos_gb300.export`` writes a ``kmc_model.py`` that does this, so ``kmos.run`` imports
it unchanged).  Without an explicit call, the first access to ``base``, ``lattice`` or
``proclist`` configures them from the ``kmc_settings`` module of the export directory:
its ``model_json`` (written by ``kmos_gb300.export``) or the project ``xml`` kmos's own
export writes there; the backend comes from ``kmc_settings.backend`` or the
``KMOS_GB300_BACKEND`` environment variable (default local_smart).  f2py lower-cases Fortran names, so process, species and site constants
are lower-case attributes.  Sites are passed as 4-vectors ``(x, y, z, n)`` where the
Fortran takes ``integer, dimension(4)``, and as 1-based indices where it takes ``nr``.

State lives on the GPU from ``proclist.init`` to ``lattice.deallocate_system``; getters
copy what they return.  Where the Fortran would ``stop``, a ``KMCError`` is raised.
"""
from __future__ import annotations

import time
import types
from typing import Optional

import numpy as np

from . import engine as E
from .model import Model, from_dict, load
from .program import compile_model


class _OtfTrajectory:
    """One otf trajectory (``engine.OtfBatch`` of one, on the gfortran stream of the
    seed) behind the calls the base / lattice / proclist namespaces make."""

    def __init__(self, program, size, layer: int, seed: int):
        self.b = E.OtfBatch(program, size, ntraj=1, layer=layer, seed=seed, rng=E.RNG_GFORTRAN)
        self.P, self.V, self.spuck = self.b.P, self.b.V, self.b.spuck
        self.nspecies = int(program.words[4])
        self.cells = self.V // self.spuck
        self._rates = np.zeros(self.P)
        self._t0 = time.time()

    def close(self):
        self.b.close()

    def _get(self, *fields):
        return self.b.state(0, fields)

    def set_rate_const(self, proc: int, rate: float):
        self.b.set_rate_const(proc, rate)
        self._rates[proc - 1] = rate

    def update_accum_rate(self):
        self.b.update_accum_rate()

    def update_integ_rate(self):
        self.b.update_integ_rate()

    def recalculate_rates_matrix(self):
        self.b.recalculate_rates_matrix()

    def do_kmc_steps(self, n: int):
        self.b.do_kmc_steps(n)

    def get_next_kmc_step(self):
        return self.b.get_next_kmc_step(0)

    def run_proc_nr(self, proc: int, site: int):
        self.b.run_proc_nr(proc, site, 0)

    @property
    def kmc_time(self) -> float:
        return self._get("clock")["kmc_time"]

    @kmc_time.setter
    def kmc_time(self, t: float):
        self.b.set_kmc_time(0, t)

    @property
    def kmc_time_step(self) -> float:
        return self._get("clock")["kmc_time_step"]

    @property
    def kmc_step(self) -> int:
        return self._get("clock")["kmc_step"]

    @property
    def walltime(self) -> float:
        return time.time() - self._t0

    def procstat(self):
        return self._get("procstat")["procstat"]

    def rates(self):
        return self._rates.copy()

    def integ_rates(self):
        return self._get("integ")["integ"]

    def accum_rates(self):
        return self._get("accum")["accum"]

    def nr_of_sites(self):
        return self._get("nsites")["nsites"]

    def get_rate(self, proc: int, site: int = -1) -> float:
        """base.get_rate (base_otf.f90:1121-1145): rates_matrix(proc, site), or the
        process total rates_matrix(proc, V+1) for site -1."""
        if site == -1:
            return float(self._get("totals")["totals"][proc - 1])
        return float(self._get("rates_matrix")["rates_matrix"][proc - 1, site])

    def avail_site(self, proc: int, idx: int, sw: int) -> int:
        key = "as1" if sw == 1 else "as2"
        return int(self._get(key)[key][proc - 1, idx])

    def get_species(self, nr: int) -> int:
        return int(self._get("lattice")["lattice"][nr - 1])

    def occupation(self) -> np.ndarray:
        """get_occupation (proclist_generic_subroutines.mpy:113-158): species per site
        index, divided by the number of cells."""
        lat = self._get("lattice")["lattice"].reshape(-1, self.spuck)
        occ = np.zeros((self.nspecies, self.spuck))
        for sp in range(self.nspecies):
            occ[sp] = (lat == sp).sum(axis=0) / self.cells
        return occ

    def replace_species(self, site: int, old: int, new: int):
        self.b.replace_species(0, site, old, new)

    def touchup_many(self, sites):
        """touchup_cell of the cells whose first sites are ``sites``, in order (the
        _State queue holds site numbers)."""
        X, Y = self.b.size[0], self.b.size[1]
        c = (np.asarray(sites, dtype=np.int64) - 1) // self.spuck
        self.b.touchup_cells(0, np.stack([c % X, (c // X) % Y, c // (X * Y)], axis=1))

    def save_reload(self, path: str):
        self.b.save_reload(0, path, self.walltime)

    def load_reload(self, path: str):
        """The file's state, rate constants and walltime (base_otf.f90:448-599)."""
        w = self.b.load_reload(0, path)
        self._rates = self.b.rate_consts()
        self._t0 = time.time() - w


class _State:
    def __init__(self, model: Model, backend: str):
        self.model = model
        self.backend = backend
        self.program = compile_model(model, backend)
        self.traj: Optional[E.Trajectory] = None
        self.system_size = np.zeros(3, dtype=np.int32)
        self.seed = 1
        self.system_name = "kmc_model"
        self.pending: list = []  # touch-ups queued, run before the next call reaches the engine

    def t(self) -> E.Trajectory:
        if self.traj is None:
            raise E.KMCError(1, "system not allocated: call proclist.init first")
        if self.pending:
            sites, self.pending = self.pending, []
            self.traj.touchup_many(sites)
        return self.traj

    def touchup(self, site) -> None:
        """touchup_<layer>_<site> / touchup_cell: queued, so that kmos.run's
        _adjust_database (one call per site, kmos/run/__init__.py:1439-1457) becomes one
        launch; the queue runs, in call order, before any other call reaches the engine
        (a touch-up error surfaces there)."""
        if self.traj is None:
            raise E.KMCError(1, "system not allocated: call proclist.init first")
        nr = self.lattice2nr(site)
        if not 1 <= nr <= int(np.prod(self.system_size)) * self.model.spuck:
            raise E.KMCError(1, "site out of range")
        self.pending.append(nr)

    # lattice mapping (lattice.mpy:146-210)
    def lattice2nr(self, site) -> int:
        x, y, z, n = (int(v) for v in site)
        X, Y, Z = (int(v) for v in self.system_size)
        return self.model.spuck * ((x % X) + X * ((y % Y) + Y * (z % Z))) + n

    def nr2lattice(self, nr: int):
        sp = self.model.spuck
        X, Y = int(self.system_size[0]), int(self.system_size[1])
        c = (int(nr) - 1) // sp
        return np.array([c % X, (c // X) % Y, c // (X * Y), int(nr) - sp * c], dtype=np.int32)


def _base(S: _State) -> types.SimpleNamespace:
    ns = types.SimpleNamespace()
    ns.null_species = S.model.null_species()
    ns.get_null_species = lambda: S.model.null_species()
    ns.is_allocated = lambda: S.traj is not None
    ns.set_rate_const = lambda proc, rate: S.t().set_rate_const(int(proc), float(rate))
    ns.update_accum_rate = lambda: S.t().update_accum_rate()
    ns.update_integ_rate = lambda: S.t().update_integ_rate()
    ns.get_kmc_time = lambda: S.t().kmc_time
    ns.get_kmc_time_step = lambda: S.t().kmc_time_step
    ns.get_kmc_step = lambda: S.t().kmc_step

    def set_kmc_time(t):
        S.t().kmc_time = float(t)

    ns.set_kmc_time = set_kmc_time
    ns.get_procstat = lambda proc: int(S.t().procstat()[int(proc) - 1])
    if S.backend == "otf":
        ns.get_rate = lambda proc, site_nr=-1: S.t().get_rate(int(proc), int(site_nr))
    else:
        ns.get_rate = lambda proc: float(S.t().rates()[int(proc) - 1])
    ns.get_integ_rate = lambda proc: float(S.t().integ_rates()[int(proc) - 1])
    ns.get_accum_rate = lambda proc: float(S.t().accum_rates()[int(proc) - 1])
    ns.get_nrofsites = lambda proc: int(S.t().nr_of_sites()[int(proc) - 1])
    ns.get_avail_site = lambda proc, idx, sw: S.t().avail_site(int(proc), int(idx), int(sw))
    ns.get_volume = lambda: S.t().V
    ns.get_walltime = lambda: S.t().walltime
    ns.get_species = lambda nr: S.t().get_species(int(nr))
    ns.replace_species = lambda nr, old, new: S.t().replace_species(int(nr), int(old), int(new))
    ns.save_system = lambda: _save_system(S)
    ns.reload_system = lambda input_system_name: _reload_system(S, input_system_name)
    return ns


def _save_system(S: _State) -> None:
    """base.save_system (base.mpy:489-575): ``<system_name>.reload`` in the working
    directory, in the reference's layout."""
    S.t().save_reload(S.system_name.strip() + ".reload")


def _reload_system(S: _State, input_system_name) -> bool:
    """base.reload_system (base.mpy:363-486): returns whether ``<name>.reload`` existed
    and was loaded.  Like the reference it allocates the system; the system size comes
    from the file's ``#gb300 system_size`` line, else from ``lattice.system_size`` when
    that was set to a size of the file's volume."""
    import os
    name = str(input_system_name).strip()
    S.system_name = name
    path = name + ".reload"
    if not os.path.exists(path):
        return False
    if S.traj is not None:
        raise E.KMCError(1, "allocate_system: tried to allocate twice, deallocate first")
    nproc, volume, dims = E.reload_info(path)
    if nproc != len(S.model.processes):
        raise E.KMCError(1, "%s holds %d processes, the model has %d" % (path, nproc, len(S.model.processes)))
    if dims is None:
        dims = [int(v) for v in S.system_size]
        if min(dims) < 1 or int(np.prod(dims)) * S.model.spuck != volume:
            raise E.KMCError(1, "%s has no system size line: set lattice.system_size to a size with volume %d "
                                "first" % (path, volume))
    S.system_size[:] = dims
    layer = S.model.layer_ids()[S.model.default_layer]
    if S.backend == "otf":
        S.traj = _OtfTrajectory(S.program, dims, layer, S.seed)
        pars = _pars(S)
        for k, v in enumerate(pars.userpar[:int(S.program.words[23])], start=1):
            S.traj.b.set_user_parameter(k, float(v))
    else:
        S.traj = E.Trajectory(S.program, dims, layer=layer, seed=S.seed, rng=E.RNG_GFORTRAN)
    S.traj.load_reload(path)
    return True


def _lattice(S: _State) -> types.SimpleNamespace:
    m = S.model
    ns = types.SimpleNamespace()
    ns.system_size = S.system_size
    ns.spuck = m.spuck
    ns.model_dimension = m.dimension
    ns.nr_of_layers = len(m.layers)
    lid = m.layer_ids()
    for name, i in lid.items():
        setattr(ns, name.lower(), i)
    ns.default_layer = lid[m.default_layer]
    ns.substrate_layer = lid.get(m.substrate_layer, ns.default_layer)
    ns.unit_cell_size = np.array(m.cell, dtype=np.float64)
    ns.site_positions = np.array([s.pos for _l, s in m.site_list()], dtype=np.float64).reshape(-1, 3)
    for (lname, sname), n in m.site_ids().items():
        setattr(ns, ("%s_%s" % (lname, sname)).lower(), n)
    ns.calculate_lattice2nr = S.lattice2nr
    ns.calculate_nr2lattice = S.nr2lattice
    ns.get_species = lambda site: S.t().get_species(S.lattice2nr(site))
    ns.replace_species = lambda site, old, new: S.t().replace_species(S.lattice2nr(site), int(old), int(new))

    def deallocate_system():
        S.pending = []
        if S.traj is not None:
            S.traj.close()
            S.traj = None

    ns.deallocate_system = deallocate_system
    ns.save_system = lambda: _save_system(S)
    ns.reload_system = lambda input_system_name: _reload_system(S, input_system_name)
    return ns


def _proclist(S: _State) -> types.SimpleNamespace:
    m = S.model
    ns = types.SimpleNamespace()
    ns.nr_of_proc = len(m.processes)
    ns.nr_of_species = len(m.species) + (0 if len(m.layers) == 1 else 1)
    for name, i in m.species_ids().items():
        setattr(ns, name.lower(), i)
    ns.default_species = m.species_ids()[m.default_species]
    if len(m.layers) > 1:
        ns.null_species = m.null_species()
    for name, i in m.process_ids().items():
        setattr(ns, name.lower(), i)
    ns.seed_size = 12
    ns.seed = S.seed
    ns.representation_length = max([len(r) for r in m.representations.values()] + [1])
    if S.backend in ("lat_int", "otf"):
        ns.backend = S.backend

    def init(input_system_size, system_name="kmc_model", layer=None, seed_in=1, no_banner=True):
        """proclist.init (proclist_generic_subroutines.mpy:166-230)."""
        size = [int(v) for v in np.atleast_1d(input_system_size)]
        size = (size + [1, 1, 1])[:3]
        if S.traj is not None:
            raise E.KMCError(1, "allocate_system: tried to allocate twice, deallocate first")
        S.system_size[:] = size
        S.seed = int(seed_in)
        S.system_name = str(system_name)
        ns.seed = S.seed
        layer = ns_default_layer if layer is None else int(layer)
        if S.backend == "otf":
            S.traj = _OtfTrajectory(S.program, size, layer, S.seed)
            pars = _pars(S)
            for k, v in enumerate(pars.userpar[:int(S.program.words[23])], start=1):
                S.traj.b.set_user_parameter(k, float(v))
        else:
            S.traj = E.Trajectory(S.program, size, layer=layer, seed=S.seed, rng=E.RNG_GFORTRAN)

    ns_default_layer = m.layer_ids()[m.default_layer]
    ns.init = init
    ns.do_kmc_steps = lambda n: S.t().do_kmc_steps(int(n))
    ns.do_kmc_step = lambda: S.t().do_kmc_steps(1)
    ns.get_next_kmc_step = lambda: S.t().get_next_kmc_step()
    ns.run_proc_nr = lambda proc, site: S.t().run_proc_nr(int(proc), int(site))

    def get_occupation():
        """(species, spuck) site-resolved coverage per unit cell: one row per species
        of the model, the null species of multi-lattice models not counted
        (proclist_generic_subroutines.mpy:113-158 declares occupation(0:nspecies-1, 1:spuck))."""
        return S.t().occupation()

    ns.get_occupation = get_occupation
    if S.backend == "otf":
        # recalculate_rates_matrix (proclist_generic_subroutines.mpy:307-325) and the
        # proclist_pars routines kmos.run reaches through proclist
        ns.recalculate_rates_matrix = lambda: S.t().recalculate_rates_matrix()
        pars = _pars(S)
        for k, v in vars(pars).items():
            if not hasattr(ns, k):
                setattr(ns, k, v)
        ns.touchup_cell = lambda cell: S.touchup([cell[0], cell[1], cell[2], 1])
    elif S.backend == "lat_int":
        ns.touchup_cell = lambda cell: S.touchup([cell[0], cell[1], cell[2], 1])
    else:
        for (lname, sname), n in m.site_ids().items():
            setattr(ns, ("touchup_%s_%s" % (lname, sname)).lower(), lambda site: S.touchup(site))
    return ns


def _pars(S: _State) -> types.SimpleNamespace:
    """proclist_pars of an otf build (kmos/io/__init__.py:2657-2800): the user
    parameters (1-based, sorted by name) and their update / get routines, and the
    byst_<process> strings of nr variable names."""
    if getattr(S, "pars", None) is not None:
        return S.pars
    from . import otf
    ns = types.SimpleNamespace()
    S.pars = ns
    names = otf.user_parameters(S.model)
    mus = otf.chempot_names(S.model)
    values = np.zeros(max(len(names) + len(mus), 1))   # user parameters, then chempots
    for k, n in enumerate(names, start=1):
        setattr(ns, n.lower(), k)

    def update_user_parameter(param, val):
        if not 1 <= int(param) <= len(names):
            raise E.KMCError(1, "user parameter %s out of range" % param)
        values[int(param) - 1] = float(val)
        if S.traj is not None:
            S.traj.b.set_user_parameter(int(param), float(val))

    ns.update_user_parameter = update_user_parameter
    ns.get_user_parameter = lambda param: float(values[int(param) - 1])
    if mus:
        # update_chempot(index, val) and the mu_* index constants (io:2740-2790)
        for j, mu in enumerate(mus, start=1):
            setattr(ns, mu.lower(), j)

        def update_chempot(index, val):
            if not 1 <= int(index) <= len(mus):
                raise E.KMCError(1, "chemical potential %s out of range" % index)
            k = len(names) + int(index)
            values[k - 1] = float(val)
            if S.traj is not None:
                S.traj.b.set_user_parameter(k, float(val))

        ns.update_chempot = update_chempot
        ns.chempots = values[len(names):]
    ns.userpar = values
    pid = S.model.process_ids()
    for proc in S.model.processes:
        setattr(ns, "byst_%s" % proc.name.lower(), " ".join(otf.nr_var_names(proc)))

        def rate(nr_vars=(), _code=otf.compile_rate(S.model, proc)[1], _p=pid[proc.name]):
            """rate_<name>(nr_vars) (io:2920-2965): the otf rate for given bystander
            counts, from the current rate constant and user parameters (what
            kmos.run's Model_Rate_Constants_OTF prints, run:1848-1882)."""
            base = float(S.traj.rates()[_p - 1]) if S.traj is not None else 0.0
            return otf.evaluate(_code, base, values, [int(v) for v in np.atleast_1d(nr_vars)])

        setattr(ns, "rate_%s" % proc.name.lower(), rate)
    return ns


def configure(model, backend: str = "local_smart"):
    """Builds ``(base, lattice, proclist)`` for ``model`` (a :class:`Model`, a project
    file path, or a JSON dict of one) on ``backend``; also sets them as attributes of
    this module so ``from kmos_gb300.kmc_model import base, lattice, proclist`` works
    after the call."""
    if isinstance(model, str):
        model = load(model)
    elif isinstance(model, dict):
        model = from_dict(model)
    S = _State(model, backend)
    b, l, p = _base(S), _lattice(S), _proclist(S)
    g = globals()
    g["base"], g["lattice"], g["proclist"], g["_state"] = b, l, p, S
    if backend == "otf":
        g["proclist_pars"] = _pars(S)
    else:
        g.pop("proclist_pars", None)
    return b, l, p


def __getattr__(name):
    if name in ("base", "lattice", "proclist", "proclist_pars"):
        import importlib
        import os
        settings = importlib.import_module("kmc_settings")
        backend = getattr(settings, "backend", os.environ.get("KMOS_GB300_BACKEND", "local_smart"))
        if hasattr(settings, "model_json"):
            model = from_dict(settings.model_json)
        elif hasattr(settings, "xml"):
            from .model import load_xml
            model = load_xml(settings.xml)
        else:
            raise AttributeError("kmc_settings has neither model_json nor xml to configure %s from" % name)
        configure(model, backend)
        if name not in globals():
            raise AttributeError(name)   # proclist_pars exists for otf builds only
        return globals()[name]
    raise AttributeError(name)
