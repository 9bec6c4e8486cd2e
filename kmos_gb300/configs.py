"""The benchmark workloads as kmos models plus per-trajectory parameters.

Each builder returns a :class:`Workload`: one compiled model, and for every trajectory
its lattice size, rate constants, Philox seed and trajectory id.  Parameter draws use
numpy's PCG64 seeded with ``1000 + config number``; all lattices start empty.

  1  20x20 square lattice, one site, CO adsorption/desorption at k=100 (local_smart).
  2  64x64 square lattice, {empty, CO, O}: CO adsorption (y), O2 dissociative
     adsorption on NN empty pairs in 4 directions ((1-y)/4 each), CO+O reaction on NN
     pairs in 4 directions (1e6); y ~ U[0.45, 0.60] per trajectory (local_smart).
  3  lat_int: uneven square lattices (side in {16,32,64,128,256}), {empty, CO}: CO
     adsorption 1e3; 16 desorption processes, one per configuration of the 4 nearest
     neighbours, 1e13*exp(-(1.3 + 0.1*n_CO)/kT); 4 hops 1e13*exp(-0.6/kT);
     T ~ U[300, 600] K; k_B = 8.617333262e-5 eV/K.
  4  two-site rectangular cell (bridge, cus; 6.39 x 3.116 A), 20x20 cells, {empty, CO, O}:
     CO adsorption/desorption per site type, O2 dissociative adsorption and associative
     desorption on the NN pairs, CO and O hops over all NN pairs, CO+O reaction on all
     directed NN pairs: 44 processes.  Arrhenius rates 1e13*exp(-Ea/kT) with
     Ea ~ U[0.5, 1.6] eV per process and trajectory, T ~ U[450, 650] K; adsorption
     1e8 * p with pCO log-uniform in [0.1, 10] bar and pO2 = 1 bar (local_smart).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .model import Condition, Coord, Layer, Model, Parameter, Process, Site
from .program import Program, compile_model

K_B_EV = 8.617333262e-5  # eV/K


@dataclass
class Workload:
    name: str
    model: Model
    backend: str
    program: Program
    sizes: List[Tuple[int, int, int]]
    rates: List[List[float]]
    seeds: List[int]
    trajs: List[int]
    steps: int
    occupation_bytes: int = 1  # int8 occupation in HBM
    notes: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.sizes)


def _c(species: str, name: str, off=(0, 0, 0), layer: str = "default") -> Condition:
    return Condition(species, Coord(name, tuple(off), layer))


def _square_model(name: str, species: Sequence[str], processes: List[Process], sites=("a",), cell=(1.0, 1.0, 1.0)) -> Model:
    layer = Layer("default", [Site(s, (0.5 * i, 0.0, 0.0), "default_species") for i, s in enumerate(sites)])
    return Model(
        name=name, dimension=2, species=list(species), default_species="empty", layers=[layer],
        default_layer="default", substrate_layer="default",
        cell=((cell[0], 0.0, 0.0), (0.0, cell[1], 0.0), (0.0, 0.0, cell[2])), parameters=[],
        processes=processes, meta={"model_name": name, "model_dimension": "2"},
    )


DIRS = [(1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, -1, 0)]


def model_config1() -> Model:
    procs = [
        Process("CO_adsorption", "100", [_c("empty", "hollow")], [_c("CO", "hollow")]),
        Process("CO_desorption", "100", [_c("CO", "hollow")], [_c("empty", "hollow")]),
    ]
    return _square_model("mini_101", ["empty", "CO"], procs, sites=("hollow",))


def model_config2() -> Model:
    procs = [Process("CO_adsorption", "y", [_c("empty", "a")], [_c("CO", "a")])]
    for i, d in enumerate(DIRS, start=1):
        procs.append(Process("O2_adsorption%d" % i, "(1-y)/4", [_c("empty", "a"), _c("empty", "a", d)],
                             [_c("O", "a"), _c("O", "a", d)]))
    for i, d in enumerate(DIRS, start=1):
        procs.append(Process("CO_oxidation%d" % i, "1e6", [_c("CO", "a"), _c("O", "a", d)],
                             [_c("empty", "a"), _c("empty", "a", d)], tof_count={"CO_oxidation": 1}))
    return _square_model("zgb_64", ["empty", "CO", "O"], procs)


def model_config3() -> Model:
    procs = [Process("CO_adsorption", "1e3", [_c("empty", "a")], [_c("CO", "a")])]
    nn = [(-1, 0, 0), (0, -1, 0), (0, 1, 0), (1, 0, 0)]
    for mask in range(16):
        conds = []
        nco = 0
        for b, d in enumerate(nn):
            occ = (mask >> (3 - b)) & 1
            nco += occ
            conds.append(_c("CO" if occ else "empty", "a", d))
        conds.append(_c("CO", "a"))
        procs.append(Process("CO_desorption_%02d" % mask, "1e13*exp(-(1.3+0.1*%d)/kT)" % nco, conds,
                             [_c("empty", "a")], tof_count={"CO_desorption": 1}))
    for i, d in enumerate(DIRS, start=1):
        procs.append(Process("CO_hop%d" % i, "1e13*exp(-0.6/kT)", [_c("CO", "a"), _c("empty", "a", d)],
                             [_c("empty", "a"), _c("CO", "a", d)]))
    return _square_model("pairwise_lat_int", ["empty", "CO"], procs)


def _config4_pairs():
    """Directed nearest-neighbour pairs of the bridge/cus cell: (site, other site, offset)."""
    return [
        ("bridge", "bridge", (0, 1, 0)), ("bridge", "bridge", (0, -1, 0)),
        ("bridge", "cus", (0, 0, 0)), ("bridge", "cus", (-1, 0, 0)),
        ("cus", "cus", (0, 1, 0)), ("cus", "cus", (0, -1, 0)),
        ("cus", "bridge", (1, 0, 0)), ("cus", "bridge", (0, 0, 0)),
    ]


def model_config4() -> Model:
    procs: List[Process] = []
    kinds: List[str] = []
    for s in ("bridge", "cus"):
        procs.append(Process("CO_adsorption_%s" % s, "pCO*1e8", [_c("empty", s)], [_c("CO", s)]))
        kinds.append("ads")
    for s in ("bridge", "cus"):
        procs.append(Process("CO_desorption_%s" % s, "1e13*exp(-Ea/kT)", [_c("CO", s)], [_c("empty", s)]))
        kinds.append("arr")
    half = [("bridge", "cus", (0, 0, 0)), ("bridge", "bridge", (0, 1, 0)),
            ("cus", "bridge", (1, 0, 0)), ("cus", "cus", (0, 1, 0))]
    for a, b, d in half:
        procs.append(Process("O2_adsorption_%s_%s_%d%d" % (a, b, d[0], d[1]), "pO2*1e8",
                             [_c("empty", a), _c("empty", b, d)], [_c("O", a), _c("O", b, d)]))
        kinds.append("ads")
    for a, b, d in half:
        procs.append(Process("O2_desorption_%s_%s_%d%d" % (a, b, d[0], d[1]), "1e13*exp(-Ea/kT)",
                             [_c("O", a), _c("O", b, d)], [_c("empty", a), _c("empty", b, d)]))
        kinds.append("arr")
    for sp in ("CO", "O"):
        for a, b, d in _config4_pairs():
            procs.append(Process("%sdiff_%s_%s_%d%d" % (sp, a, b, d[0], d[1]), "1e13*exp(-Ea/kT)",
                                 [_c(sp, a), _c("empty", b, d)], [_c("empty", a), _c(sp, b, d)]))
            kinds.append("arr")
    for first, second in (("O", "CO"), ("CO", "O")):
        for a, b, d in _config4_pairs():
            procs.append(Process("React_%s_%s_%s_%d%d" % (first, a, b, d[0], d[1]), "1e13*exp(-Ea/kT)",
                                 [_c(first, a), _c(second, b, d)], [_c("empty", a), _c("empty", b, d)],
                                 tof_count={"CO_oxidation": 1}))
            kinds.append("arr")
    m = _square_model("ruo2_44", ["empty", "CO", "O"], procs, sites=("bridge", "cus"), cell=(6.39, 3.116, 20.0))
    m.meta["rate_kinds"] = ",".join(kinds)
    return m


def build(config: int, n: Optional[int] = None, steps: Optional[int] = None, sides: Optional[Sequence[int]] = None) -> Workload:
    """Workload of benchmark configuration ``config`` (1-4).  ``n`` and ``steps``
    override the trajectory count and the steps per trajectory (parity tests use
    small values); ``sides`` overrides config 3's side choices."""
    rng = np.random.Generator(np.random.PCG64(1000 + config))
    if config == 1:
        m = model_config1()
        n = 1 if n is None else n
        sizes = [(20, 20, 1)] * n
        rates = [[100.0, 100.0]] * n
        wl = Workload("config1_mini101_20x20", m, "local_smart", compile_model(m, "local_smart"), sizes, rates,
                      [0] * n, list(range(n)), int(1e6) if steps is None else steps)
    elif config == 2:
        m = model_config2()
        n = 4096 if n is None else n
        y = rng.uniform(0.45, 0.60, size=n)
        rates = [[float(v)] + [float((1.0 - v) / 4.0)] * 4 + [1e6] * 4 for v in y]
        wl = Workload("config2_zgb_64x64", m, "local_smart", compile_model(m, "local_smart"), [(64, 64, 1)] * n,
                      rates, [2] * n, list(range(n)), int(1e7) if steps is None else steps, notes={"y": y})
    elif config == 3:
        m = model_config3()
        n = 2048 if n is None else n
        choices = [16, 32, 64, 128, 256] if sides is None else list(sides)
        side = rng.choice(choices, size=n)
        T = rng.uniform(300.0, 600.0, size=n)
        rates = []
        for t in T:
            kT = K_B_EV * t
            r = [1e3]
            for mask in range(16):
                nco = bin(mask).count("1")
                r.append(1e13 * np.exp(-(1.3 + 0.1 * nco) / kT))
            r += [1e13 * np.exp(-0.6 / kT)] * 4
            rates.append([float(x) for x in r])
        wl = Workload("config3_lat_int_uneven", m, "lat_int", compile_model(m, "lat_int"),
                      [(int(s), int(s), 1) for s in side], rates, [3] * n, list(range(n)),
                      int(1e6) if steps is None else steps, notes={"side": side, "T": T})
    elif config == 4:
        m = model_config4()
        kinds = m.meta["rate_kinds"].split(",")
        n = 8192 if n is None else n
        T = rng.uniform(450.0, 650.0, size=n)
        pco = 10.0 ** rng.uniform(-1.0, 1.0, size=n)
        Ea = rng.uniform(0.5, 1.6, size=(n, len(kinds)))
        rates = []
        for i in range(n):
            kT = K_B_EV * T[i]
            r = []
            for j, (p, kind) in enumerate(zip(m.processes, kinds)):
                if kind == "ads":
                    r.append((pco[i] if p.name.startswith("CO") else 1.0) * 1e8)
                else:
                    r.append(1e13 * np.exp(-Ea[i, j] / kT))
            rates.append([float(x) for x in r])
        wl = Workload("config4_ruo2_2site_20x20", m, "local_smart", compile_model(m, "local_smart"),
                      [(20, 20, 1)] * n, rates, [4] * n, list(range(n)), int(1e7) if steps is None else steps,
                      notes={"T": T, "pCO": pco})
    else:
        raise ValueError("config must be 1..4")
    return wl


def serving_requests(rate: float = 500.0, duration: float = 60.0, seed: int = 5, steps_scale: float = 1.0,
                     side_range=(10, 200), steps_range=(1e4, 1e7)):
    """Configuration 5: a Poisson request stream mixing configurations 1-3.

    Arrivals at ``rate`` per second for ``duration`` seconds; model uniform in {1, 2, 3};
    side uniform in ``side_range``; kMC steps log-uniform in ``steps_range`` times
    ``steps_scale``; per-request parameters drawn as in the batch configurations.
    Returns (requests, {model key: program})."""
    from .serving import Request
    rng = np.random.Generator(np.random.PCG64(1000 + 5 + seed))
    progs = {"c1": build(1, n=1, steps=0).program, "c2": build(2, n=1, steps=0).program,
             "c3": build(3, n=1, steps=0).program}
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        kind = int(rng.integers(1, 4))
        side = int(rng.integers(side_range[0], side_range[1] + 1))
        n = int(np.exp(rng.uniform(np.log(steps_range[0]), np.log(steps_range[1]))) * steps_scale)
        if kind == 1:
            rates = [100.0, 100.0]
        elif kind == 2:
            y = rng.uniform(0.45, 0.60)
            rates = [y] + [(1.0 - y) / 4.0] * 4 + [1e6] * 4
        else:
            kT = K_B_EV * rng.uniform(300.0, 600.0)
            rates = [1e3] + [1e13 * np.exp(-(1.3 + 0.1 * bin(m).count("1")) / kT) for m in range(16)] + \
                    [1e13 * np.exp(-0.6 / kT)] * 4
        reqs.append(Request(model="c%d" % kind, size=(side, side, 1), rates=[float(x) for x in rates],
                            steps=max(1, n), seed=5, traj_id=len(reqs), rid=len(reqs), arrival=t))
    return reqs, progs
