import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


def fixture_model(name):
    from kmos_gb300 import model as M
    return M.load_json(os.path.join(GOLDEN, "models", name + ".json"))


def trimer_model():
    """A square-lattice model with three-site adsorption (A3 in x and in y), desorption
    and a hop: its local_smart adds carry two conditions, and its lat_int groups have
    three coordinates, edit forms the fixture models do not reach."""
    from kmos_gb300 import configs
    from kmos_gb300.model import Process
    c = configs._c
    procs = [Process("A_desorption", "1", [c("A", "a")], [c("empty", "a")])]
    for i, d in enumerate([(1, 0, 0), (0, 1, 0)]):
        d2 = (2 * d[0], 2 * d[1], 0)
        procs.append(Process("A3_adsorption%d" % i, "1", [c("empty", "a"), c("empty", "a", d), c("empty", "a", d2)],
                             [c("A", "a"), c("A", "a", d), c("A", "a", d2)]))
    procs.append(Process("A_hop", "1", [c("A", "a"), c("empty", "a", (1, 0, 0))],
                         [c("empty", "a"), c("A", "a", (1, 0, 0))]))
    return configs._square_model("trimer", ["empty", "A"], procs)


def many_species_model(nspecies=16):
    """A square-lattice model with ``nspecies`` adsorbates, each with adsorption,
    desorption and hops in four directions (6 * nspecies processes): 16 species give 96
    processes (four per lane of the step kernel), 30 give 180 (eight per lane), and
    processes past the 64th, whose list tops the kernel does not load ahead."""
    from kmos_gb300 import configs
    from kmos_gb300.model import Process
    c = configs._c
    names = ["A%02d" % i for i in range(nspecies)]
    procs = []
    for sp in names:
        procs.append(Process(sp + "_adsorption", "1", [c("empty", "a")], [c(sp, "a")]))
        procs.append(Process(sp + "_desorption", "1", [c(sp, "a")], [c("empty", "a")]))
        for i, d in enumerate(configs.DIRS, start=1):
            procs.append(Process("%s_hop%d" % (sp, i), "1", [c(sp, "a"), c("empty", "a", d)],
                                 [c("empty", "a"), c(sp, "a", d)]))
    return configs._square_model("many_species", ["empty"] + names, procs)


def rows_model(k=8):
    """Adsorption, desorption, and desorption of a whole row of ``k`` adsorbates at once:
    the row event clears k sites, so one process (the row process anchored at each of
    the 2k-1 cells around them, and the single desorption at each of the k sites) gets
    many dels in one step -- more than the kernel loads list tops for ahead and more
    writes than its replay log holds."""
    from kmos_gb300 import configs
    from kmos_gb300.model import Process
    c = configs._c
    procs = [Process("A_adsorption", "1", [c("empty", "a")], [c("A", "a")]),
             Process("A_desorption", "1", [c("A", "a")], [c("empty", "a")]),
             Process("A_row_desorption", "1", [c("A", "a", (i, 0, 0)) for i in range(k)],
                     [c("empty", "a", (i, 0, 0)) for i in range(k)])]
    return configs._square_model("rows", ["empty", "A"], procs)
