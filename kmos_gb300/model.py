"""Model description for the kMC step engine.

A kmos model is a *Project*: species, a lattice of layers and sites, parameters and
processes made of conditions and actions (kmos/types.py:62-1434 in mhoffman/kmos).
This module reads the two project file formats kmos writes — the ``.ini`` layout of
``Project.import_ini_file`` (kmos/types.py:623-913) and the ``.xml`` layout of
``Project.import_xml_file`` (kmos/types.py:915-1159) — into a small, self-contained
intermediate representation, :class:`Model`.  A live ``kmos.types.Project`` object can
be converted too (:func:`from_project`), so a kmos user can hand the project they
already have to the engine.

Only what the step loop and the ``kmc_model`` interface need is kept: names, numbering
rules, coordinates, rate expressions, TOF counts.  Colours, representations and other
GUI data are carried as opaque strings.
"""
from __future__ import annotations

import ast
import configparser
import io
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple


@dataclass(frozen=True)
class Coord:
    """A lattice coordinate relative to a unit cell: site ``name`` of ``layer``,
    shifted by ``offset`` unit cells (kmos/types.py:1778-1948)."""

    name: str
    offset: Tuple[int, int, int]
    layer: str

    def same_site_type(self, other: "Coord") -> bool:
        """kmos ``Coord.eq_mod_offset``: same layer and site, any offset."""
        return (self.layer, self.name) == (other.layer, other.name)

    def sort_key(self) -> str:
        """The string key kmos sorts actions by to find the executing coordinate
        (kmos/types.py:1922-1929).  It is a *string*, so offsets compare as text."""
        return "%s_%s_%s_%s_%s" % (self.layer, self.name, self.offset[0], self.offset[1], self.offset[2])


@dataclass(frozen=True)
class Condition:
    """A condition or an action: ``species`` at ``coord``.  ``species`` may hold
    ``"A or B"`` alternatives (lat_int only) or a ``^``/``$`` multi-lattice prefix."""

    species: str
    coord: Coord
    implicit: bool = False


@dataclass(frozen=True)
class Bystander:
    """A site whose species changes an otf process's rate but not whether it can run
    (kmos/types.py:2160-2200): each ``allowed_species`` found at ``coord`` counts one
    towards ``nr_<species>_<flag>``."""

    allowed_species: Tuple[str, ...]
    coord: Coord
    flag: str = ""


@dataclass
class Process:
    name: str
    rate_constant: str
    conditions: List[Condition] = field(default_factory=list)
    actions: List[Condition] = field(default_factory=list)
    enabled: bool = True
    tof_count: Optional[Dict[str, float]] = None
    bystanders: List[Bystander] = field(default_factory=list)
    otf_rate: Optional[str] = None   # otf backend: the rate at a site, from base_rate and bystanders

    def executing_coord(self) -> Coord:
        """kmos ``Process.executing_coord`` (kmos/types.py:2094-2097): the action
        coordinate with the smallest *string* sort key; the first one on ties."""
        best = None
        for action in self.actions:
            if best is None or action.coord.sort_key() < best.coord.sort_key():
                best = action
        return best.coord


@dataclass
class Site:
    name: str
    pos: Tuple[float, float, float]
    default_species: str
    tags: str = ""


@dataclass
class Layer:
    name: str
    sites: List[Site] = field(default_factory=list)


@dataclass
class Parameter:
    name: str
    value: str
    adjustable: bool = False
    min: float = 0.0
    max: float = 0.0
    scale: str = "linear"


@dataclass
class Model:
    """Intermediate representation of one kmos project."""

    name: str
    dimension: int
    species: List[str]                 # in file order
    default_species: str
    layers: List[Layer]
    default_layer: str
    substrate_layer: str
    cell: Tuple[Tuple[float, float, float], ...]
    parameters: List[Parameter]
    processes: List[Process]           # in file order: process number = index + 1
    meta: Dict[str, str] = field(default_factory=dict)
    representations: Dict[str, str] = field(default_factory=dict)

    # ---- numbering rules shared with the generated kmos modules ----------------
    def species_ids(self) -> Dict[str, int]:
        """Species are numbered 0.. by *sorted name* (proclist_constants.mpy:65)."""
        return {name: i for i, name in enumerate(sorted(self.species))}

    def null_species(self) -> int:
        """-1 for one layer; the species count for multi-lattice models
        (base.mpy:85 and proclist_constants.mpy:67-70)."""
        return -1 if len(self.layers) == 1 else len(self.species)

    def site_list(self) -> List[Tuple[str, Site]]:
        """(layer name, site) in the order kmos numbers them: layer by layer,
        1-based (``<layer>_<site>`` constants of lattice.f90)."""
        return [(layer.name, site) for layer in self.layers for site in layer.sites]

    def site_ids(self) -> Dict[Tuple[str, str], int]:
        return {(ln, s.name): i + 1 for i, (ln, s) in enumerate(self.site_list())}

    def layer_ids(self) -> Dict[str, int]:
        """Layers are numbered 0.. in file order (lattice.f90 layer constants)."""
        return {layer.name: i for i, layer in enumerate(self.layers)}

    @property
    def spuck(self) -> int:
        return len(self.site_list())

    def process_ids(self) -> Dict[str, int]:
        """Processes are numbered 1.. in file order (proclist_constants.mpy:77)."""
        return {p.name: i + 1 for i, p in enumerate(self.processes)}

    def site_default_species(self, site: Site) -> str:
        ds = site.default_species
        if ds in ("default_species", "", None):
            return self.default_species
        return ds

    def parameter_dict(self) -> Dict[str, Dict[str, str]]:
        return {p.name: {"value": p.value} for p in self.parameters}

    def tof_names(self) -> List[str]:
        names = set()
        for p in self.processes:
            if p.tof_count:
                names.update(p.tof_count.keys())
        return sorted(names)


# --------------------------------------------------------------------------------------
# .ini reader (layout of kmos/types.py:623-913)
# --------------------------------------------------------------------------------------
def _literal(text: str):
    return ast.literal_eval(text.strip())


def _parse_offset(text: str) -> Tuple[int, int, int]:
    value = _literal(text)
    if isinstance(value, int):
        value = (value,)
    value = tuple(int(v) for v in value)
    return (value + (0, 0, 0))[:3]


def _ini_coord(text: str, first_layer: str) -> Coord:
    parts = text.strip().split(".")
    if len(parts) == 3:
        name, offset, layer = parts
        return Coord(name.strip(), _parse_offset(offset), layer.strip())
    if len(parts) == 2:
        name, offset = parts
        return Coord(name.strip(), _parse_offset(offset), first_layer)
    return Coord(parts[0].strip(), (0, 0, 0), first_layer)


def _parse_tof_count(value) -> Optional[Dict[str, float]]:
    if value is None:
        return None
    if isinstance(value, dict):
        return dict(value)
    text = str(value).strip()
    if not text or text == "None":
        return {} if text == "" else None
    return dict(_literal(text))


def load_ini(path_or_text: str) -> Model:
    """Read a kmos ``.ini`` project.  Plain ini files are supported; the template
    pre-processing kmos applies before parsing (``#@`` Python blocks) is not."""
    if os.path.exists(path_or_text):
        with open(path_or_text) as fh:
            text = fh.read()
    else:
        text = path_or_text
    config = configparser.ConfigParser(interpolation=None)
    config.optionxform = str
    config.read_file(io.StringIO(text))
    sections = config.sections()
    first_layer = [s.split()[-1] for s in sections if s.startswith("Layer")]
    first_layer = first_layer[0] if first_layer else ""

    meta: Dict[str, str] = {}
    species: List[str] = []
    representations: Dict[str, str] = {}
    default_species = None
    layers: List[Layer] = []
    default_layer = None
    substrate_layer = None
    cell = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))
    parameters: List[Parameter] = []
    processes: List[Process] = []

    for section in sections:
        opts = config.options(section)
        get = lambda o, d=None: config.get(section, o) if o in opts else d  # noqa: E731
        if section == "Lattice":
            if "cell_size" in opts:
                vals = [float(v) for v in get("cell_size").split()]
                if len(vals) == 3:
                    cell = ((vals[0], 0.0, 0.0), (0.0, vals[1], 0.0), (0.0, 0.0, vals[2]))
                elif len(vals) == 9:
                    cell = tuple(tuple(vals[3 * i:3 * i + 3]) for i in range(3))
                else:
                    raise ValueError("cell_size %r not understood" % vals)
            if "default_layer" in opts:
                default_layer = get("default_layer")
            if "substrate_layer" in opts:
                substrate_layer = get("substrate_layer")
        elif section.startswith("Layer "):
            layer = Layer(section.split()[-1])
            layers.append(layer)
            if default_layer is None:
                default_layer = layer.name
            if substrate_layer is None:
                substrate_layer = layer.name
            for opt in opts:
                if not opt.startswith("site"):
                    continue
                name = opt.split()[-1].strip()
                fields = config.get(section, opt).split(";")
                pos = tuple(float(v) for v in _literal(fields[0]))
                ds = fields[1].strip() if len(fields) >= 2 else "default_species"
                tags = fields[2].strip() if len(fields) >= 3 else ""
                layer.sites.append(Site(name, pos, ds, tags))
        elif section == "Meta":
            for opt in opts:
                meta[opt] = config.get(section, opt)
        elif section.startswith("Parameter "):
            parameters.append(Parameter(
                name=section.split()[-1],
                value=get("value"),
                adjustable=config.getboolean(section, "adjustable") if "adjustable" in opts else False,
                min=float(get("min", 0.0)),
                max=float(get("max", 0.0)),
                scale=get("scale", "linear"),
            ))
        elif section.startswith("Process "):
            proc = Process(
                name=section.split()[-1],
                rate_constant=get("rate_constant"),
                enabled=config.getboolean(section, "enabled") if "enabled" in opts else True,
                tof_count=_parse_tof_count(get("tof_count")) if "tof_count" in opts else None,
            )
            for term in [t.strip() for t in get("actions").split("+")]:
                sp, co = term.split("@")
                proc.actions.append(Condition(sp.strip(), _ini_coord(co, first_layer)))
            for term in [t.strip() for t in get("conditions").split("+")]:
                sp, co = term.split("@")
                proc.conditions.append(Condition(sp.strip(), _ini_coord(co, first_layer)))
            otf = get("otf_rate")
            proc.otf_rate = None if otf is None or otf.strip() == "None" else otf
            if get("bystanders"):
                # allowed@coord|flag (kmos/types.py:855-890), allowed a Python list literal
                for term in [t.strip() for t in get("bystanders").split("+")]:
                    allowed, co = term.split("@")
                    co, flag = co.split("|")
                    proc.bystanders.append(Bystander(tuple(_literal(allowed)), _ini_coord(co, first_layer), flag.strip()))
            processes.append(proc)
        elif section == "SpeciesList":
            default_species = get("default_species", "")
        elif section.startswith("Species "):
            name = section.split()[-1]
            species.append(name)
            representations[name] = get("representation", "") or ""
    if default_species is None and species:
        default_species = species[0]
    return Model(
        name=meta.get("model_name", "kmc_model"),
        dimension=int(meta.get("model_dimension", 2)),
        species=species,
        default_species=default_species,
        layers=layers,
        default_layer=default_layer,
        substrate_layer=substrate_layer,
        cell=cell,
        parameters=parameters,
        processes=processes,
        meta=meta,
        representations=representations,
    )


# --------------------------------------------------------------------------------------
# .xml reader (layout of kmos/types.py:915-1159, project versions (0, 2) and (0, 3))
# --------------------------------------------------------------------------------------
def load_xml(path: str) -> Model:
    """Read a kmos ``.xml`` project file, or an XML string (kmc_settings.xml holds one)."""
    if path.lstrip().startswith("<"):
        root = ET.fromstring(path.strip())
    else:
        root = ET.parse(path).getroot()
    meta: Dict[str, str] = {}
    species: List[str] = []
    representations: Dict[str, str] = {}
    default_species = ""
    layers: List[Layer] = []
    default_layer = substrate_layer = None
    cell = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))
    parameters: List[Parameter] = []
    processes: List[Process] = []
    for child in root:
        if child.tag == "lattice":
            vals = [float(v) for v in child.attrib["cell_size"].split()]
            if len(vals) == 3:
                cell = ((vals[0], 0.0, 0.0), (0.0, vals[1], 0.0), (0.0, 0.0, vals[2]))
            else:
                cell = tuple(tuple(vals[3 * i:3 * i + 3]) for i in range(3))
            default_layer = child.attrib["default_layer"]
            substrate_layer = child.attrib.get("substrate_layer", default_layer)
            for elem in child:
                if elem.tag != "layer":
                    continue
                layer = Layer(elem.attrib["name"])
                for s in elem:
                    layer.sites.append(Site(
                        name=s.attrib["type"],
                        pos=tuple(float(v) for v in s.attrib["pos"].split()),
                        default_species=s.attrib.get("default_species", "default_species"),
                        tags=s.attrib.get("tags", ""),
                    ))
                layers.append(layer)
        elif child.tag == "meta":
            for k in ("author", "debug", "email", "model_dimension", "model_name"):
                if k in child.attrib:
                    meta[k] = child.attrib[k]
        elif child.tag == "parameter_list":
            for p in child:
                parameters.append(Parameter(
                    name=p.attrib["name"],
                    value=p.attrib["value"],
                    adjustable=p.attrib.get("adjustable", "False") == "True",
                    min=float(p.attrib.get("min", 0.0)),
                    max=float(p.attrib.get("max", 0.0)),
                    scale=p.attrib.get("scale", "linear"),
                ))
        elif child.tag == "process_list":
            for p in child:
                enabled = p.attrib.get("enabled", "True")
                proc = Process(
                    name=p.attrib["name"],
                    rate_constant=p.attrib["rate_constant"],
                    enabled=enabled.strip() not in ("False", "0"),
                    tof_count=_parse_tof_count(p.attrib.get("tof_count")),
                    otf_rate=p.attrib.get("otf_rate"),
                )
                for sub in p:
                    if sub.tag == "bystander":
                        proc.bystanders.append(Bystander(
                            tuple(sub.attrib["allowed_species"].split()),
                            Coord(sub.attrib["coord_name"], tuple(int(v) for v in sub.attrib["coord_offset"].split()),
                                  sub.attrib["coord_layer"]),
                            sub.attrib.get("flag", "")))
                        continue
                    if sub.tag not in ("action", "condition"):
                        continue
                    coord = Coord(
                        sub.attrib["coord_name"],
                        tuple(int(v) for v in sub.attrib["coord_offset"].split()),
                        sub.attrib["coord_layer"],
                    )
                    ca = Condition(sub.attrib["species"], coord, sub.attrib.get("implicit", "") == "True")
                    (proc.actions if sub.tag == "action" else proc.conditions).append(ca)
                processes.append(proc)
        elif child.tag == "species_list":
            default_species = child.attrib.get("default_species", "")
            for s in child:
                species.append(s.attrib["name"])
                representations[s.attrib["name"]] = s.attrib.get("representation", "")
    return Model(
        name=meta.get("model_name", "kmc_model"),
        dimension=int(meta.get("model_dimension", 2)),
        species=species,
        default_species=default_species,
        layers=layers,
        default_layer=default_layer,
        substrate_layer=substrate_layer,
        cell=cell,
        parameters=parameters,
        processes=processes,
        meta=meta,
        representations=representations,
    )


def load(path: str) -> Model:
    """Read a kmos project file by extension (``.ini`` or ``.xml``; ``.json``: this
    package's JSON form)."""
    if path.endswith(".xml"):
        return load_xml(path)
    if path.endswith(".json"):
        return load_json(path)
    return load_ini(path)


def from_project(project) -> Model:
    """Convert a live ``kmos.types.Project`` (duck-typed) into a :class:`Model`."""

    def coord(c):
        return Coord(c.name, tuple(int(v) for v in list(c.offset)[:3]), c.layer)

    layers = [Layer(l.name, [Site(s.name, tuple(getattr(s, "pos", (0, 0, 0))),
                                  getattr(s, "default_species", "default_species"),
                                  getattr(s, "tags", "")) for s in l.sites])
              for l in project.layer_list]
    procs = []
    for p in project.process_list:
        procs.append(Process(
            name=p.name,
            rate_constant=p.rate_constant,
            conditions=[Condition(c.species, coord(c.coord), bool(getattr(c, "implicit", False)))
                        for c in p.condition_list],
            actions=[Condition(a.species, coord(a.coord), bool(getattr(a, "implicit", False)))
                     for a in p.action_list],
            enabled=bool(getattr(p, "enabled", True)),
            tof_count=_parse_tof_count(getattr(p, "tof_count", None)),
            bystanders=[Bystander(tuple(b.allowed_species), coord(b.coord), b.flag or "")
                        for b in getattr(p, "bystander_list", [])],
            otf_rate=getattr(p, "otf_rate", None),
        ))
    meta = {}
    for k in ("author", "email", "model_name", "model_dimension", "debug"):
        if hasattr(project.meta, k):
            meta[k] = str(getattr(project.meta, k))
    cell = tuple(tuple(float(v) for v in row) for row in project.layer_list.cell)
    return Model(
        name=meta.get("model_name", "kmc_model"),
        dimension=int(meta.get("model_dimension", 2)),
        species=[s.name for s in project.species_list],
        default_species=project.species_list.default_species,
        layers=layers,
        default_layer=project.layer_list.default_layer,
        substrate_layer=getattr(project.layer_list, "substrate_layer", project.layer_list.default_layer),
        cell=cell,
        parameters=[Parameter(p.name, str(p.value), bool(getattr(p, "adjustable", False)),
                              float(getattr(p, "min", 0.0) or 0.0), float(getattr(p, "max", 0.0) or 0.0),
                              getattr(p, "scale", "linear")) for p in project.parameter_list],
        processes=procs,
        meta=meta,
        representations={s.name: getattr(s, "representation", "") for s in project.species_list},
    )


# --------------------------------------------------------------------------------------
# JSON form (used for test fixtures and the serving protocol)
# --------------------------------------------------------------------------------------
def to_dict(model: Model) -> dict:
    def cd(c: Condition):
        d = {"species": c.species, "coord": [c.coord.name, list(c.coord.offset), c.coord.layer]}
        if c.implicit:
            d["implicit"] = True
        return d

    def proc(p: Process):
        d = {"name": p.name, "rate_constant": p.rate_constant, "enabled": p.enabled,
             "tof_count": p.tof_count, "conditions": [cd(c) for c in p.conditions],
             "actions": [cd(a) for a in p.actions]}
        if p.bystanders:
            d["bystanders"] = [{"allowed_species": list(b.allowed_species), "flag": b.flag,
                                "coord": [b.coord.name, list(b.coord.offset), b.coord.layer]} for b in p.bystanders]
        if p.otf_rate is not None:
            d["otf_rate"] = p.otf_rate
        return d

    return {
        "name": model.name,
        "dimension": model.dimension,
        "species": list(model.species),
        "default_species": model.default_species,
        "layers": [{"name": l.name, "sites": [[s.name, list(s.pos), s.default_species, s.tags] for s in l.sites]}
                   for l in model.layers],
        "default_layer": model.default_layer,
        "substrate_layer": model.substrate_layer,
        "cell": [list(r) for r in model.cell],
        "parameters": [[p.name, p.value, p.adjustable, p.min, p.max, p.scale] for p in model.parameters],
        "processes": [proc(p) for p in model.processes],
        "meta": dict(model.meta),
        "representations": dict(model.representations),
    }


def from_dict(d: dict) -> Model:
    def co(x):
        n, off, lay = x["coord"]
        return Coord(n, tuple(int(v) for v in off), lay)

    def cd(x):
        return Condition(x["species"], co(x), bool(x.get("implicit", False)))

    return Model(
        name=d["name"],
        dimension=int(d["dimension"]),
        species=list(d["species"]),
        default_species=d["default_species"],
        layers=[Layer(l["name"], [Site(s[0], tuple(s[1]), s[2], s[3]) for s in l["sites"]]) for l in d["layers"]],
        default_layer=d["default_layer"],
        substrate_layer=d["substrate_layer"],
        cell=tuple(tuple(r) for r in d["cell"]),
        parameters=[Parameter(*p) for p in d["parameters"]],
        processes=[Process(p["name"], p["rate_constant"], [cd(c) for c in p["conditions"]],
                           [cd(a) for a in p["actions"]], p.get("enabled", True), p.get("tof_count"),
                           [Bystander(tuple(b["allowed_species"]), co(b), b.get("flag", ""))
                            for b in p.get("bystanders", [])], p.get("otf_rate"))
                   for p in d["processes"]],
        meta=dict(d.get("meta", {})),
        representations=dict(d.get("representations", {})),
    )


def save_json(model: Model, path: str):
    import json
    with open(path, "w") as fh:
        json.dump(to_dict(model), fh, indent=1)


def load_json(path: str) -> Model:
    import json
    with open(path) as fh:
        return from_dict(json.load(fh))
