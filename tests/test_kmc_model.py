"""The f2py-compatible drop-in namespaces (no GPU needed: nothing is allocated before
proclist.init)."""
import importlib
import os
import sys

import pytest

from conftest import GOLDEN
from kmos_gb300 import export, kmc_model, model as M

XML = """<?xml version="1.0" ?>
<kmc version="(0, 2)">
  <meta author="x" debug="0" email="x" model_dimension="2" model_name="mini"/>
  <species_list default_species="empty">
    <species name="CO" representation=""/>
    <species name="empty" representation=""/>
  </species_list>
  <parameter_list><parameter name="k" value="100"/></parameter_list>
  <lattice cell_size="1.0 1.0 1.0" default_layer="sq">
    <layer name="sq"><site default_species="default_species" type="hollow" pos="0 0 0"/></layer>
  </lattice>
  <process_list>
    <process enabled="True" name="CO_ads" rate_constant="k">
      <condition coord_layer="sq" coord_name="hollow" coord_offset="0 0 0" species="empty"/>
      <action coord_layer="sq" coord_name="hollow" coord_offset="0 0 0" species="CO"/>
    </process>
    <process enabled="True" name="CO_des" rate_constant="k">
      <condition coord_layer="sq" coord_name="hollow" coord_offset="0 0 0" species="CO"/>
      <action coord_layer="sq" coord_name="hollow" coord_offset="0 0 0" species="empty"/>
    </process>
  </process_list>
</kmc>"""


def test_names_follow_f2py_conventions():
    b, l, p = kmc_model.configure(M.load_json(os.path.join(GOLDEN, "models", "default_xml.json")))
    assert p.nr_of_proc == 36
    assert p.co_adsorption_bridge == 1  # process constants, file order, lower case
    assert (p.co, p.empty, p.oxygen) == (0, 1, 2)  # species by sorted name
    assert (l.ruo2_bridge, l.ruo2_cus, l.spuck) == (1, 2, 2)
    assert hasattr(p, "touchup_ruo2_bridge") and hasattr(p, "touchup_ruo2_cus")
    assert b.null_species == -1 and not b.is_allocated()
    with pytest.raises(Exception):
        b.get_kmc_time()


def test_lazy_configuration_from_a_kmos_export_directory(tmp_path):
    (tmp_path / "kmc_settings.py").write_text('backend = "lat_int"\nxml = """%s"""\n' % XML)
    sys.path.insert(0, str(tmp_path))
    sys.modules.pop("kmc_settings", None)
    try:
        for name in ("base", "lattice", "proclist", "_state"):
            kmc_model.__dict__.pop(name, None)
        p = kmc_model.proclist
        assert p.backend == "lat_int" and p.co_ads == 1 and hasattr(p, "touchup_cell")
    finally:
        sys.path.remove(str(tmp_path))
        sys.modules.pop("kmc_settings", None)


def test_export_writes_an_importable_model_directory(tmp_path):
    (tmp_path / "mini.xml").write_text(XML)
    out = tmp_path / "out"
    export.export(str(tmp_path / "mini.xml"), str(out), "local_smart")
    sys.path.insert(0, str(out))
    for mod in ("kmc_settings", "kmc_model"):
        sys.modules.pop(mod, None)
    try:
        settings = importlib.import_module("kmc_settings")
        assert settings.rate_constants["CO_ads"][0] == "k"
        assert settings.parameters["k"]["value"] == "100"
        drop_in = importlib.import_module("kmc_model")
        assert drop_in.proclist.co_des == 2 and drop_in.lattice.sq_hollow == 1
    finally:
        sys.path.remove(str(out))
        for mod in ("kmc_settings", "kmc_model"):
            sys.modules.pop(mod, None)


def test_every_attribute_kmos_run_reads():
    """The base / lattice / proclist attributes kmos.run and the kmos CLI read
    (tests/golden/kmc_model_attrs.json, collected from their source by
    tests/golden/make_kmc_model_attrs.py) are all there, for single- and multi-lattice
    models under both backends -- except names from docstring examples (lattice_bridge,
    site, co), the touchup_ prefix of an eval, the otf backend's rate-matrix calls, and
    the lat_int-only backend / touchup_cell under local_smart (as in the f2py module)."""
    import json
    from conftest import GOLDEN, fixture_model
    want = json.load(open(os.path.join(GOLDEN, "kmc_model_attrs.json")))
    examples = {"lattice_bridge", "site", "co", "touchup_"}
    otf = {"recalculate_rates_matrix", "update_chempot", "update_user_parameter"}
    for name in ("CO_oxidation_Ruo2", "pdopd_xml"):
        for backend in ("local_smart", "lat_int"):
            base, lattice, proclist = kmc_model.configure(fixture_model(name), backend)
            objs = {"base": base, "lattice": lattice, "proclist": proclist}
            for mod, obj in objs.items():
                skip = examples | otf | ({"backend", "touchup_cell"} if backend == "local_smart" else set())
                missing = [a for a in want[mod] if a not in skip and not hasattr(obj, a)]
                assert not missing, (name, backend, mod, missing)
