"""The XML configuration reader against the reference's own reader.

tests/golden/configs.json holds every field CConfiguration<T>
(src/CConfiguration.cpp:28-172) returned for each tests/golden/configs/*.xml,
in double and float (generated by tests/golden/make_golden.py).  The reader
must return the same fields, and reader + lbm_derive_lattice the same lattice
parameters the reference's solver constructor derives (params.json)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc

CONFIGS = json.load(open(os.path.join(GOLDEN, "configs.json")))
PARAMS = json.load(open(os.path.join(GOLDEN, "params.json")))
CFG_DIR = os.path.join(GOLDEN, "configs")


def _same(got, want, tag):
    """Reals compare in the reference's precision: exactly in double, and
    after rounding our double to float for the float reader."""
    if isinstance(want, list):
        return all(_same(g, w, tag) for g, w in zip(got, want)) and len(got) == len(want)
    if isinstance(want, float):
        return (np.float32(got) == np.float32(want)) if tag == "f32" else got == want
    return got == want


@pytest.mark.parametrize("name", sorted(CONFIGS))
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_reader_matches_reference_reader(lib, name, tag):
    from cavityflow_cuda_gb300 import read_configuration

    want = CONFIGS[name][tag]
    assert not want.get("error"), "every fixture configuration passes the reference's checks"
    got = read_configuration(os.path.join(CFG_DIR, name + ".xml"))
    assert set(got) == set(want)
    bad = {k: (got[k], want[k]) for k in want if not _same(got[k], want[k], tag)}
    assert not bad, bad


@pytest.mark.parametrize("name", sorted(PARAMS))
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_configuration_lattice_matches_reference(lib, name, tag):
    from cavityflow_cuda_gb300 import LbmError, configuration_lattice

    want = PARAMS[name][tag]
    path = os.path.join(CFG_DIR, name + ".xml")
    if want.get("error"):
        with pytest.raises(LbmError) as ei:
            configuration_lattice(path, tag)
        assert ei.value.status == 6
        return
    got = configuration_lattice(path, tag)
    assert got["tau"] == want["tau"] and got["inv_tau"] == want["tau_inv"]
    assert got["velocity"] == (want["ux"], want["uy"], want["uz"])
    assert got["acceleration"] == (want["gx"], want["gy"], want["gz"])
    assert got["viscosity"] == want["nu"] and got["timestep"] == want["timestep"]


def _variant(tmp_path, old, new, name="c.xml"):
    text = open(os.path.join(CFG_DIR, "cavity64_re100.xml")).read()
    assert old in text
    p = tmp_path / name
    p.write_text(text.replace(old, new, 1))
    return str(p)


@pytest.mark.parametrize("old,new", [
    ("<timestep>1</timestep>", "<timestep>0</timestep>"),
    ("<max-velocity>0.1</max-velocity>", "<max-velocity>-0.1</max-velocity>"),
    ("<domain-size><x>64</x>", "<domain-size><x>0</x>"),
    ("<domian-length><x>64</x>", "<domian-length><x>65</x>"),             # cells not cubes
    ("<cpu-subdomain-ratio>0.0</cpu-subdomain-ratio>", "<cpu-subdomain-ratio>1.5</cpu-subdomain-ratio>"),
    ("<rate>100</rate>", "<rate>0</rate>"),
    ("<alpha-grid-configuration><x>32</x><y>8</y>", "<alpha-grid-configuration><x>256</x><y>8</y>"),  # 2048
    ("<beta-block-configuration><x>32</x>", "<beta-block-configuration><x>0</x>"),
])
def test_reader_rejects_what_the_reference_asserts(lib, tmp_path, old, new):
    """Each case breaks one assert of src/CConfiguration.cpp:174-197."""
    from cavityflow_cuda_gb300 import LbmError, read_configuration

    with pytest.raises(LbmError) as ei:
        read_configuration(_variant(tmp_path, old, new))
    assert ei.value.status == 6


def test_reader_reports_missing_elements_and_files(lib, tmp_path):
    from cavityflow_cuda_gb300 import LbmError, read_configuration

    with pytest.raises(LbmError) as ei:
        read_configuration(_variant(tmp_path, "<loops>1000</loops>", ""))
    assert ei.value.status == 6 and "loops" in str(ei.value)
    with pytest.raises(LbmError) as ei:
        read_configuration(str(tmp_path / "absent.xml"))
    assert ei.value.status == 7
    p = tmp_path / "broken.xml"
    p.write_text("<lbm-configuration><physics><velocity><x>1</x></velocity>")
    with pytest.raises(LbmError) as ei:
        read_configuration(str(p))
    assert ei.value.status in (6, 7)


@pytest.mark.parametrize("text", [
    "<lbm-configuration></lbm-configuration",          # closing tag cut off at the end of the file
    "<lbm-configuration><grid></grid",
    "<lbm-configuration><grid/><x",                    # unterminated start tag
    "<a>" * 100 + "</a>" * 100,                       # nested deeper than the reader follows
    "",
    "<",
])
def test_reader_rejects_malformed_xml(lib, tmp_path, text):
    """Malformed documents are configuration errors (LBM_ERR_CONFIG), never a
    read past the end of the text or an unbounded recursion."""
    from cavityflow_cuda_gb300 import LbmError, read_configuration

    p = tmp_path / "malformed.xml"
    p.write_text(text)
    with pytest.raises(LbmError) as ei:
        read_configuration(str(p))
    assert ei.value.status == 6, text[:40]


def test_reader_ignores_subdomain_num_as_the_serial_reference(lib, tmp_path):
    from cavityflow_cuda_gb300 import read_configuration

    path = _variant(tmp_path, "<subdomain-num><x>1</x>", "<subdomain-num><x>4</x>")
    assert read_configuration(path)["subdomain_num"] == (1, 1, 1)


_REF = orc.reference_checkout()
REF_CONFIGS = os.path.join(_REF, "configurations") if _REF else ""


@pytest.mark.skipif(not os.path.isdir(REF_CONFIGS), reason="reference checkout not present")
@pytest.mark.parametrize("name", sorted(f for f in (os.listdir(REF_CONFIGS) if os.path.isdir(REF_CONFIGS) else [])
                                        if f.endswith(".xml")))
def test_reader_on_the_reference_configurations(lib, reference, name):
    """The reference's shipped configurations, read by both readers (the
    reference's in a child process, since its checks assert)."""
    import subprocess
    import sys

    from cavityflow_cuda_gb300 import LbmError, read_configuration

    path = os.path.join(REF_CONFIGS, name)
    for tag in ("f64", "f32"):
        r = subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), "--config-one", path, tag],
                           capture_output=True, text=True)
        if r.returncode != 0:
            with pytest.raises(LbmError):
                read_configuration(path)
            continue
        want = json.loads(r.stdout.strip().splitlines()[-1])
        got = read_configuration(path)
        bad = {k: (got[k], want[k]) for k in want if not _same(got[k], want[k], tag)}
        assert not bad, bad
