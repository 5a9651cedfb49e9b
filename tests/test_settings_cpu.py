"""settings.xml, the reference's configuration file, read into a problem case
(minimmerflow_gb300.settings; problem.cpp:37-211, main.cpp:98-121,
body.cpp:49-72)."""
import os

import pytest

import minimmerflow_gb300 as mmf

REF_TESTS = os.path.join(os.environ.get("MMF_REFERENCE", "/root/reference"), "test")

FFSTEP_XML = """<?xml version="1.0"?>
<minimmerflow version="1">
    <problem>
        <type>ffstep</type>
        <dimensions>2</dimensions>
        <domain>
            <origin><x>0</x><y>0</y></origin>
            <length>3.2</length>
        </domain>
        <start>0.7</start>
    </problem>
    <discretization>
        <space><order>1</order><nCells>96</nCells></space>
        <time><CFL>0.4</CFL></time>
    </discretization>
    <bodies>
        <step><type>box</type><xMin>0.6</xMin><xMax>4</xMax><yMin>-1</yMin><yMax>0.2</yMax>
              <zMin>-1</zMin><zMax>1</zMax></step>
    </bodies>
</minimmerflow>"""


def test_settings_with_domain_body_and_defaults():
    s = mmf.settings.load(FFSTEP_XML)
    c = s.case
    assert c.problem == mmf.problem.FFSTEP and c.dim == 2 and c.n == (96, 96, 1)
    assert c.origin == (0.0, 0.0, 0.0) and c.length == 3.2 and c.cfl == 0.4
    assert c.t_end == 4.0                       # problem.cpp:205 default for ffstep
    assert s.t_start == 0.0                     # the reference reads <start> as an integer
    assert s.order == 1
    assert s.bodies == [((0.6, -1.0, -1.0), (4.0, 0.2, 1.0))]
    assert s.needs_face_list
    assert mmf.settings.load(FFSTEP_XML, n_cells=40).case.n == (40, 40, 1)   # argv[1]


def test_settings_errors_follow_the_reference():
    bad = FFSTEP_XML.replace("<type>ffstep</type>", "<type>shock_tube</type>")
    with pytest.raises(ValueError, match="not supported"):
        mmf.settings.load(bad)
    nolength = FFSTEP_XML.replace("<length>3.2</length>", "")
    with pytest.raises(ValueError):
        mmf.settings.load(nolength)             # the domain length is mandatory for ffstep
    sphere = FFSTEP_XML.replace("<type>box</type>", "<type>sphere</type>")
    with pytest.raises(ValueError, match="Body shape"):
        mmf.settings.load(sphere)


@pytest.mark.skipif(not os.path.isdir(REF_TESTS), reason="reference tree not present")
@pytest.mark.parametrize("name", ["2dIsentropicVortex", "2dRadSod", "3dIsentropicVortexXY", "3dIsentropicVortexYZ",
                                  "3dRadSod"])
def test_reference_settings_files(orc, name):
    """The reference's own regression settings give the cases its goldens
    were computed on."""
    s = mmf.settings.load(os.path.join(REF_TESTS, name, "settings.xml"))
    pname, dim, n, cfl, t_end, _ = orc.GOLDEN_CASES[name]
    c = s.case
    assert c.problem == mmf.problem.PROBLEMS[pname] and c.dim == dim and c.n[0] == n
    assert c.cfl == cfl and c.t_end == t_end and s.order == 1 and not s.needs_face_list
    origin, length = orc.reference_domain(orc.PROBLEMS[pname])
    assert c.origin == origin and c.length == length
