"""Mitsuba-XML / OBJ loading (CPU): round trip of the library's own exporter,
the reference's CBox fixtures where the reference tree is present, and
malformed input."""
import os

import numpy as np
import pytest

import gr
from gr import mitsuba, scenes as sc

REF_CBOX = "/root/reference/scene/CBox"


def test_exported_cornell_box_round_trip(tmp_path):
    d = sc.cornell_box(64, 48)
    path = mitsuba.write_scene(d, str(tmp_path))
    p = gr.ParsedScene(path)
    assert p.warnings == []
    assert p.num_triangles == d.num_triangles == 36
    assert p.num_light_triangles == 2
    assert (p.camera["width"], p.camera["height"]) == (64, 48)
    np.testing.assert_allclose(p.camera["to_world"], d.camera["to_world"], rtol=0, atol=0)
    v, mesh, mats = p.triangles()
    soup, _, tmat = d.flatten()
    np.testing.assert_array_equal(v, soup)
    assert mats[5].emission[:] == [15.0, 15.0, 15.0]


def test_exported_glossy_scene_round_trip(tmp_path):
    d = sc.glossy_scene(32, 24, level=2, glass_level=1)
    path = mitsuba.write_scene(d, str(tmp_path))
    p = gr.ParsedScene(path)
    v, _, mats = p.triangles()
    np.testing.assert_array_equal(v, d.flatten()[0])
    assert p.env == pytest.approx(d.env)
    types = [m.type for m in mats]
    assert gr.MAT_CONDUCTOR in types and gr.MAT_DIELECTRIC in types
    alphas = sorted(m.alpha_u for m in mats if m.type == gr.MAT_CONDUCTOR)
    assert alphas == pytest.approx([0.01, 0.1, 0.25, 0.5])


@pytest.mark.parametrize("name,tris", [("cbox.xml", None), ("cbox(mesh).xml", None), ("cbox(sphere).xml", None)])
def test_reference_cbox_fixtures_parse(name, tris):
    path = os.path.join(REF_CBOX, name)
    if not os.path.exists(path):
        pytest.skip("reference scenes not present")
    p = gr.ParsedScene(path)
    assert p.num_triangles > 0 and p.num_light_triangles >= 2
    assert p.camera["width"] == 800 and p.camera["height"] == 600
    v, _, mats = p.triangles()
    assert np.isfinite(v).all()
    if "sphere" in name:
        # two lat-long spheres of subdiv 100: 2 * 99 * 200 triangles
        assert p.num_triangles - 2 * 99 * 200 >= 0


def test_malformed_xml_is_reported(tmp_path):
    bad = tmp_path / "bad.xml"
    bad.write_text("<scene><shape type=\"obj\"><string name=\"filename\" value=\"missing.obj\"/></shape>")
    with pytest.raises(gr.GrError) as e:
        gr.ParsedScene(str(bad))
    assert e.value.status == 4
    bad.write_text("<scene><shape type=\"obj\"><string name=\"filename\" value=\"missing.obj\"/></shape></scene>")
    with pytest.raises(gr.GrError) as e:
        gr.ParsedScene(str(bad))
    assert "missing.obj" in str(e.value)


def test_procedural_shapes(tmp_path):
    x = tmp_path / "s.xml"
    x.write_text("""<scene>
      <sensor type="perspective"><float name="fov" value="45"/>
        <transform name="toWorld"><lookat target="0,0,0" origin="0,0,5" up="0,1,0"/></transform>
        <film type="ldrfilm"><integer name="width" value="32"/><integer name="height" value="32"/></film></sensor>
      <bsdf type="diffuse" id="grey"><rgb name="reflectance" value="0.5"/></bsdf>
      <shape type="sphere"><integer name="subdiv" value="10"/><ref id="grey"/>
        <transform name="toWorld"><scale value="2 2 2"/><translate x="1"/></transform></shape>
      <shape type="rectangle"><emitter type="area"><rgb name="radiance" value="5 5 5"/></emitter>
        <transform name="toWorld"><rotate x="1" angle="90"/><translate y="3"/></transform></shape>
      <shape type="cube"><bsdf type="roughplastic"/></shape>
    </scene>""")
    p = gr.ParsedScene(str(x))
    assert p.num_triangles == 9 * 20 * 2 + 2 + 12
    assert p.num_light_triangles == 2
    assert any("roughplastic" in w for w in p.warnings)
    v, mesh, mats = p.triangles()
    sph = v[mesh == 0].reshape(-1, 3)
    # the reference composes a transform's children by right-multiplication
    # (m_transform *= X), so the later <translate> acts first: centre (2, 0, 0)
    r = np.linalg.norm(sph - np.array([2, 0, 0], np.float32), axis=1)
    np.testing.assert_allclose(r, 2.0, atol=1e-5)
