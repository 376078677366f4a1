"""Mitsuba-XML / OBJ loading (CPU): round trip of the library's own exporter,
the reference's CBox fixtures where the reference tree is present, and
malformed input."""
import ctypes
import os
import sys

import numpy as np
import pytest

import gr
from gr import mitsuba, scenes as sc

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import refsrc  # noqa: E402


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
    path = refsrc.cbox_scenes().get(name)
    if not path:
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
    assert not p.warnings
    v, mesh, mats = p.triangles()
    assert mats[2].type == gr.MAT_PLASTIC  # roughplastic: Lambert + GGX lobes (reference defaults)
    assert tuple(mats[2].color) == pytest.approx((0.5, 0.5, 0.5)) and tuple(mats[2].specular) == (1.0, 1.0, 1.0)
    assert mats[2].eta_i[0] == pytest.approx(1.5) and mats[2].eta_t[0] == 1.0 and mats[2].alpha_v == mats[2].alpha_u
    sph = v[mesh == 0].reshape(-1, 3)
    # the reference composes a transform's children by right-multiplication
    # (m_transform *= X), so the later <translate> acts first: centre (2, 0, 0)
    r = np.linalg.norm(sph - np.array([2, 0, 0], np.float32), axis=1)
    np.testing.assert_allclose(r, 2.0, atol=1e-5)


def _write_ppm(path, rgb8):
    h, w, _ = rgb8.shape
    path.write_bytes(b"P6\n# test image\n%d %d\n255\n" % (w, h) + rgb8.astype(np.uint8).tobytes())


def _write_pfm(path, rgb):
    h, w, _ = rgb.shape  # rows bottom first, little endian
    path.write_bytes(b"PF\n%d %d\n-1.0\n" % (w, h) + np.ascontiguousarray(rgb, "<f4").tobytes())


def test_textures_envmap_and_texcoords(tmp_path):
    """Checkerboard and bitmap textures, an envmap and OBJ texcoords load into
    the material maps and the environment: PPM bytes become (c/255)^2.2 with
    row 0 the image's bottom row; PFM rows are taken as stored."""
    img = np.arange(4 * 3 * 3).reshape(4, 3, 3) * 7  # 4 rows, 3 columns
    _write_ppm(tmp_path / "tex.ppm", img)
    env = np.random.default_rng(5).random((8, 16, 3)).astype(np.float32)
    _write_pfm(tmp_path / "sky.pfm", env)
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                                    "f 1/1 2/2 3/3\nf 1/1 3/3 4/4\n")
    x = tmp_path / "t.xml"
    x.write_text("""<scene>
      <sensor type="perspective"><float name="fov" value="45"/>
        <transform name="toWorld"><lookat target="0,0,0" origin="0,0,5" up="0,1,0"/></transform>
        <film type="ldrfilm"><integer name="width" value="16"/><integer name="height" value="16"/></film></sensor>
      <emitter type="envmap"><string name="filename" value="sky.pfm"/>
        <transform name="toWorld"><rotate y="1" angle="30"/></transform></emitter>
      <shape type="obj"><string name="filename" value="q.obj"/>
        <bsdf type="diffuse"><texture type="checkerboard" name="reflectance">
          <rgb name="color0" value="0.9 0.1 0.1"/><rgb name="color1" value="0.1 0.9 0.1"/>
          <float name="uscale" value="4"/><float name="voffset" value="0.5"/></texture></bsdf></shape>
      <shape type="cube"><bsdf type="diffuse"><texture type="bitmap" name="reflectance">
          <string name="filename" value="tex.ppm"/></texture></bsdf></shape>
      <shape type="rectangle"><bsdf type="diffuse"><texture type="bitmap" name="reflectance">
          <string name="filename" value="missing.png"/></texture></bsdf></shape>
    </scene>""")
    p = gr.ParsedScene(str(x))
    assert p.env_map_size == (16, 8)
    assert len(p.warnings) == 1 and "missing.png" in p.warnings[0], p.warnings
    _, _, mats = p.triangles()
    chk, bmp, grey = mats[0], mats[1], mats[2]
    assert (chk.color_map_width, chk.color_map_height) == (2, 2)
    assert tuple(chk.uv_scale) == (4.0, 1.0) and tuple(chk.uv_offset) == (0.0, 0.5)
    c = np.ctypeslib.as_array(ctypes.cast(chk.color_map, ctypes.POINTER(ctypes.c_float)), (12,)).reshape(2, 2, 3)
    np.testing.assert_allclose(c, [[[0.9, 0.1, 0.1], [0.1, 0.9, 0.1]], [[0.1, 0.9, 0.1], [0.9, 0.1, 0.1]]], rtol=1e-6)
    assert (bmp.color_map_width, bmp.color_map_height) == (3, 4)
    b = np.ctypeslib.as_array(ctypes.cast(bmp.color_map, ctypes.POINTER(ctypes.c_float)), (36,)).reshape(4, 3, 3)
    np.testing.assert_allclose(b, (img[::-1] / 255.0) ** 2.2, rtol=1e-5)
    assert not grey.color_map


def test_parsed_scene_as_records_round_trip(tmp_path):
    """gr_scene_desc_mesh / ParsedScene.scene_desc: a scene written as XML + OBJ
    and parsed back gives the same meshes, normals, materials and camera."""
    from gr import mitsuba
    d = sc.glossy_scene(40, 30, level=1, glass_level=1)
    path = mitsuba.write_scene(d, str(tmp_path))
    back = gr.ParsedScene(path).scene_desc()
    assert len(back.meshes) == len(d.meshes)
    for a, b in zip(d.meshes, back.meshes):
        np.testing.assert_array_equal(b.positions[b.indices], a.positions[a.indices])
        assert (a.normals is None) == (b.normals is None)
        if a.normals is not None:  # renormalised by the loader, as the reference's does
            np.testing.assert_allclose(b.normals[b.indices], a.normals[a.indices], atol=1e-6)
        ma, mb = gr.material_record(d.materials[a.material]), gr.material_record(back.materials[b.material])
        assert ma.type == mb.type
        np.testing.assert_allclose(list(mb.color), list(ma.color))
        np.testing.assert_allclose(list(mb.emission), list(ma.emission))
    np.testing.assert_allclose(back.camera["to_world"], d.camera["to_world"], atol=1e-6)
    assert (back.camera["width"], back.camera["height"]) == (40, 30)


def test_scene_desc_file_round_trip(tmp_path):
    import ref_gpu
    d = sc.glossy_scene(40, 30, level=1, glass_level=1)
    ref_gpu.save_desc(d, tmp_path / "s.npz")
    back = ref_gpu.load_desc(tmp_path / "s.npz", 20, 15)
    assert (back.camera["width"], back.camera["height"]) == (20, 15) and back.camera["fov"] == d.camera["fov"]
    assert back.env == tuple(np.float32(d.env))
    for a, b in zip(d.meshes, back.meshes):
        np.testing.assert_array_equal(a.positions, b.positions)
        np.testing.assert_array_equal(a.indices, b.indices)
        assert a.material == b.material
    assert [gr.material_record(m).type for m in back.materials] == [gr.material_record(m).type for m in d.materials]


def test_reference_cbox_parses():
    path = refsrc.cbox_scenes().get("cbox.xml")
    if not path:
        pytest.skip("reference tree absent")
    d = gr.ParsedScene(path).scene_desc()
    assert len(d.meshes) == 6 and sum(m.normals is not None for m in d.meshes) == 2
    kinds = sorted((gr.material_record(m).type, round(gr.material_record(m).ior, 3)) for m in d.materials)
    assert kinds.count((gr.MAT_DIELECTRIC, 100.0)) == 1 and kinds.count((gr.MAT_DIELECTRIC, 1.5)) == 1
    assert sum(1 for m in d.materials if any(m["emission"])) == 1
