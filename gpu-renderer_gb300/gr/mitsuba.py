"""Writes a SceneDesc as a Mitsuba-XML scene with one OBJ file per mesh, in
the subset the reference's loader reads (mitsubaloader.cpp), so the reference
build and this library can render the same synthetic scene."""
import os

import numpy as np

import gr


def _v(x):
    return " ".join("%.9g" % float(c) for c in x)


def write_obj(path, mesh):
    with open(path, "w") as f:
        for p in mesh.positions:
            f.write("v %s\n" % _v(p))
        if mesh.normals is not None:
            for n in mesh.normals:
                f.write("vn %s\n" % _v(n))
        for t in mesh.indices + 1:
            if mesh.normals is not None:
                f.write("f %d//%d %d//%d %d//%d\n" % (t[0], t[0], t[1], t[1], t[2], t[2]))
            else:
                f.write("f %d %d %d\n" % (t[0], t[1], t[2]))


def _bsdf(m):
    r = gr.material_record(m)
    if r.type == gr.MAT_DIFFUSE:
        return '<bsdf type="diffuse"><rgb name="reflectance" value="%s"/></bsdf>' % _v(r.color)
    if r.type == gr.MAT_DIELECTRIC:
        return ('<bsdf type="dielectric"><float name="ior" value="%.9g"/>'
                '<rgb name="reflectance" value="%s"/></bsdf>' % (r.ior, _v(r.color)))
    return ('<bsdf type="roughconductor"><float name="alpha" value="%.9g"/>'
            '<rgb name="specularReflectance" value="%s"/><rgb name="eta" value="%s"/>'
            '<rgb name="k" value="%s"/></bsdf>' % (r.alpha_u, _v(r.color), _v(r.eta_t), _v(r.k)))


def write_scene(desc, directory, name="scene.xml"):
    os.makedirs(os.path.join(directory, "meshes"), exist_ok=True)
    lines = ["<scene>"]
    cam = desc.camera
    M = np.asarray(cam["to_world"], np.float32).reshape(16)
    lines.append('  <sensor type="perspective">')
    lines.append('    <float name="fov" value="%.9g"/>' % cam["fov"])
    lines.append('    <transform name="toWorld"><matrix value="%s"/></transform>' % _v(M))
    lines.append('    <film type="hdrfilm"><integer name="width" value="%d"/><integer name="height" value="%d"/>'
                 '</film>' % (cam["width"], cam["height"]))
    lines.append("  </sensor>")
    if desc.env is not None:
        lines.append('  <emitter type="constant"><rgb name="radiance" value="%s"/></emitter>' % _v(desc.env))
    for i, m in enumerate(desc.meshes):
        rel = "meshes/mesh%03d.obj" % i
        write_obj(os.path.join(directory, rel), m)
        mat = desc.materials[m.material]
        lines.append('  <shape type="obj">')
        lines.append('    <string name="filename" value="%s"/>' % rel)
        lines.append("    " + _bsdf(mat))
        em = mat.get("emission", (0, 0, 0))
        if any(float(x) != 0.0 for x in em):
            lines.append('    <emitter type="area"><rgb name="radiance" value="%s"/></emitter>' % _v(em))
        lines.append("  </shape>")
    lines.append("</scene>")
    path = os.path.join(directory, name)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path
