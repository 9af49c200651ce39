"""Procedural scenes, host material categorisation and the configs/*.json
scene-selection format (src/scene_desc.cpp:50-153 of the reference)."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT


def test_cornell_box_shape(built):
    import optix_pt_gb300 as opt
    s = opt.Scene.procedural("cornell")
    a = s.arrays()
    assert s.num_triangles == 36
    P, I = a["positions"], a["triIndices"]
    # every geometric normal of the room faces the interior (towards y = 1)
    ng = np.cross(P[I[:, 1]] - P[I[:, 0]], P[I[:, 2]] - P[I[:, 0]])
    cen = P[I].mean(1)
    walls = np.arange(12)
    inward = (np.array([0, 1, 0]) - cen[walls]) * np.array([1, 1, 1])
    assert (np.einsum("ij,ij->i", ng[walls], inward) > 0).all()
    assert a["resX"] == 512 and a["spp"] == 64 and a["maxDepth"] == 8


def test_spheres_shape(built):
    import optix_pt_gb300 as opt
    s = opt.Scene.procedural("spheres")
    a = s.arrays()
    assert s.num_triangles == 64 * 5120 + 4
    assert a["normals"] is not None and np.allclose(np.linalg.norm(a["normals"], axis=1), 1.0, atol=1e-5)
    assert a["numLights"] == 1 and (a["resX"], a["resY"]) == (1920, 1080)


def test_host_categories_follow_reference_rules(built):
    """Deterministic materials get a host category (material_params.h:116-223);
    the blended ones stay 0 and are categorised per hit."""
    import ctypes

    import optix_pt_gb300 as opt
    from optix_pt_gb300 import _ffi
    s = opt.Scene.procedural("spheres")
    mats = (_ffi.MaterialData * s.struct.numMaterials).from_address(ctypes.addressof(s.struct.materials.contents))
    cats = {}
    for m in mats:
        cats[(round(m.metallic, 3), m.specular, m.emission[0] > 0)] = m.category
    for (metallic, specular, emissive), c in cats.items():
        if emissive:
            assert c == 4
        elif metallic == 1.0:
            assert c == 1          # Metal
        elif metallic == 0.0 and specular == 0.0:
            assert c & 2 and c & 8 and c & 64   # Dielectric | Opaque | Diffuse
        else:
            assert c == 0          # blended: categorised per hit


def test_config_selection(built, tmp_path):
    import optix_pt_gb300 as opt
    s = opt.Scene.from_config(os.path.join(ROOT, "configs", "scene_selection.json"))
    assert s.num_triangles == 36
    # the list's "scene" id selects the file; renderer settings override
    (tmp_path / "list.json").write_text(json.dumps({"scene": "7", "7": "box"}))
    (tmp_path / "box.json").write_text(json.dumps({"scene": {"procedural scene": "cornell", "renderer": {
        "dimensions": [64, 32], "background colour": [0.1, 0.2, 0.3], "spp": 9, "max depth": 5}}}))
    s2 = opt.Scene.from_config(str(tmp_path / "list.json"))
    a = s2.arrays()
    assert (a["resX"], a["resY"], a["spp"], a["maxDepth"]) == (64, 32, 9, 5)
    assert np.allclose(a["bgColour"], [0.1, 0.2, 0.3])


@pytest.mark.parametrize("case,code", [
    ("missing_list", -3), ("bad_json", -4), ("no_id", -4), ("gltf", -3), ("no_renderer", -4), ("missing_scene", -3),
])
def test_config_errors(built, tmp_path, case, code):
    import optix_pt_gb300 as opt
    lst = tmp_path / "list.json"
    if case != "missing_list":
        body = {"scene": "1", "1": "s"}
        if case == "no_id":
            body = {"scene": "2", "1": "s"}
        lst.write_text("{ nope" if case == "bad_json" else json.dumps(body))
    scene = {"scene": {"procedural scene": "cornell", "renderer": {"dimensions": [8, 8]}}}
    if case == "gltf":
        scene = {"scene": {"gltf scene file": "x.gltf", "renderer": {"dimensions": [8, 8]}}}
    if case == "no_renderer":
        scene = {"scene": {"procedural scene": "cornell"}}
    if case != "missing_scene":
        (tmp_path / "s.json").write_text(json.dumps(scene))
    with pytest.raises(opt.OptptError) as e:
        opt.Scene.from_config(str(lst))
    assert e.value.code == code


def test_scenes_are_deterministic(built):
    import optix_pt_gb300 as opt
    a = opt.Scene.procedural("spheres", 3).arrays()
    b = opt.Scene.procedural("spheres", 3).arrays()
    assert np.array_equal(a["positions"], b["positions"]) and a["materials"] == b["materials"]
    c = opt.Scene.procedural("spheres", 4).arrays()
    assert a["materials"] != c["materials"]
