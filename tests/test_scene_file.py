"""Scenes written by the library (Scene.save) and read by the oracle without
the library (oracle.scene_file): same optpt_scene layout, same oracle
renders. The CPU baseline uses this path so that its process never loads the
CUDA library."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc
from oracle import scene_file


def test_scene_record_layout_matches_the_abi(built):
    from optix_pt_gb300 import _ffi
    for mine, theirs in ((scene_file.SceneRecord, _ffi.SceneStruct), (scene_file.TextureRecord, _ffi.Texture)):
        assert ctypes.sizeof(mine) == ctypes.sizeof(theirs)
        for (name, _), (name2, _) in zip(mine._fields_, theirs._fields_):
            assert name == name2
            assert getattr(mine, name).offset == getattr(theirs, name2).offset


@pytest.mark.parametrize("name", ["cornell", "spheres", "terrain_small"])
def test_saved_scene_renders_identically_in_the_oracle(built, tmp_path, name):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural(name)
    path = str(tmp_path / (name + ".npz"))
    sc.save(path)
    fs = scene_file.load(path)
    assert fs.num_triangles == sc.num_triangles
    a, b = sc.arrays(), fs.arrays()
    for k in ("positions", "triIndices", "matIndices"):
        assert np.array_equal(a[k], b[k])
    cam = [0.0, 1.0, 4.0, 0.4, 0, 0, 0, 0.4, 0, 0, 0, -1, 0, 0, 0]
    r1 = orc.SceneView(sc.struct, 4).render(cam, 24, 16, 1, 0, 2, 6, precision=32, threads=2)
    r2 = orc.SceneView(fs.struct, 4).render(cam, 24, 16, 1, 0, 2, 6, precision=32, threads=2)
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)
