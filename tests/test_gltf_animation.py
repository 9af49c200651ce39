"""glTF animation and skinning on the host against the animation oracle
(oracle/anim_oracle.py, a float64 restatement of the reference's
updateScene): channel sampling (STEP, LINEAR with slerp, CUBICSPLINE), time
wrapping, the reference's choice of animation, node hierarchies, skins with
joint matrices relative to the mesh node, and normals through the mesh
node's inverse transpose."""
import numpy as np
import pytest

import optix_pt_gb300 as opt
from gltf_writer import animated_scene
from oracle import anim_oracle as ao

TIMES = [0.0, 0.25, 0.5, 0.99, 1.0, 1.6, 2.0, 2.7, 4.3]


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    g = animated_scene()
    path = g.save(tmp_path_factory.mktemp("anim") / "anim.gltf")
    m = opt.GltfModel(path)
    yield m, g.doc, bytes(g.bin)
    m.close()


def test_info(model):
    m, doc, _ = model
    assert m.info["numShapes"] == 4 and m.info["numJointSlots"] == 2 and m.info["skinned"] == 1
    assert m.info["numChannels"] == 4 and m.info["duration"] == 2.0


@pytest.mark.parametrize("t", TIMES)
def test_pose_matches_oracle(model, t):
    m, doc, binary = model
    p, n = m.apply(t)
    op, on = ao.vertices(doc, binary, t)
    assert p.shape == op.shape
    assert np.allclose(p, op, rtol=1e-5, atol=2e-6), np.abs(p - op).max()
    assert np.allclose(n, on, rtol=1e-5, atol=2e-6), np.abs(n - on).max()


def test_scene_at_time_is_the_applied_pose(model):
    m, _, _ = model
    for t in (0.0, 1.3):
        a = m.scene(t, animate=True).arrays()
        p, n = m.apply(t)
        assert np.array_equal(a["positions"], p) and np.array_equal(a["normals"], n)
    rest = m.scene(0.0, animate=False).arrays()
    p0, _ = m.apply(0.0)
    # at t = 0 every channel sits on its first key except the box's STEP
    # channel, whose first key is at 0.5 (held before it: the first value)
    assert np.allclose(rest["positions"], p0, atol=1e-6)


def test_motion_and_wrap(model):
    m, _, _ = model
    p1, _ = m.apply(1.0)
    p2, _ = m.apply(1.6)
    assert np.abs(p1 - p2).max() > 0.1
    pa, _ = m.apply(0.7)
    pb, _ = m.apply(0.7 + 2.0)  # every channel's last key is at 2.0 or 1.5 ...
    # ... the STEP channel (last key 1.5) wraps with its own period
    pc, _ = m.apply(0.7 + 3.0)
    assert np.isfinite(pb).all() and np.isfinite(pc).all()


@pytest.mark.parametrize("count,moving_index", [(1, 0), (2, 0), (3, 2), (4, 2)])
def test_animation_choice(tmp_path, count, moving_index):
    g = animated_scene(num_animations=count)
    m = opt.GltfModel(g.save(tmp_path / ("a%d.gltf" % count)))
    assert m.info["numChannels"] == 4  # the moving animation, never the decoy
    ground_before, _ = m.apply(0.0)
    ground_after, _ = m.apply(0.9)
    # ground is the last shape: its 4 vertices stay put
    assert np.array_equal(ground_before[-4:], ground_after[-4:])
    m.close()


def test_deformation_data(model):
    m, _, _ = model
    d = m.deformation()
    assert d.numVertices == m.info["numVertices"] and d.numShapes == 4 and d.numJoints == 2
    assert d.joints and d.weights and d.restNormals
