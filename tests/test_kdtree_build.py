"""The product's kd-tree builder reproduces the reference builder's node
stream word for word (golden trees built by the reference itself)."""
import numpy as np
import pytest

from conftest import golden
from yar_gb300 import native
from yar_gb300.scene import FlatScene


@pytest.mark.parametrize("name", ["raycast_small.yfs", "transform_small.yfs", "cornell_c1_64.yfs"])
@pytest.mark.parametrize("threads", [1, 4])
def test_builder_matches_reference_trees(name, threads):
    ref = FlatScene.read(golden(name))
    for m in ref.meshes:
        bounds, nodes = native.build_mesh_kdtree(m.vertices, m.indices, threads)
        assert np.array_equal(bounds.view(np.uint32), m.bounds.view(np.uint32))
        assert np.array_equal(nodes, m.nodes)
    mine = FlatScene.read(golden(name))
    mine.build_scene_kdtree()
    assert np.array_equal(mine.scene_nodes, ref.scene_nodes)
    assert np.array_equal(mine.scene_bounds.view(np.uint32), ref.scene_bounds.view(np.uint32))


def test_builder_matches_reference_regression_meshes():
    g = np.load(golden("kdtree_regression.npz"))
    for k in range(2):
        bounds, nodes = native.build_mesh_kdtree(g["mesh%d_vertices" % k], g["mesh%d_indices" % k], 1)
        assert np.array_equal(nodes, g["mesh%d_nodes" % k])
        assert np.array_equal(bounds, g["mesh%d_bounds" % k])


def test_builder_edge_cases():
    # one triangle: a single leaf holding index 0
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b, nodes = native.build_mesh_kdtree(v, [[0, 1, 2]], 1)
    assert nodes.tolist() == [[3 | (1 << 2), 0]]
    # all triangles in one plane perpendicular to an axis
    rng = np.random.default_rng(0)
    v = rng.random((300, 3)).astype(np.float32)
    v[:, 2] = 0.5
    idx = rng.integers(0, 300, (100, 3)).astype(np.int32)
    idx = idx[(idx[:, 0] != idx[:, 1]) & (idx[:, 1] != idx[:, 2]) & (idx[:, 0] != idx[:, 2])]
    b, nodes = native.build_mesh_kdtree(v, idx, 2)
    assert b[2] == b[5] == np.float32(0.5)
    # invalid input is rejected, not built
    with pytest.raises(native.YarError):
        native.build_mesh_kdtree(v, [[0, 1, 999]], 1)
    with pytest.raises(native.YarError):
        native.build_mesh_kdtree(v, np.zeros((0, 3), np.int32), 1)


def test_leaf_layout():
    """Leaves store count << 2 | 3 and the sorted primitive indices from word1
    on, padded to a node boundary (src/ref/kdtree_builder.cpp:304-321)."""
    ref = FlatScene.read(golden("raycast_small.yfs"))
    nodes = ref.meshes[0].nodes
    words = nodes.reshape(-1)
    i = 0
    seen_multi = False
    while i < nodes.shape[0]:
        w0 = nodes[i, 0]
        if w0 & 3 == 3:
            count = int(w0 >> 2)
            idx = words[2 * i + 1: 2 * i + 1 + count]
            assert np.all(np.diff(idx.astype(np.int64)) > 0)
            seen_multi |= count > 1
            i += 1 + (count // 2 if count > 1 else 0)
        else:
            i += 1
    assert seen_multi


def test_kdtree_cache_files_match_the_reference(tmp_path):
    """Cache files the reference wrote (KdTree::save) read back as the nodes
    and bounds of the reference-built scene, and writing those nodes gives
    byte-identical files."""
    import os
    from yar_gb300 import native
    s = FlatScene.read(golden("raycast_small.yfs"))
    cache = golden("kdtree_cache")
    for name, bounds, nodes in (("mesh_0.kdtree", s.meshes[0].bounds, s.meshes[0].nodes),
                                ("mesh_1.kdtree", s.meshes[1].bounds, s.meshes[1].nodes),
                                ("scene.kdtree", s.scene_bounds, s.scene_nodes)):
        b, n, h = native.read_kdtree_cache(os.path.join(cache, name))
        assert h == 0
        assert np.array_equal(b.view(np.uint32), np.asarray(bounds, np.float32).view(np.uint32))
        assert np.array_equal(n, nodes)
        out = os.path.join(tmp_path, name)
        native.write_kdtree_cache(out, b, n)
        assert open(out, "rb").read() == open(os.path.join(cache, name), "rb").read()
    # a whole scene round trip through the cache directory
    s.write_kdtree_caches(str(tmp_path / "all"))
    t = FlatScene.read(golden("raycast_small.yfs")).read_kdtree_caches(str(tmp_path / "all"))
    for m, mm in zip(s.meshes, t.meshes):
        assert np.array_equal(m.nodes, mm.nodes)
    # truncated and missing files are refused
    bad = os.path.join(tmp_path, "bad.kdtree")
    open(bad, "wb").write(open(os.path.join(cache, "mesh_0.kdtree"), "rb").read()[:-3])
    with pytest.raises(native.YarError):
        native.read_kdtree_cache(bad)
    with pytest.raises(native.YarError):
        native.read_kdtree_cache(os.path.join(tmp_path, "missing.kdtree"))
