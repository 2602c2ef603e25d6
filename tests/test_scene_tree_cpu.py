"""Scene trees on the CPU: the builders behave like the reference's
(src/scene.rs:85-150), the pre-order node packing, and the oracle's tree
render against its flat scene render (pinned by the reference's KATs)."""
import numpy as np

from rasterize_gb300 import FillRule, LinColor, Scene, Transform, _ffi
from rasterize_gb300 import workloads as W
from tests.paint_oracle import oracle_scene, oracle_scene_tree


def star(seed, r=10.0, c=(20.0, 20.0)):
    return W.contour(np.random.default_rng(seed), 12, r, center=c)


def test_builders_merge_like_the_reference():
    a = Scene().fill(star(1), LinColor(1, 0, 0, 1))
    assert Scene.group([a]) is a  # a group of one child is the child
    o = a.opacity(0.5).opacity(0.5)
    assert o.kind == "opacity" and o.params["opacity"] == 0.25 and o.children[0] is a
    assert a.opacity(7.0).params["opacity"] == 1.0 and a.opacity(-1).params["opacity"] == 0.0
    t1, t2 = Transform.new_translate(3, 4), Transform.new_scale(2, 2)
    t = a.transform(t1).transform(t2)
    assert t.kind == "transform" and t.children[0] is a and t.params["tr"].m == (t2 * t1).m


def test_preorder_nodes_and_entries():
    f1, f2 = (star(1), LinColor(1, 0, 0, 1)), (star(2), LinColor(0, 1, 0, 1))
    inner = Scene().fill(*f1).fill(*f2)
    root = Scene().fill(star(3), LinColor(0, 0, 1, 1)).add(inner.clip(star(4, 5.0), fill_rule=FillRule.EvenOdd)
                                                           .opacity(0.5))
    entries, nodes, n = root.entries_and_nodes()
    kinds = [nodes[i].kind for i in range(n)]
    assert kinds == [_ffi.NODE_GROUP, _ffi.NODE_FILL, _ffi.NODE_OPACITY, _ffi.NODE_CLIP, _ffi.NODE_GROUP,
                     _ffi.NODE_FILL, _ffi.NODE_FILL]
    assert nodes[0].arg == 2 and nodes[4].arg == 2
    assert [nodes[i].arg for i in (1, 5, 6)] == [0, 1, 2]
    assert nodes[3].arg == 3 and len(entries) == 4 and int(entries[3][2]) == int(FillRule.EvenOdd)
    assert nodes[2].opacity == 0.5
    assert not root.is_flat() and inner.is_flat()
    assert len(root.fills) == 3


def test_oracle_tree_of_a_flat_group_is_the_flat_render():
    sc = W.scene(seed=5, n=30, size=128, seg_range=(20, 80), radius_range=(8, 40))
    bg = (0.1, 0.2, 0.3, 1.0)
    assert np.array_equal(oracle_scene(sc, 128, 96, bg=bg), oracle_scene_tree(sc, 128, 96, bg=bg))


def test_oracle_tree_out_of_view_is_background():
    far = Scene().fill(W.contour(np.random.default_rng(0), 8, 5.0, center=(500.0, 500.0)), LinColor(1, 1, 1, 1))
    img = oracle_scene_tree(far.opacity(0.5), 32, 16, bg=(0.25, 0.0, 0.0, 1.0))
    assert (img == np.float32([0.25, 0, 0, 1])).all()
