"""Subsystem (a) on the GPU: Morton sort, compressed octree, batches and
interaction lists must equal the CPU oracle's integer for integer, and the
node geometry bit for bit (both follow the same FP64 operation order)."""
import numpy as np
import pytest

from conftest import point_sets, to_cuda

pytestmark = pytest.mark.gpu

TREE_INT = ("codes", "perm", "begin", "end", "parent", "first_child", "nchild")
TREE_FP = ("center", "half", "radius")


def _plans(dev, oracle, tpts, spts, w, theta, degree, sl, tl, sc=1.0):
    tx, ty, tz = tpts.T
    sx, sy, sz = spts.T
    g = dev.TreecodePlan(*to_cuda(tx, ty, tz, sx, sy, sz, w), theta=theta, degree=degree,
                         source_leaf=sl, target_leaf=tl, size_check=sc)
    c = oracle.Plan(tx, ty, tz, sx, sy, sz, w, theta, degree, sl, tl, sc)
    return g, c


def _compare(g, c):
    for which in (0, 1):
        gt, ct = g.tree(which), c.tree(which)
        for k in TREE_INT:
            assert np.array_equal(gt[k], ct[k]), f"tree {which} field {k}"
        for k in TREE_FP:
            assert np.array_equal(gt[k], ct[k]), f"tree {which} field {k} (bitwise)"
    gl, cl = g.lists(), c.lists()
    for k in cl:
        assert np.array_equal(gl[k], cl[k]), f"list {k}"


@pytest.mark.parametrize("name", list(point_sets()))
@pytest.mark.parametrize("theta,degree,leaf", [(0.7, 7, 64), (0.5, 3, 16), (0.9, 5, 200)])
def test_tree_and_lists_match_oracle(dev, oracle, name, theta, degree, leaf):
    pts = point_sets()[name]
    w = np.random.default_rng(1).uniform(0.5, 1.5, len(pts))
    g, c = _plans(dev, oracle, pts, pts, w, theta, degree, leaf, leaf, sc=0.05)
    _compare(g, c)


def test_distinct_targets_and_sources(dev, oracle):
    rng = np.random.default_rng(11)
    t = rng.uniform(-1, 1, (2500, 3))
    s = rng.normal(0, 0.4, (4000, 3))
    g, c = _plans(dev, oracle, t, s, rng.uniform(0.1, 1, 4000), 0.6, 4, 50, 80, sc=0.2)
    _compare(g, c)


def test_mesh_lists(dev, oracle, small_mesh):
    mesh = small_mesh[0]
    pts = np.stack([mesh.x, mesh.y, mesh.z], 1)
    g, c = _plans(dev, oracle, pts, pts, mesh.w, 0.7, 7, 500, 500)
    _compare(g, c)
    assert g.info()["slots"] == c.n_slots


def test_lists_partition_sources(dev, small_mesh):
    """Every batch sees every source exactly once (near ranges + far clusters)."""
    mesh = small_mesh[0]
    g = dev.TreecodePlan.for_mesh(*to_cuda(mesh.x, mesh.y, mesh.z, mesh.w), theta=0.7, degree=5,
                                  source_leaf=100, target_leaf=100)
    st, lists = g.tree(0), g.lists()
    n = mesh.n
    for b in range(len(lists["batch_node"])):
        cover = np.zeros(n, np.int32)
        for e in range(lists["near_off"][b], lists["near_off"][b + 1]):
            c = lists["near_list"][e]
            cover[st["begin"][c]:st["end"][c]] += 1
        for e in range(lists["far_off"][b], lists["far_off"][b + 1]):
            c = lists["far_list"][e]
            cover[st["begin"][c]:st["end"][c]] += 1
        assert cover.min() == 1 and cover.max() == 1, f"batch {b}"
