"""The device inputs prepared for the reference's own GPU path tracer
(oracle/ref_gpu.py, which times and checks that kernel on the GPU) equal what
the reference's host code gives it: the breadth-first KDTreeGPUNode array
and leaf index list of buildGPUTreeFromKDTree (src/gpu_util.cpp:7-57),
field by field, on median trees of several sizes. Skipped where the
reference was not built from source (oracle/_ref)."""
import numpy as np
import pytest

from nostrum_pray_gb300 import scenes


@pytest.mark.parametrize("n,seed", [(14, 0), (100, 1), (3000, 4), (20_000, 2)])
def test_breadth_first_tree_matches_reference(oracle, n, seed):
    if not oracle.ref_available("default"):
        pytest.skip("reference not built from source on this machine")
    from oracle import ref_gpu as G
    m = scenes.soup(n, seed)
    nodes, tris, idx = G.gpu_tree(m)
    ref, ridx = oracle.ReferenceScene(m, "median", "default").gpu_tree()
    for k, want in ref.items():
        got = np.ascontiguousarray(nodes[k]).astype(want.dtype)
        np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=k)
    np.testing.assert_array_equal(idx, ridx)
    # triangles carry the reference's precomputed fields
    pre = oracle.ReferenceScene(m, "median", "default").precompute()
    np.testing.assert_array_equal(tris["box"], pre[:, 0:6])
    np.testing.assert_array_equal(tris["mid"], pre[:, 6:9])
    np.testing.assert_array_equal(tris["ab"], pre[:, 9:12])
    np.testing.assert_array_equal(tris["ac"], pre[:, 12:15])
    np.testing.assert_array_equal(tris["normal"], pre[:, 15:18])
