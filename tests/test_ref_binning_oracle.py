"""The C restatement of the reference binning (oracle/ref_binning.c) is bit-exact with the
reference CUDA rasterizer's own kernels (preprocessCUDA, getGaussianTileKeys, thrust sort,
getPerTileRanges) on the golden fixtures produced by tests/golden/make_ref_binning_golden.py.
No GPU."""

import os

import numpy as np
import pytest

from oracle.ref_binning import ref_binning
from tests.golden.binning_cases import binning_cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_binning_golden.npz")
CASES = {c["name"]: c for c in binning_cases()}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def run(case):
    return ref_binning(case["means"], case["scales"], case["rots"], case["view"], case["proj"],
                       case["H"], case["W"], case["tan_fovx"], case["tan_fovy"], case["n_std"])


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("variant", ["nofma", "fma"])
def test_oracle_matches_reference_kernels(golden, name, variant):
    case = CASES[name]
    for k in ("means", "scales", "rots", "view", "proj"):
        assert np.array_equal(golden[f"{name}/in_{k}"], np.asarray(case[k], np.float32)), k
    r = run(case)
    assert np.array_equal(r["radii"], golden[f"{name}/{variant}_radii"])
    assert np.array_equal(r["means2d"].view(np.uint32), golden[f"{name}/{variant}_means2d"].view(np.uint32))
    assert np.array_equal(r["tiles_touched"], golden[f"{name}/{variant}_tiles_touched"])
    assert np.array_equal(r["keys"], golden[f"{name}/{variant}_keys"])
    assert np.array_equal(r["ranges"], golden[f"{name}/{variant}_ranges"])


def test_structure_of_keys_and_ranges():
    r = run(CASES["odd_size"])
    keys = r["keys"]
    assert np.all(np.diff(keys.astype(np.float64)) > 0)  # strictly ascending, unique
    tiles = (keys >> np.uint64(32)).astype(np.int64)
    ranges = r["ranges"]
    for t in np.unique(tiles):
        s, e = ranges[t]
        assert np.all(tiles[s:e] == t)
    empty = np.setdiff1d(np.arange(ranges.shape[0]), np.unique(tiles))
    assert np.all(ranges[empty] == 0)  # empty tiles keep {0,0} (zeroed scratch in the reference)
    assert r["tiles_touched"][-1] == keys.size


def test_empty_input():
    c = dict(CASES["single"])
    for k in ("means", "scales", "rots"):
        c[k] = np.zeros((0, c[k].shape[1]), np.float32)
    r = run(c)
    assert r["num_keys"] == 0 and np.all(r["ranges"] == 0)


def test_near_plane_and_offscreen_cull():
    r = run(CASES["edges"])
    assert r["radii"][0] == 0          # z == 0.2 is culled (auxiliary.h:159, z <= 0.2)
    assert r["radii"][2] == 0          # behind the camera
    assert r["radii"][3] == 0          # far off-screen: empty rectangle
    gx, gy = (96 + 7) // 8, (72 + 7) // 8
    touched = np.diff(np.concatenate([[0], r["tiles_touched"]]))
    assert touched[4] == gx * gy       # the huge Gaussian covers every tile
