"""Generate the key-parity golden fixtures by running the reference CUDA rasterizer's own binning
kernels (compiled from its sources into oracle/_ref/*.cubin by ``make -C oracle ref``; launched by
oracle/ref_driver.cu) on a GPU.

Run on a machine with a GPU, from the repository root, after ``make -C oracle ref`` was run where
the reference sources are available (the cubins then travel with the repository):

    make -C oracle driver && python tests/golden/make_ref_binning_golden.py OUT_DIR

Writes OUT_DIR/ref_binning_golden.npz with, per case, the inputs and the reference's outputs from
both the -fmad=false build (``nofma``, the bit-exact parity target) and the default-flags build
(``fma``, reported for context).
"""

from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from tests.golden.binning_cases import binning_cases  # noqa: E402


def run_driver(case, variant, tmp):
    inp = os.path.join(tmp, f"{case['name']}_in.bin")
    out = os.path.join(tmp, f"{case['name']}_{variant}_out.bin")
    P = case["means"].shape[0]
    with open(inp, "wb") as f:
        np.array([P, case["H"], case["W"]], np.int32).tofile(f)
        np.array([case["n_std"], case["tan_fovx"], case["tan_fovy"]], np.float32).tofile(f)
        for k in ("means", "scales", "rots", "view", "proj"):
            np.asarray(case[k], np.float32).ravel().tofile(f)
    drv = os.path.join(ROOT, "oracle", "_build", "ref_driver")
    fwd = os.path.join(ROOT, "oracle", "_ref", f"forward_{variant}.cubin")
    imp = os.path.join(ROOT, "oracle", "_ref", f"rasterizer_impl_{variant}.cubin")
    subprocess.run([drv, fwd, imp, inp, out], check=True)
    gx, gy = (case["W"] + 7) // 8, (case["H"] + 7) // 8
    with open(out, "rb") as f:
        K = int(np.fromfile(f, np.int64, 1)[0])
        radii = np.fromfile(f, np.int32, P)
        xy = np.fromfile(f, np.float32, 2 * P).reshape(P, 2)
        touched = np.fromfile(f, np.uint32, P)
        keys = np.fromfile(f, np.uint64, K)
        ranges = np.fromfile(f, np.uint32, 2 * gx * gy).reshape(-1, 2)
    return {"radii": radii, "means2d": xy, "tiles_touched": touched, "keys": keys, "ranges": ranges}


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    blob = {}
    with tempfile.TemporaryDirectory() as tmp:
        for case in binning_cases():
            name = case["name"]
            for k in ("means", "scales", "rots", "view", "proj"):
                blob[f"{name}/in_{k}"] = np.asarray(case[k], np.float32)
            blob[f"{name}/in_scalars"] = np.array(
                [case["H"], case["W"], case["n_std"], case["tan_fovx"], case["tan_fovy"]], np.float64)
            for variant in ("nofma", "fma"):
                res = run_driver(case, variant, tmp)
                for k, v in res.items():
                    blob[f"{name}/{variant}_{k}"] = v
            print(name, "P", case["means"].shape[0], "K", blob[f"{name}/nofma_keys"].size, flush=True)
    path = os.path.join(out_dir, "ref_binning_golden.npz")
    np.savez_compressed(path, **blob)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
