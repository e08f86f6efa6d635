"""Oracle: CPU restatements of the reference's render path (TEST INFRASTRUCTURE ONLY).

* fm_render_np     -- float64 NumPy restatement of baseline/fm_render.py (depth/alpha oracle)
* fm_render_torch  -- the same in torch float64, for gradients by autograd (stand-in for jax.grad)
* ref_binning      -- C restatement of the reference CUDA rasterizer's binning (key parity)
* ref_driver.cu    -- runs the reference's own binning kernels, compiled from its sources, on a GPU
                      to produce golden fixtures

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this package, and
only as the checker or as the timed CPU baseline; the product never imports it.
"""
