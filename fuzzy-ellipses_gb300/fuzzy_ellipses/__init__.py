"""fuzzy_ellipses -- GB300-native fuzzy-metaball renderer (sm_103a).

Drop-in for the render path of the reference's ``fuzzy_ellipses`` package: the same entry-point
name and legacy signature (``rasterize``), plus the re-specified ``render`` that takes the
Gaussian precision factor and a (quaternion, translation) pose like ``baseline/fm_render.py``'s
``render_func_quat``, with a native backward. Every stage is a CUDA kernel in
``_lib/libfuzzy_ellipses.so``; there is no CPU path.
"""

from . import adapters, autotune, serve, synthetic  # noqa: F401
from ._native import FEError, NativeLibraryMissing, load as load_native  # noqa: F401
from .api import (Batch, bench_peak, device_status, gmm_log_likelihood,  # noqa: F401
                  projection_matrix, rasterize, reference_binning, reference_num_stds, render,
                  render_binning, render_features, render_forward, render_pixels,
                  render_pixels_cam,
                  silhouette_bce)

__version__ = "0.1.0"
