"""Failure detection without a GPU fault: a device wait that nothing completes gives up after
its limit and reports a status the host reads, and the context stays usable."""

import ctypes

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import _native as N
from fuzzy_ellipses import synthetic as S
from tests.helpers import TOL_ALPHA, oracle_pixels, scene_to_dev

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports_timeout(cuda_device):
    lib = N.load()
    status, elapsed = ctypes.c_uint32(0), ctypes.c_uint64(0)
    limit = 2_000_000  # 2 ms
    N.check(lib.fe_selftest_bounded_wait(limit, ctypes.byref(status), ctypes.byref(elapsed),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    assert status.value == N.FE_DEVERR_TIMEOUT
    assert limit <= elapsed.value < 500_000_000
    # The context is still usable: a render right afterwards matches the oracle.
    scene, cams = S.config0(seed=0)
    c = cams[0]
    m, p, w = scene_to_dev(scene, cuda_device)
    _, a = fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
    assert fe.device_status() == 0
    pix = np.arange(0, c.height * c.width, 97)
    _, a_ref = oracle_pixels(scene, c, pix)
    assert np.max(np.abs(a.cpu().numpy().ravel()[pix] - a_ref)) <= TOL_ALPHA


def test_selftest_rejects_unbounded_limits(cuda_device):
    lib = N.load()
    status, elapsed = ctypes.c_uint32(0), ctypes.c_uint64(0)
    for bad in (0, 10, 5_000_000_000):
        assert lib.fe_selftest_bounded_wait(bad, ctypes.byref(status), ctypes.byref(elapsed),
                                            None) == 1  # FE_ERR_INVALID_ARGUMENT
