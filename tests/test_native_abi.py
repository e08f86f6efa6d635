"""The C-ABI library loads, exports every symbol include/fuzzy_ellipses.h declares, its ctypes
mirrors match the C struct layouts, and host-side argument checks return status codes (no GPU
work is issued by these checks)."""

import ctypes
import os
import re
import subprocess

import pytest

import fuzzy_ellipses
from fuzzy_ellipses import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fuzzy_ellipses.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fe_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = fuzzy_ellipses.load_native()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(N.PROTOTYPES), set(names) ^ set(N.PROTOTYPES)
    assert lib.fe_version().startswith(b"fuzzy_ellipses_gb300")


def test_struct_layouts_match_c(tmp_path):
    prog = tmp_path / "sizes.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "fuzzy_ellipses.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(fe_render_desc),"
        " sizeof(fe_legacy_desc), sizeof(fe_view), sizeof(fe_scene),"
        " offsetof(fe_view, pixel_offset), offsetof(fe_render_desc, tile_w),"
        " sizeof(fe_server_config), offsetof(fe_server_config, desc), sizeof(fe_request),"
        " offsetof(fe_request, user_tag), sizeof(fe_completion), sizeof(fe_server_stats));return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert [int(x) for x in out] == [ctypes.sizeof(N.RenderDesc), ctypes.sizeof(N.LegacyDesc),
                                     ctypes.sizeof(N.View), ctypes.sizeof(N.SceneEntry),
                                     N.View.pixel_offset.offset, N.RenderDesc.tile_w.offset,
                                     ctypes.sizeof(N.ServerConfig), N.ServerConfig.desc.offset,
                                     ctypes.sizeof(N.Request), N.Request.user_tag.offset,
                                     ctypes.sizeof(N.Completion), ctypes.sizeof(N.ServerStats)]
    assert ctypes.sizeof(N.LegacyDesc) == 20  # the reference's RasterizeDescriptor: 3 int + 2 float


def test_desc_init_defaults():
    d = N.make_desc(40, 200, 200, 200.0, 200.0, 100.0, 100.0)
    assert d.magic == N.FE_DESC_MAGIC and d.version == N.FE_DESC_VERSION
    assert abs(d.beta2 - 21.4) < 1e-6 and abs(d.beta3 - 2.66) < 1e-6
    assert d.cull_mode == N.FE_CULL_EPS and abs(d.cull_param - 1e-7) < 1e-12
    assert (d.tile_w, d.tile_h) == (16, 16)


def _fwd(d):
    lib = fuzzy_ellipses.load_native()
    null = ctypes.c_void_p(0)
    dummy = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    return lib.fe_render_fwd(ctypes.byref(d) if d is not None else None, dummy, dummy, dummy, dummy,
                             dummy, dummy, dummy, null, null)


def test_descriptor_validation_returns_status_codes():
    lib = fuzzy_ellipses.load_native()
    d = N.make_desc(4, 8, 8, 8.0, 8.0, 4.0, 4.0)
    bad = N.make_desc(4, 8, 8, 8.0, 8.0, 4.0, 4.0)
    bad.magic = 0
    assert _fwd(bad) == 2  # FE_ERR_DESCRIPTOR
    assert b"magic" in lib.fe_last_error_message()
    bad = N.make_desc(4, 8, 8, 8.0, 8.0, 4.0, 4.0)
    bad.tile_w = 12
    assert _fwd(bad) == 1  # FE_ERR_INVALID_ARGUMENT
    bad = N.make_desc(4, 0, 8, 8.0, 8.0, 4.0, 4.0)
    assert _fwd(bad) == 1
    bad = N.make_desc(4, 8, 8, 0.0, 8.0, 4.0, 4.0)
    assert _fwd(bad) == 1
    bad = N.make_desc(4, 8, 8, 8.0, 8.0, 4.0, 4.0)
    bad.cull_mode = 7
    assert _fwd(bad) == 1
    assert _fwd(None) == 1
    with pytest.raises(N.FEError):
        N.check(2)
    assert lib.fe_status_string(5) == b"key capacity exceeded"


def test_xla_target_rejects_bad_opaque_without_touching_buffers():
    lib = fuzzy_ellipses.load_native()
    # A wrong opaque length is reported through the (absent) XLA status and never reaches CUDA.
    lib.fe_render_fwd_xla(None, None, b"\x00" * 3, 3, None)
    assert b"opaque" in lib.fe_last_error_message()
    lib.fe_rasterize_legacy_xla(None, None, b"\x00" * 7, 7, None)
    assert b"opaque" in lib.fe_last_error_message()


def test_batch_create_validates_views():
    lib = fuzzy_ellipses.load_native()
    d = N.make_desc(0, 1, 1, 1.0, 1.0, 0.0, 0.0)
    sc = (N.SceneEntry * 1)()
    sc[0].gauss_offset, sc[0].n = 0, 10
    vs = (N.View * 1)()
    vs[0].scene = 3  # out of range
    vs[0].height = vs[0].width = 8
    vs[0].fx = vs[0].fy = 8.0
    h = ctypes.c_void_p()
    assert lib.fe_batch_create(ctypes.byref(d), sc, 1, vs, 1, ctypes.byref(h)) == 1
    assert not h.value


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(N.NativeLibraryMissing):
        saved = N._lib
        try:
            N._lib = None
            N.load(str(tmp_path / "nope.so"))
        finally:
            N._lib = saved
