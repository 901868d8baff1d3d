"""The C ABI: the library loads and exports every entry point the header
declares, and the ctypes structs mirror the header's layout (checked with
the C compiler, no GPU needed)."""
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "so3g_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(so3g_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import so3g_gb300.build as b
    b.build()
    from so3g_gb300 import _abi
    return _abi.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 17
    out = subprocess.run(["nm", "-D", "--defined-only",
                          os.path.join(ROOT, "so3g_gb300", "_lib", "libso3g_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (so3g_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)
    from so3g_gb300 import _abi
    assert sorted(_abi.symbols()) == names


def test_library_state_calls_without_gpu(lib):
    import numpy as np
    from so3g_gb300 import _abi
    assert lib.so3g_abi_version() == _abi.ABI_VERSION
    a = np.empty(_abi.LUT_N)
    b = np.empty(_abi.LUT_N)
    assert lib.so3g_get_trig_tables(a.ctypes.data, b.ctypes.data, _abi.LUT_N) == 0
    assert a[0] == 0.0 and abs(a[-1] - np.pi / 2) < 1e-15
    assert abs(b[-1] - np.pi / 4) < 1e-15
    assert lib.so3g_get_trig_tables(a.ctypes.data, b.ctypes.data, 7) == -1
    assert "table size" in _abi.last_error()
    assert lib.so3g_launch_count() >= 0


def test_chunked_threshold_setter_without_gpu(lib):
    """so3g_set_chunked_min_samples stores the threshold and returns the
    previous one (3e7 at load); negative values count as 0."""
    import so3g_gb300
    old = so3g_gb300.set_chunked_min_samples(12345)
    try:
        assert old >= 0
        assert so3g_gb300.set_chunked_min_samples(-5) == 12345
        assert so3g_gb300.set_chunked_min_samples(1 << 40) == 0
        assert lib.so3g_set_chunked_min_samples(old) == 1 << 40
    finally:
        so3g_gb300.set_chunked_min_samples(old)


def test_struct_layout_matches_header(tmp_path):
    from so3g_gb300 import _abi
    import ctypes
    structs = {"so3g_pixelization": _abi.Pixelization, "so3g_map": _abi.Map,
               "so3g_ranges": _abi.Ranges, "so3g_precomp_geom": _abi.PrecompGeom, "so3g_obs": _abi.Obs,
               "so3g_sightline": _abi.SightLine}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "so3g_gb300.h"',
             'int main(void) {']
    for cname, py in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for ln in out.splitlines():
        name, field, val = ln.split()
        got[(name, field)] = int(val)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_new_entry_points_validate_arguments(lib):
    """so3g_boresight, so3g_quat_left_multiply and the mask-segment entry
    points reject bad arguments before any device work (no GPU needed)."""
    import ctypes
    import numpy as np
    from so3g_gb300 import _abi
    sl = _abi.SightLine()
    sl.kind = 7
    assert lib.so3g_boresight(ctypes.byref(sl), None, None, None, None, 10, None, None) == -1
    assert "sight-line kind" in _abi.last_error()
    sl.kind = _abi.SIGHT_NAIVE_AZEL
    buf = np.zeros(64)
    p = buf.ctypes.data
    # naive az/el needs the times
    assert lib.so3g_boresight(ctypes.byref(sl), None, p, p, None, 4, p, None) == -1
    assert "NULL" in _abi.last_error()
    assert lib.so3g_boresight(ctypes.byref(sl), p, p, p, None, -1, p, None) == -1
    assert lib.so3g_boresight(ctypes.byref(sl), None, None, None, None, 0, None, None) == 0
    # output not 16-byte aligned
    assert lib.so3g_boresight(ctypes.byref(sl), p, p, p, None, 4, p + 8, None) == -1
    assert "aligned" in _abi.last_error()
    assert lib.so3g_quat_left_multiply(p, p, 4, p + 8, None) == -1
    assert lib.so3g_quat_left_multiply(None, p, 4, p, None) == -1
    assert lib.so3g_quat_left_multiply(p, p, 0, p, None) == 0
    cnt = np.zeros(4, np.int32)
    assert lib.so3g_mask_count_segments(p, -1, 10, 10, cnt.ctypes.data, None) == -1
    assert lib.so3g_mask_count_segments(p, 4, 10, 5, cnt.ctypes.data, None) == -1
    assert "det_stride" in _abi.last_error()
    assert lib.so3g_mask_count_segments(p, 0, 10, 10, cnt.ctypes.data, None) == 0
    assert lib.so3g_mask_fill_segments(p, 4, 10, 10, None, None, None, None, None) == -1
    assert lib.so3g_mask_fill_segments(p, 4, 0, 10, None, None, None, None, None) == 0
