"""CPU checks of the C ABI: libfsg.so builds, loads and exports every symbol
that include/*.h declares; the ctypes signatures cover the same set.  No
compute calls (no GPU here)."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(fsg_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def built_lib():
    from fujishadergpu_gb300 import build
    try:
        return build.build()
    except RuntimeError as e:  # nvcc missing
        pytest.skip(str(e))


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    lib = ctypes.CDLL(built_lib)
    names = declared_symbols()
    assert names, "no fsg_* declarations found"
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(built_lib):
    from fujishadergpu_gb300 import _native
    assert set(_native.exported_symbols()) == declared_symbols()
    L = _native.lib()
    assert L.fsg_abi_version() == 1
    assert b"sm_103a" in L.fsg_version()


STRUCTS = {"fsg_plane": "Plane", "fsg_tile": "Tile", "fsg_stencil_params": "StencilParams",
           "fsg_topousm_params": "TopoUSMParams", "fsg_openness_params": "OpennessParams"}


def test_struct_layouts_match_header(tmp_path):
    """Compile a C probe against include/fsg.h and compare sizeof/offsetof with ctypes."""
    import ctypes
    import shutil
    import subprocess
    from fujishadergpu_gb300 import _native as N
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fsg.h"', "int main(void){"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in getattr(N, pyname)._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line.strip():
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(N, pyname)
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


@pytest.mark.parametrize("ndir", [4, 8, 12, 16, 24, 32, 36])
@pytest.mark.parametrize("dist", [1, 5, 40, 50, 256, 300])
def test_openness_ray_offsets_match_numpy(built_lib, ndir, dist):
    """Host-only table: Python banker's rounding of r*cos/sin of np.linspace angles."""
    import ctypes as C
    import numpy as np
    from fujishadergpu_gb300 import _native as N
    from oracle import restated as R
    for mode, rays in ((0, R.openness_offsets(ndir, dist)), (1, R.dense_offsets(ndir, dist))):
        cap = sum(len(r) for r in rays)
        ox = (C.c_int32 * max(1, cap))()
        oy = (C.c_int32 * max(1, cap))()
        rl = (C.c_int32 * ndir)()
        assert N.lib().fsg_openness_offsets(ndir, dist, mode, ox, oy, rl, cap) == 0
        k = 0
        for d, ray in enumerate(rays):
            assert rl[d] == len(ray), (mode, d)
            for (x, y) in ray:
                assert (ox[k], oy[k]) == (x, y), (mode, d, k)
                k += 1


@pytest.mark.parametrize("dtype,qmin,qmax", [("uint8", 0, 300), ("uint8", -1, 255), ("int16", -40000, 32767),
                                             ("int16", -32768, 40000)])
def test_stencil_rejects_code_ranges_outside_the_type(built_lib, dtype, qmin, qmax):
    """Integer planes store codes clamped to [q_min, q_max]: a range outside the type is
    rejected (FSG_ERR_INVALID) before the call touches the device, so the call returns
    without reading its pointers (placeholders here)."""
    import ctypes as C
    from fujishadergpu_gb300 import _native as N
    from fujishadergpu_gb300.algorithms import _stencil as S
    planes = (N.Plane * N.FSG_STENCIL_NOUT)()
    planes[0].ptr = 0x100000
    planes[0].ld = 64
    planes[0].dtype = N.DTYPE_CODES[dtype]
    planes[0].q_a, planes[0].q_b, planes[0].q_min, planes[0].q_max = 1.0, 0.0, qmin, qmax
    tiles = (N.Tile * 1)(S.whole_window_tile(64, 64, 1.0, -1.0))
    params = S.make_params(pixel_size=1.0)
    st = N.lib().fsg_stencil(C.c_void_p(0x200000), 64, 64, 64, tiles, 1, C.byref(params), planes, None)
    assert st == -1, st
    assert b"code range" in N.lib().fsg_last_error()
