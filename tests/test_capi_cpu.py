"""CPU-only checks of the C ABI: the library loads, exports every declared
symbol, agrees with the ctypes struct layouts and fills the same defaults."""
import ctypes

import pytest

from libfluid_gb300 import capi


@pytest.fixture(scope="module")
def lib():
    from libfluid_gb300 import build
    build.build()
    return capi.load()


def test_exports_every_declared_symbol(lib):
    names = capi.exported_symbols()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_ctypes(lib):
    out = (ctypes.c_uint64 * 32)()
    m = lib.fgb_struct_sizes(out, 32)
    ours = [capi.Params, capi.Config, capi.Particles, capi.Triangle, capi.MeshTriangle, capi.Mesh,
            capi.GridInfo, capi.Well, capi.ServeOptions, capi.ServeResult, capi.ServeStats, capi.TuneResult,
            capi.Source, capi.Drain, capi.Query, capi.QueryResult, capi.Records]
    assert m == len(ours)
    for i, t in enumerate(ours):
        assert out[i] == ctypes.sizeof(t), (t.__name__, out[i], ctypes.sizeof(t))


@pytest.mark.parametrize("profile", [capi.PROFILE_REF, capi.PROFILE_BASELINE])
def test_param_defaults_match_python(lib, profile):
    a = capi.params(profile, 0.1)
    b = capi.default_params(profile, 0.1)
    for name, _ in capi.Params._fields_:
        assert getattr(a, name) == pytest.approx(getattr(b, name), rel=0, abs=0), name


def test_version_and_no_error(lib):
    assert lib.fgb_version() == 1
    assert lib.fgb_last_error() == b""


def test_invalid_arguments_fail_without_a_gpu(lib):
    assert lib.fgb_create(None, None) == capi.FGB_ERR_INVALID
    assert b"null" in lib.fgb_last_error()
    p = capi.default_params(capi.PROFILE_BASELINE, -1.0)
    h = ctypes.c_void_p()
    assert lib.fgb_create(ctypes.byref(p), ctypes.byref(h)) == capi.FGB_ERR_INVALID
    assert lib.fgb_radix_sort_pairs_u32(None, None, None, None, 10, 8, None, 0, None) == capi.FGB_ERR_INVALID


def test_header_constants_match_python():
    """Every FGB_* integer #define of the header that capi.py mirrors (error codes,
    profiles, particle types, probes, serving states, wire tags) has the same value."""
    import os
    import re
    hdr = open(os.path.join(os.path.dirname(capi.__file__), "..", "include", "fluid_gb300.h")).read()
    defines = {m.group(1): int(m.group(2), 0)
               for m in re.finditer(r"#define\s+FGB_(\w+)\s+(0x[0-9a-fA-F]+|\d+)\b", hdr)}
    checked = 0
    for name, value in defines.items():
        for py in (name, "FGB_" + name):
            if hasattr(capi, py) and isinstance(getattr(capi, py), int):
                assert getattr(capi, py) == value, name
                checked += 1
                break
    assert checked >= 15
