"""The C-ABI library without a GPU: it loads, exports every symbol the headers declare, and answers the calls that
need no device with the reference's status conventions."""
import ctypes as C
import re
from pathlib import Path

import pytest

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def _declared_functions():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:void|int|const char \*)\s+(opensps_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    declared = _declared_functions()
    assert len(declared) >= 30
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_headers(built_lib):
    from libopensps_gb300 import capi
    assert _declared_functions() == set(capi.SIGNATURES)


def test_host_only_calls(built_lib):
    from libopensps_gb300 import capi
    lib = capi.load_library()
    nb = C.c_int(0)
    lib.opensps_get_nbgrad(C.byref(nb))
    assert nb.value == 44
    buf, st = C.create_string_buffer(32), C.c_int(-1)
    lib.opensps_get_grad_param_name(22, buf, 32, C.byref(st))
    assert st.value == 0 and buf.value == b"zred"
    lib.opensps_get_grad_param_name(44, buf, 32, C.byref(st))
    assert st.value == 3
    # a bad handle is status 1, never an abort
    st = C.c_int(0)
    lib.opensps_context_destroy(9999, C.byref(st))
    assert st.value == 1
    ns = C.c_int(0)
    lib.opensps_context_get_nspec(9999, C.byref(ns), C.byref(st))
    assert st.value == 1
    # a context that is not set up is status 301
    h = C.c_int(0)
    lib.opensps_context_create(C.byref(h), C.byref(st))
    assert st.value == 0 and h.value >= 1
    lib.opensps_context_get_nspec(h.value, C.byref(ns), C.byref(st))
    assert st.value == 301
    lib.opensps_context_set_int(h.value, b"no_such_setting", 1, C.byref(st))
    assert st.value == 101
    lib.opensps_context_set_float(h.value, b"dust2", 0.5, C.byref(st))
    assert st.value == 0
    # the tabular SFH (host only): ntab out of range and decreasing ages are status 3
    import numpy as np
    age, sfr = np.array([0.0, 1.0, 2.0]), np.array([1.0, 2.0, 1.0])
    dp = C.POINTER(C.c_double)
    lib.opensps_context_set_sfh_tab(h.value, 3, age.ctypes.data_as(dp), sfr.ctypes.data_as(dp), None, C.byref(st))
    assert st.value == 0
    lib.opensps_context_set_sfh_tab(h.value, 0, age.ctypes.data_as(dp), sfr.ctypes.data_as(dp), None, C.byref(st))
    assert st.value == 3
    back = age[::-1].copy()
    lib.opensps_context_set_sfh_tab(h.value, 3, back.ctypes.data_as(dp), sfr.ctypes.data_as(dp), None, C.byref(st))
    assert st.value == 3
    lib.opensps_context_set_sfh_tab(9999, 3, age.ctypes.data_as(dp), sfr.ctypes.data_as(dp), None, C.byref(st))
    assert st.value == 1
    lib.opensps_context_set_str(h.value, b"sfh_filename", b"my_sfh.dat", C.byref(st))
    assert st.value == 0
    lib.opensps_context_destroy(h.value, C.byref(st))
    assert st.value == 0


def test_setup_without_a_gpu_reports_a_status(built_lib, data):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from libopensps_gb300 import capi
    lib = capi.load_library()
    h, st = C.c_int(0), C.c_int(0)
    lib.opensps_context_create(C.byref(h), C.byref(st))
    lib.opensps_context_setup(-1, b"synthetic", b"synthetic", b"none", h.value, C.byref(st))
    assert st.value == 4
    msg, s2 = C.create_string_buffer(256), C.c_int(0)
    lib.opensps_get_last_error(C.byref(s2), msg, 256)
    assert s2.value == 4 and b"CUDA" in msg.value
    lib.opensps_context_destroy(h.value, C.byref(st))
