"""The C-ABI library loads and exports every function include/radgpu.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "radgpu.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"RAD_API\s+int\s+(rad_\w+)\s*\(", text)))


def test_header_lists_match_binding():
    from radiantiumplusplus_gb300 import _capi
    assert sorted(_capi.EXPORTS) == _declared()


def test_library_exports_every_symbol():
    from radiantiumplusplus_gb300 import _capi
    if not os.path.exists(_capi.LIB_PATH):
        import radiantiumplusplus_gb300.build as b
        b.build()
    lib = ctypes.CDLL(_capi.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name


def test_no_device_is_a_status_not_a_crash():
    """Without a GPU, rad_init reports RAD_ERR_NO_DEVICE (or succeeds on a GPU machine)."""
    import radiantiumplusplus_gb300 as rad
    st = rad.lib().rad_init(None)
    assert st in (0, 11)
