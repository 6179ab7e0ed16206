"""The C ABI library loads and exports every symbol include/kvgpu.h declares
(no GPU needed: no compute call is made), and the oracle's C API loads."""
import ctypes
import os
import re

import kvtest_util as U

U.load_package()


def _declared():
    with open(os.path.join(U.ROOT, "include", "kvgpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(kv_\w+)\s*\(", txt, re.M)))


def test_library_exports_all_declared_symbols():
    import __graft_entry__ as ge  # noqa: F401
    from kylin_v_gb300 import build, kvgpu

    build.build()
    L = ctypes.CDLL(kvgpu.LIB_PATH)
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(kvgpu.EXPORTS) | set(names)
    assert L.kv_version() == 1


def test_calls_before_init_fail_cleanly():
    from kylin_v_gb300 import kvgpu

    L = kvgpu.lib()
    out = ctypes.c_void_p()
    dirs = (ctypes.c_int * 3)(1, 1, -1)
    rc = L.kv_tensor_create(3, dirs, 0, None, None, None, ctypes.byref(out))
    assert rc == -6  # KV_ENOTINIT
    assert b"kv_init" in L.kv_last_error()


def test_oracle_library_loads():
    O = U.load_oracle()
    assert O.lib() is not None
