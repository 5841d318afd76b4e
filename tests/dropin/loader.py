"""Loads the drop-in library behind a shim that defines CU-BENs' globals.

The drop-in library binds NJ, NEQ, ... weakly at load time, so the shim
(tests/dropin/globals.c, compiled here with the host C compiler) is loaded
with RTLD_GLOBAL first. Test infrastructure only.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import tempfile
from pathlib import Path

import cubens

HERE = Path(__file__).resolve().parent
_libs = None


def load():
    global _libs
    if _libs is not None:
        return _libs
    out = Path(tempfile.mkdtemp(prefix="cbg_")) / "libcbglobals.so"
    subprocess.run(["gcc", "-shared", "-fPIC", "-O2", "-o", str(out), str(HERE / "globals.c")], check=True)
    g = C.CDLL(str(out), mode=C.RTLD_GLOBAL)
    g.cbg_set.argtypes = [C.c_long] * 5 + [C.c_int, C.c_int, C.c_double]
    cubens.build.build()
    d = C.CDLL(str(cubens.build.DROPIN_LIB), mode=C.RTLD_GLOBAL)
    d.dot.restype = C.c_double
    d.dot.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    _libs = (g, d)
    return _libs
