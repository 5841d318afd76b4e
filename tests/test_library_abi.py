"""The C-ABI library loads and exports every symbol its headers declare
(no GPU needed: nothing here launches a kernel)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import cubens

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "sizeof", "return")))


@pytest.fixture(scope="module")
def lib():
    cubens.build.build()
    return cubens.load()


def test_headers_declare_functions():
    names = declared_functions()
    assert "cb_model_create" in names and "cb_msal_step" in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_parse_errors_need_no_gpu(lib):
    opt = cubens.Options()
    lib.cb_default_options(C.byref(opt))
    h = C.c_void_p()
    bad = b"2\n1\n0\n1\n2\n1,0,0,0,0\n"
    rc = lib.cb_model_create(bad, len(bad), C.byref(opt), C.byref(h))
    assert rc in (2, 4)
    assert lib.cb_last_error(h)
    lib.cb_model_destroy(h)
