"""The C-ABI library loads and exports every symbol its headers declare
(no GPU needed: nothing here launches a kernel)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import cubens

ROOT = Path(__file__).resolve().parents[1]


def declared_functions(header: str = "cubens_gb300.h"):
    names = []
    for h in [ROOT / "include" / header]:
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


def test_dropin_library_exports_the_prototypes_symbols():
    from dropin import loader
    _, d = loader.load()
    names = declared_functions("cubens_gb300_dropin.h")
    assert {"forces_sh", "stiff_sh", "forces_fr", "updatc", "solve", "skyfact", "quad", "test"} <= set(names)
    missing = [n for n in names if not hasattr(d, n)]
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


def _create(lib, text: bytes):
    opt = cubens.Options()
    lib.cb_default_options(C.byref(opt))
    h = C.c_void_p()
    rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
    msg = lib.cb_last_error(h).decode()
    lib.cb_model_destroy(h)
    return rc, msg


def test_unsupported_frame_and_newmark_inputs_are_refused_before_upload(lib):
    from cubens import models
    spec = models.frame_building(1, 1, 1, steps=4)
    lines = spec.text.splitlines()
    # member end offsets (frame.c:85-108) are outside the GPU path
    i = lines.index("0,0,0,0,0,0,0")
    bad = "\n".join(lines[:i] + ["1,0.1,0,0,0,0,0", "0,0,0,0,0,0,0"] + lines[i + 1:]) + "\n"
    rc, msg = _create(lib, bad.encode())
    assert rc == 4 and "offsets" in msg
    # prescribed support motion in a Newmark model
    j = lines.index("0,0", 7 + spec.ne_fr) + 1  # the list after the constraints
    bad = "\n".join(lines[:j] + ["2,1", "0,0"] + lines[j + 1:]) + "\n"
    rc, msg = _create(lib, bad.encode())
    assert rc == 4 and "prescribed" in msg
    # a Newmark model with truss elements
    truss = models.space_truss(bays=2).text.splitlines()
    truss[1] = "5"
    truss.insert(2, "0,0")
    rc, msg = _create(lib, ("\n".join(truss) + "\n").encode())
    assert rc == 4 and "frame-only" in msg


def test_fgmres_is_accepted_for_msal_models_and_bad_solvers_refused(lib):
    """The arc-length loop runs on FGMRES too (det and psi from substitutes
    for the factor's pivots): the create call gets as far as the device
    check. The double-word band factor has no Krylov form and is refused
    with FGMRES before any upload, as is an unknown solver code."""
    from cubens import models
    text = models.space_truss(bays=2).text.encode()
    opt = cubens.Options()
    lib.cb_default_options(C.byref(opt))
    opt.solver = cubens.SOLVER_FGMRES
    h = C.c_void_p()
    rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
    msg = lib.cb_last_error(h).decode()
    lib.cb_model_destroy(h)
    assert rc in (0, 3), (rc, msg)  # 3: no CUDA device here
    opt.precision = cubens.FP32X2
    h = C.c_void_p()
    rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
    msg = lib.cb_last_error(h).decode()
    lib.cb_model_destroy(h)
    assert rc == 4 and "FGMRES" in msg, (rc, msg)
    opt.precision = cubens.FP64
    opt.solver = 7
    h = C.c_void_p()
    rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
    lib.cb_model_destroy(h)
    assert rc == 1


def test_newton_raphson_models_parse_and_fgmres_is_refused_for_them(lib):
    """ALGFLAG 1 and 2 (static load control) pass the parser: without a GPU
    the create call gets as far as the device check. FGMRES is refused for
    them before any upload."""
    from cubens import models
    for alg in (1, 2):
        text = models.space_truss(controls=models.NewtonControls(alg=alg)).text.encode()
        opt = cubens.Options()
        lib.cb_default_options(C.byref(opt))
        h = C.c_void_p()
        rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
        msg = lib.cb_last_error(h).decode()
        lib.cb_model_destroy(h)
        assert rc in (0, 3), (rc, msg)  # 3: no CUDA device here
        opt.solver = cubens.SOLVER_FGMRES
        h = C.c_void_p()
        rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
        lib.cb_model_destroy(h)
        assert rc == 4


def test_linear_newmark_models_take_the_fp64_band_only(lib):
    """ALGFLAG 4 (ANAFLAG 1) parses; it factors its effective stiffness once
    with the FP64 band, so FGMRES and the other precisions are refused before
    any upload."""
    from cubens import models
    text = models.frame_building(2, 2, 3, steps=10, dt=0.005, seed=3, linear=True).text.encode()
    opt = cubens.Options()
    lib.cb_default_options(C.byref(opt))
    h = C.c_void_p()
    rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
    msg = lib.cb_last_error(h).decode()
    lib.cb_model_destroy(h)
    assert rc in (0, 3), (rc, msg)  # 3: no CUDA device here
    for solver, precision in ((cubens.SOLVER_FGMRES, cubens.FP64), (cubens.SOLVER_BAND, cubens.MIXED)):
        opt.solver, opt.precision = solver, precision
        h = C.c_void_p()
        rc = lib.cb_model_create(text, len(text), C.byref(opt), C.byref(h))
        msg = lib.cb_last_error(h).decode()
        lib.cb_model_destroy(h)
        assert rc == 4 and "linear Newmark" in msg, (rc, msg)
    # the DKT panel with its lumped shell mass parses too
    panel = models.shell_panel_linear(8, steps=10).text.encode()
    opt.solver, opt.precision = cubens.SOLVER_BAND, cubens.FP64
    h = C.c_void_p()
    rc = lib.cb_model_create(panel, len(panel), C.byref(opt), C.byref(h))
    msg = lib.cb_last_error(h).decode()
    lib.cb_model_destroy(h)
    assert rc in (0, 3), (rc, msg)
    # ALGFLAG 4 with ANAFLAG 2 is not an analysis the reference runs (main.c:393)
    bad = b"2" + text[1:]
    h = C.c_void_p()
    opt.solver, opt.precision = cubens.SOLVER_BAND, cubens.FP64
    rc = lib.cb_model_create(bad, len(bad), C.byref(opt), C.byref(h))
    lib.cb_model_destroy(h)
    assert rc == 4
