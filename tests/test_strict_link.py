"""Strict mode: the reference's own driver (main.c and the other units,
unmodified, compiled from the reference tree by `make -C oracle ref`) with
every hot-path call forwarded to libcubens_dropin.so by link-time wrapping
(oracle/refshim/gpu_forward.c). The binary exists only where the reference
tree was present at build time; elsewhere the test is skipped.

Without a GPU the library reports the missing device at each forwarded
call, which shows that main.c's calls reach it; with one, the run is the
reference's own MSAL loop on the GPU routines and must follow the
reference's path (1e-6, the FP64 tolerance)."""
import os
from pathlib import Path

import numpy as np
import pytest

import cubens

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "oracle" / "_ref" / "cuben_gpu"


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_reference_driver_runs_on_the_dropin_library(golden_dir, monkeypatch):
    if not BIN.exists():
        pytest.skip("the reference tree was not present at build time")
    import refrun
    cubens.build.build()
    monkeypatch.setenv("CUBENS_DROPIN", str(cubens.build.DROPIN_LIB))
    z = np.load(golden_dir / "run_truss_c1.npz")
    r = refrun.run(str(z["model_def"]), 3, timeout=120, binary=BIN)
    if not _gpu_present():
        called = {l.split(":")[0].split()[-1] for l in r["stderr"].splitlines() if l.startswith("cubens ")}
        assert {"updatc", "stiff_tr", "forces_tr", "test", "dot"} <= called, called
        return
    assert r["returncode"] == 0
    np.testing.assert_array_equal(r["iterations"], z["iterations"][:3])
    assert np.max(np.abs(r["lam"] - z["lam"][:3]) / np.abs(z["lam"][:3])) < 1e-6
