"""Run the reference's own driver binary (oracle/_ref/cuben_ref, built by
``make -C oracle ref``) on a model_def text and read back its FP64 step dump.

Test infrastructure only: the golden-fixture script and the CPU timing of the
reference use it; nothing in the product imports it. The reference opens its
input with a busy-wait loop (main.c:335-337), so every run has a timeout.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_BIN = HERE / "_ref" / "cuben_ref"


def available(binary: Path = REF_BIN) -> bool:
    return binary.exists()


def read_dump(path: Path, neq: int):
    """Parse the shim_output.c dump: (steps, iterations, lambdas, d[steps, neq])."""
    raw = path.read_bytes()
    rec = 8 + 8 + 8 * neq
    n = len(raw) // rec
    steps, its, lam, d = [], [], [], []
    for k in range(n):
        b = raw[k * rec:(k + 1) * rec]
        s, it = np.frombuffer(b[:8], dtype=np.int32)
        steps.append(int(s))
        its.append(int(it))
        lam.append(float(np.frombuffer(b[8:16], dtype=np.float64)[0]))
        d.append(np.frombuffer(b[16:], dtype=np.float64).copy())
    return (np.array(steps), np.array(its), np.array(lam),
            np.array(d) if d else np.zeros((0, neq)))


def neq_from_results(workdir: Path) -> int:
    for line in (workdir / "results1.txt").read_text().splitlines():
        if "Number of equations" in line:
            return int(line.split(":")[1])
    raise RuntimeError("NEQ not found in results1.txt")


def run(model_text: str, cap_steps: int, timeout: float = 600.0,
        binary: Path = REF_BIN, testlog: bool = False):
    """Run the reference on ``model_text`` for ``cap_steps`` converged steps.

    Returns dict(neq, steps, iterations, lam, d, seconds, step_times, testlog).
    """
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "model_def.txt").write_text(model_text)
        env = dict(os.environ, CAP_STEPS=str(cap_steps), CUBEN_DUMP=str(wd / "dump.bin"),
                   CUBEN_TIMES="1")
        if testlog:
            env["CUBEN_TESTLOG"] = str(wd / "test.bin")
        t0 = time.perf_counter()
        proc = subprocess.run([str(binary)], cwd=wd, env=env, capture_output=True,
                              text=True, timeout=timeout)
        secs = time.perf_counter() - t0
        neq = neq_from_results(wd)
        steps, its, lam, d = read_dump(wd / "dump.bin", neq) if (wd / "dump.bin").exists() \
            else (np.zeros(0), np.zeros(0), np.zeros(0), np.zeros((0, neq)))
        times = [float(l.split(" t ")[1]) for l in proc.stderr.splitlines() if l.startswith("step ")]
        log = None
        if testlog and (wd / "test.bin").exists():
            rawl = np.fromfile(wd / "test.bin", dtype=np.uint8)
            recs = rawl.reshape(-1, 48)
            vals = recs[:, :40].copy().view(np.float64).reshape(-1, 5)
            cc = recs[:, 40:48].copy().view(np.int32).reshape(-1, 2)
            log = (vals, cc)
        errors = (wd / "results1.txt").read_text()
        files = {k: (wd / f"results{k}.txt").read_text() for k in range(2, 6) if (wd / f"results{k}.txt").exists()}
        return dict(neq=neq, steps=steps, iterations=its, lam=lam, d=d, seconds=secs,
                    step_times=np.array(times), testlog=log, returncode=proc.returncode,
                    stdout=proc.stdout, stderr=proc.stderr, results1=errors, results=files)
