"""results*.txt writers against the reference's own files (output(),
misc.c:345-451): the same layout byte for byte (headers, tabs, record
lines with the same iteration counts) and the same values to the printed
precision (%e, 7 digits)."""
import re
import numpy as np
import pytest

import cubens

pytestmark = pytest.mark.gpu

NUM = re.compile(r"-?\d\.\d{6}e[+-]\d{2,3}")


def _skeleton(t: str) -> str:
    return NUM.sub("N", t)


def _values(t: str) -> np.ndarray:
    return np.array([float(x) for x in NUM.findall(t)])


def _run(name, text, steps, out_dir):
    m = cubens.Model(text, precision=cubens.FP64)
    m.results_open(out_dir)
    try:
        _steps(m, steps)
    finally:
        m.results_close()


def _steps(m, steps):
    alg = m.info["algflag"]
    if alg == 3:
        r = m.begin()
        m.results_write(r.lam, r.iterations)
        for _ in range(steps - 1):
            r = m.step()
            m.results_write(r.lam, r.iterations)
    elif alg == 5:
        m.newmark_begin()
        for _ in range(steps):
            r = m.newmark_step()
            m.results_write(r.lam, r.iterations)
    else:
        m.newton_begin()
        for _ in range(steps):
            r = m.newton_step()
            if r.done:
                break
            m.results_write(r.lam, r.iterations)


def test_results_files_match_the_reference(golden_dir, tmp_path):
    z = np.load(golden_dir / "results_files.npz")
    for name, text, files, steps in zip(z["names"], z["model_def"], z["files"], z["steps"]):
        d = tmp_path / str(name)
        d.mkdir()
        _run(str(name), str(text), int(steps), d)
        for k, ref in zip(range(2, 6), files):
            ours = (d / f"results{k}.txt").read_text()
            ref = str(ref)
            assert _skeleton(ours) == _skeleton(ref), (name, k)
            a, b = _values(ours), _values(ref)
            assert a.shape == b.shape, (name, k)
            if b.size:
                scale = np.max(np.abs(b))
                assert np.max(np.abs(a - b)) <= 2e-6 * scale + 1e-300, (name, k)


def test_results1_matches_the_reference(golden_dir, tmp_path):
    """results1.txt byte for byte: the input echo, then the run's messages
    (the closing "Solution successful" of the Newton-Raphson run, the error
    and "Solution failed" of an arc-length run whose first increment does not
    converge; the capped runs end after the echo, as the reference's do)."""
    z = np.load(golden_dir / "results1_files.npz")
    for name, text, ref, steps in zip(z["names"], z["model_def"], z["results1"], z["steps"]):
        d = tmp_path / str(name)
        d.mkdir()
        try:
            _run(str(name), str(text), int(steps), d)
        except cubens.CubensError:
            assert str(name) == "panel8_too_large"
        ours = (d / "results1.txt").read_text()
        assert ours == str(ref), (name, ours[-200:], str(ref)[-200:])
