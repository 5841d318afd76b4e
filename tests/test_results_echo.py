"""results1.txt's input echo against the reference's own files, byte for
byte, without a GPU: cb_input_echo parses the model_def and writes what the
reference writes while it reads it (main.c:383-433, 1035, 1357, 1392-1414,
struc model.c:314-391, prop_tr/prop_fr/prop_sh, load model.c:1316-1319,
arc.c:52-53). The rest of each file is the run's messages, which the GPU
tests check."""
import numpy as np
import pytest

import cubens


@pytest.fixture(scope="module")
def lib():
    cubens.build.build()
    return cubens.load()


def test_input_echo_matches_the_reference_results1(golden_dir, lib):
    z = np.load(golden_dir / "results1_files.npz")
    for name, text, ref in zip(z["names"], z["model_def"], z["results1"]):
        echo = cubens.input_echo(str(text))
        ref = str(ref)
        assert ref.startswith(echo), name
        rest = ref[len(echo):]
        # what follows is a message line or nothing (capped runs)
        assert rest == "" or rest.startswith("\n"), (name, rest[:80])


def test_input_echo_reports_parse_errors(lib):
    with pytest.raises(cubens.CubensError):
        cubens.input_echo("2\n3\n0\n1\n")
