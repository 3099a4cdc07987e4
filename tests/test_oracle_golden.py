"""The oracle (with the product's host initialisation) against golden outputs
of the reference program itself (tests/golden/, made by make_golden.py).

Every fixture pins, bit for bit: the three evol_*.txt files, seeds.in,
master_seedJ.in, conf_Js, every conf.<t> record (spins, energies and
generator states) and the final walkers file (demon words + stream states).
"""
import pytest

import runs
from conftest import golden_cases


@pytest.mark.parametrize("golden", golden_cases(max_volume=64 ** 3 * 64))
def test_oracle_reproduces_reference(golden):
    got = runs.oracle_run(golden["cfg"])
    keys = runs.compare(got, golden, golden["cfg"])
    assert len(keys) >= 4


def test_lut_builder_matches_reference_lut():
    """The LUT builder (preparation.c:265-388) reproduces the shipped
    LUT_for_PRNG_nbits10_NB1.bin: its digest is recorded in every fixture."""
    import glob
    import json
    import os
    digests = {json.load(open(f))["lut_sha256"]
               for f in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.json"))}
    assert digests == {runs.sha(runs.lut_bytes())}
    assert runs.sha(runs.lut_bytes()) == \
        "cb173404721c37dafad735670c2abb94bd23d31af55b3ff1abf4cf48b4c84ed0"
