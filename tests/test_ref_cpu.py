"""The oracle against the reference program itself, built for the CPU from
the reference sources (oracle/ref_cpu/build_ref.sh), on fresh seeds.  Runs
only where the reference sources are present."""
import shutil
import tempfile

import pytest

import oracle
import runs

pytestmark = pytest.mark.skipif(not oracle.reference_available(),
                                reason="reference sources not present")

CASES = [
    dict(L=8, nr=32, nbits=1, nc=2, nterm=5, maxtime=24, times=[3, 7, 24], seed_J=77, seed_u=78,
         seed_MC0=79, isample=3),
    dict(L=16, nr=32, nbits=1, nc=4, nterm=0, maxtime=12, times=[1, 6, 12], seed_J=8, seed_u=9,
         seed_MC0=10, list_samples=[1]),
    dict(L=8, nr=64, nbits=2, nc=6, nterm=1, maxtime=9, times=[2, 9], seed_J=13, seed_u=14,
         seed_MC0=15, isample=1234),
]


@pytest.mark.parametrize("cfg", CASES)
def test_oracle_equals_reference_program(cfg):
    exe = oracle.build_reference(cfg["L"], cfg["nr"])
    work = tempfile.mkdtemp(prefix="micsa_ref_")
    try:
        want, _ = runs.run_program(exe, cfg, work, exit_race_ok=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    got = runs.oracle_run(cfg)
    runs.compare(got, want, cfg)
