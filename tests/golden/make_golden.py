"""Generate the golden fixtures of tests/golden/ from the reference itself.

Each case runs the reference program (IsidoroGlez/micSA-EA-MC PROGRAM/),
compiled for the CPU by oracle/ref_cpu/build_ref.sh, on seeded inputs and
stores what it wrote: the three evol_*.txt files verbatim, seeds.in and
master_seedJ.in verbatim, and SHA-256 digests of conf_Js, of every conf.<t>
record (spins, energies, generator states) and of the final walkers file.

Needs the reference sources, named by MICSA_REFERENCE_DIR; run from the
repository root:

    MICSA_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py [case ...]
"""
import json
import os
import shutil
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import runs  # noqa: E402
import oracle  # noqa: E402  (path set up by runs)

# Seeded runs.  Seeds are arbitrary non-zero values (a zero seed would read
# /dev/urandom).  "times" are the measurement times (input list_times).
CASES = {
    "L8_NR32_nc6": dict(L=8, nr=32, nbits=1, nc=6, nterm=0, maxtime=64,
                        times=[1, 2, 3, 4, 8, 16, 32, 64], seed_J=1234567, seed_u=7654321,
                        seed_MC0=0x5EED0000),
    "L8_NR64_2s_nc3_therm": dict(L=8, nr=64, nbits=2, nc=3, nterm=3, maxtime=40,
                                 times=[1, 2, 5, 8, 16, 40], seed_J=99, seed_u=31337,
                                 seed_MC0=0xC0FFEE00),
    "L16_NR32_nc6_therm": dict(L=16, nr=32, nbits=1, nc=6, nterm=2, maxtime=256,
                               times=[1, 2, 4, 16, 64, 100, 256], seed_J=20260101,
                               seed_u=424242, seed_MC0=0x5EED0000),
    "L24_NR32_2s_nc5": dict(L=24, nr=32, nbits=2, nc=5, nterm=1, maxtime=33,
                            times=[1, 3, 8, 33], seed_J=5, seed_u=6, seed_MC0=7),
    "L16_NR64_2s_nc6": dict(L=16, nr=64, nbits=2, nc=6, nterm=0, maxtime=128,
                            times=[1, 2, 4, 8, 16, 32, 64, 128], seed_J=11, seed_u=12,
                            seed_MC0=0xABCDEF00),
    "L32_NR32_nc1": dict(L=32, nr=32, nbits=1, nc=1, nterm=0, maxtime=20,
                         times=[1, 5, 20], seed_J=3, seed_u=4, seed_MC0=0x1000),
    # headline shape: L=160, 2 samples x 64 replicas, 6 demons per site
    "L160_NR64_2s_nc6": dict(L=160, nr=64, nbits=2, nc=6, nterm=0, maxtime=2, times=[1, 2],
                             seed_J=20260101, seed_u=1729, seed_MC0=0x5EED0000),
}


def make(name, cfg):
    exe = oracle.build_reference(cfg["L"], cfg["nr"])
    if exe is None:
        raise SystemExit("reference sources not available; cannot generate fixtures")
    work = tempfile.mkdtemp(prefix="micsa_golden_")
    try:
        t0 = time.time()
        summary, _ = runs.run_program(exe, cfg, work, exit_race_ok=True)
        summary["cfg"] = cfg
        summary["generated_by"] = "reference program built for the CPU (oracle/ref_cpu/build_ref.sh)"
        summary["lut_sha256"] = runs.sha(open(os.path.join(work, "lut.bin"), "rb").read())
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(summary, f, indent=1, sort_keys=True)
        print("%-24s %.1fs" % (name, time.time() - t0))
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make(n, CASES[n])
