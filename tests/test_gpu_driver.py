"""micsa_run, the command-line drop-in, against the reference program's own
outputs: same argv and input files, byte-identical measurement files, seed
files, conf.<t> records and walkers files."""
import os
import shutil
import tempfile

import pytest

import micsa
import runs
from conftest import golden_cases

pytestmark = pytest.mark.gpu


@pytest.fixture
def workdir():
    d = tempfile.mkdtemp(prefix="micsa_drv_")
    yield d
    shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("golden", golden_cases())
def test_driver_matches_reference_files(golden, workdir):
    got, out = runs.run_program(micsa.DRIVER_PATH, golden["cfg"], workdir)
    runs.compare(got, golden, "micsa_run %s" % golden["cfg"])
    assert "finished at iteration" in out


@pytest.mark.parametrize("name", ["L16_NR64_2s_nc6", "L8_NR64_2s_nc3_therm"])
def test_driver_host_refresh_matches_reference_files(name, workdir):
    """MICSA_REFRESH=host: demons drawn on host threads while the GPU sweeps,
    as the reference does, instead of on the GPU."""
    import json
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", name + ".json")))
    env = dict(os.environ, MICSA_REFRESH="host")
    got, _ = runs.run_program(micsa.DRIVER_PATH, g["cfg"], workdir, env=env)
    runs.compare(got, g, "micsa_run (host refresh) %s" % name)


@pytest.mark.parametrize("refresh", ["gpu", "host"])
def test_driver_resume_is_bit_exact(workdir, refresh):
    """Stop at an intermediate measurement (maxtime), resume with flag 0 from
    the conf/walkers checkpoints, and end where an uninterrupted run ends.
    (A case without thermalisation: the reference re-runs its nterm
    Metropolis steps on every start, main.cu:124-128, resumed or not; and a
    resumed run records flag 0 in its conf records.)"""
    import json
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "L16_NR64_2s_nc6.json")))
    cfg = dict(g["cfg"])
    assert cfg["nterm"] == 0
    env = dict(os.environ, MICSA_REFRESH=refresh)
    runs.run_program(micsa.DRIVER_PATH, dict(cfg, maxtime=16), workdir, env=env)
    got, _ = runs.run_program(micsa.DRIVER_PATH, dict(cfg, flag=0), workdir, env=env)
    for t in ("32", "64", "128"):
        for b in ("0", "1"):
            assert got["times"][t][b]["spins"] == g["times"][t][b]["spins"]
            assert got["times"][t][b]["energies"] == g["times"][t][b]["energies"]
    assert got["walkers"] == g["walkers"]
    assert got["evol"] == g["evol"]


def test_driver_rejects_bad_input(workdir):
    import subprocess
    cfg = dict(L=12, nr=32, nbits=1, nc=6, nterm=0, maxtime=4, times=[1], seed_J=1, seed_u=2,
               seed_MC0=3)
    argv = runs.write_inputs(workdir, cfg)
    p = subprocess.run([micsa.DRIVER_PATH] + argv, cwd=workdir, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    assert p.returncode != 0 and "multiple of 8" in p.stdout


def test_driver_observable_files(workdir):
    """MICSA_OBSERVABLES=1: evol_q.txt, evol_C4.txt and evol_xi.txt against
    the scalar oracle of q and C4 on the spins of the run's own conf.<t>
    records, and the correlation lengths of that C4."""
    import json
    import numpy as np
    import oracle
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "L16_NR64_2s_nc6.json")))
    cfg = dict(g["cfg"])
    L, nr = cfg["L"], cfg["nr"]
    V, nd = L ** 3, L // 2 + 1
    env = dict(os.environ, MICSA_OBSERVABLES="1")
    runs.run_program(micsa.DRIVER_PATH, cfg, workdir, env=env)
    spin_off, nsb = runs.conf_layout(L, nr)
    for b in range(cfg["nbits"]):
        sd = os.path.join(workdir, "I000", "BIT%03d" % b)
        qlines = [l.split() for l in open(os.path.join(sd, "evol_q.txt"))]
        c4lines = [l.split() for l in open(os.path.join(sd, "evol_C4.txt"))]
        xitext = open(os.path.join(sd, "evol_xi.txt")).read()
        assert xitext.startswith("# t xi12 xi23 r_cut") and "standard error" in xitext
        xilines = [l.split() for l in xitext.splitlines() if not l.startswith("#")]
        assert [int(l[0]) for l in qlines] == runs.measured(cfg)
        for k, t in enumerate(runs.measured(cfg)):
            uu = np.zeros((nr, V), np.uint8)
            for r in range(nr):
                with open(os.path.join(sd, "R%02d" % r, "conf.%016d" % t), "rb") as f:
                    c = f.read()
                uu[r] = np.unpackbits(np.frombuffer(c[spin_off:spin_off + nsb], np.uint8),
                                      bitorder="little")[:V]
            q, c4 = oracle.overlap_c4(L, nr, uu)
            assert [int(x) for x in qlines[k][1:]] == list(q), (b, t)
            got = {int(l[1]): int(l[2]) for l in c4lines if int(l[0]) == t}
            assert got == {d: int(c4[:, :, d].sum()) for d in range(nd)}, (b, t)
            _, x12, x23, cut, _ = micsa.correlation_lengths(L, c4, kappa=micsa.XI_KAPPA,
                                                            with_cut=True)
            assert xilines[k][0] == str(t) and int(xilines[k][3]) == cut
            assert abs(float(xilines[k][1]) - x12) <= 1e-9 * abs(x12) + 1e-12
            assert abs(float(xilines[k][2]) - x23) <= 1e-9 * abs(x23) + 1e-12


def _small_cfg(**kw):
    cfg = dict(L=16, nr=32, nbits=1, nc=6, nterm=0, maxtime=8, times=[1, 2, 4, 8], seed_J=5,
               seed_u=7, seed_MC0=11)
    cfg.update(kw)
    return cfg


def test_driver_lock_refuses_a_second_run(workdir):
    """create_running (io.c:1016-1047): a `running` lock in the sample folder
    stops a second program on the same folder."""
    import subprocess
    argv = runs.write_inputs(workdir, _small_cfg())
    os.makedirs(os.path.join(workdir, "I000"), exist_ok=True)
    open(os.path.join(workdir, "I000", "running"), "w").close()
    p = subprocess.run([micsa.DRIVER_PATH] + argv, cwd=workdir, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert p.returncode != 0 and "exists" in p.stdout, p.stdout[-2000:]


def test_driver_changentimes_replaces_the_measurements(workdir):
    """changentimes.in ("n t_1 ... t_n") replaces the list of measurement times."""
    cfg = _small_cfg()
    runs.write_inputs(workdir, cfg)
    os.makedirs(os.path.join(workdir, "I000"), exist_ok=True)
    with open(os.path.join(workdir, "I000", "changentimes.in"), "w") as f:
        f.write("2\n1\n4\n")
    import subprocess
    argv = runs.write_inputs(workdir, cfg)
    p = subprocess.run([micsa.DRIVER_PATH] + argv, cwd=workdir, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert p.returncode == 0, p.stdout[-2000:]
    lines = open(os.path.join(workdir, "I000", "BIT000", "evol_E_spins.txt")).read().splitlines()
    assert [int(l.split()[0]) for l in lines] == [1, 4]


def test_driver_sigterm_stops_between_iterations(workdir):
    """A SIGTERM is recorded by the handler and acted on between iterations
    (stop_run, io.c:970-994): exit status 1, the error file names the signal,
    the running lock is gone."""
    import signal
    import subprocess
    import time
    cfg = _small_cfg(maxtime=1 << 26, times=[1 << 26])
    argv = runs.write_inputs(workdir, cfg)
    p = subprocess.Popen([micsa.DRIVER_PATH] + argv, cwd=workdir, stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True)
    lock = os.path.join(workdir, "I000", "running")
    t0 = time.time()
    while not os.path.exists(lock) and time.time() - t0 < 120 and p.poll() is None:
        time.sleep(0.05)
    assert os.path.exists(lock), "the run never took its lock"
    time.sleep(0.5)
    p.send_signal(signal.SIGTERM)
    out, _ = p.communicate(timeout=300)
    assert p.returncode == 1, out[-2000:]
    assert "Received SIGTERM" in open(os.path.join(workdir, "I000", "error")).read()
    assert not os.path.exists(lock)
