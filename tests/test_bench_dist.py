"""Multi-process plumbing of bench.py on CPU (gloo, world size 2): the
barrier, the max over ranks that the timed value uses, and the reference
arm's rank-0-only JSON line.  The path shards as independent replicas (one
lattice per GPU, no exchange), so these are the only collectives."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _port()] + args
    env = dict(os.environ, OMP_NUM_THREADS="1", CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                          text=True, timeout=timeout, env=env)


def test_dist_barrier_and_max_over_two_gloo_ranks(tmp_path):
    w = tmp_path / "worker.py"
    w.write_text(
        "import sys\n"
        "sys.path.insert(0, %r)\n"
        "import bench\n"
        "d = bench.Dist(backend='gloo')\n"
        "d.barrier()\n"
        "v = d.max(1.5 * (d.rank + 1))\n"
        "d.barrier()\n"
        "print('RANK %%d WORLD %%d MAX %%.3f' %% (d.rank, d.world, v), flush=True)\n"
        "d.close()\n" % ROOT)
    p = _torchrun([str(w)])
    assert p.returncode == 0, p.stdout[-3000:]
    for r in (0, 1):
        assert "RANK %d WORLD 2 MAX 3.000" % r in p.stdout, p.stdout[-3000:]


def test_reference_arm_prints_one_line_from_rank_zero():
    p = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--L", "8", "--nr", "32",
                   "--nsamples", "1", "--nc", "2", "--steps", "2", "--warmup", "1"])
    assert p.returncode == 0, p.stdout[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout[-3000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_roofline_traffic_comes_from_the_profile_of_the_tuned_kernel():
    """bench.py's roofline.traffic is read from the committed ncu summary of
    the kernel the autotuner picked (the dataflow sweep or the per-launch
    sweep), and scaled by sites only from a capture of that same kernel."""
    sys.path.insert(0, ROOT)
    import bench
    dep, note = bench.traffic_per_launch(160, 64, 2, "k_sweep_dep")
    plain, note2 = bench.traffic_per_launch(160, 64, 2, "k_sweep")
    assert dep and plain and dep != plain
    assert "k_sweep_dep" in note and "this shape" in note and "this shape" in note2
    scaled, note3 = bench.traffic_per_launch(80, 64, 2, "k_sweep")
    assert scaled == plain / 8 and "scaled by sites" in note3
    assert bench.traffic_per_launch(160, 64, 2, "no_such_kernel") == (None, None)


def test_autotune_summary_keeps_the_pick_and_the_fastest_candidates():
    """The bench line carries the tuner's pick, how many candidates it timed
    and the three fastest, not the whole list (hundreds at L=160)."""
    sys.path.insert(0, ROOT)
    import bench
    t = ("zc=8 pd=2 split=1 occ=4 load=flow tile=row fit=16 | 4/0/0/3/0/0:0.04516ms "
         "8/2/1/4/4/1:0.03152ms 8/2/1/3/4/1:0.03223ms 16/0/0/3/0/0:0.05557ms")
    got = bench._tuning_summary(t)
    assert got.startswith("zc=8 pd=2 split=1 occ=4 load=flow tile=row fit=16 | 4 candidates timed")
    assert got.endswith("fastest 8/2/1/4/4/1:0.03152ms 8/2/1/3/4/1:0.03223ms 4/0/0/3/0/0:0.04516ms")
    assert bench._tuning_summary("zc=4 pd=0 split=0 occ=3 load=direct tile=default fit=1 cached |") \
        == "zc=4 pd=0 split=0 occ=3 load=direct tile=default fit=1 cached | 0 candidates timed"


def test_reference_arm_never_maps_the_product_library(tmp_path):
    """The reference arm times the CPU restatement only: after a whole
    `bench.py --impl reference` run in one process, libmicsa must not be among
    the process's mappings (its ratio against the GPU arm would otherwise
    compare the product with itself)."""
    w = tmp_path / "ref_arm.py"
    w.write_text(
        "import sys\n"
        "sys.path.insert(0, %r)\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--L', '8', '--nr', '32', '--nsamples',"
        " '1', '--nc', '2', '--steps', '2', '--warmup', '1']\n"
        "import bench\n"
        "bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LIBMICSA_MAPPED', 'libmicsa' in maps, 'LIBORACLE_MAPPED', 'liboracle' in maps)\n"
        % ROOT)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, str(w)], cwd=ROOT, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stdout[-3000:]
    assert "LIBMICSA_MAPPED False LIBORACLE_MAPPED True" in p.stdout, p.stdout[-3000:]
    line = json.loads(next(l for l in p.stdout.splitlines() if l.startswith("{")))
    assert line["impl"] == "reference" and line["value"] > 0
