"""Run descriptions shared by the golden-vector generator and the tests.

A run is the reference program's main loop (PROGRAM/src/main.cu:10-195) on
seeded inputs.  Three implementations produce the same summary dict:
  * reference_run: the reference program built for the CPU (oracle/_ref);
  * oracle_run:    the product's host initialisation + the CPU oracle;
  * driver_run:    the product's micsa_run driver on the GPU.
The summary holds the measurement files verbatim and SHA-256 digests of the
spin and demon states, so fixtures stay small.
"""
import ctypes as C
import hashlib
import math
import os
import struct
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "micsa-ea-mc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import micsa  # noqa: E402

BETA_TEXT = "0.90909090909090"  # input/BETAS/beta.in
JANUS_SEED = 9164166177945067407


def sha(b):
    return hashlib.sha256(b).hexdigest()


def lut_bytes(beta=None):
    """4104-byte LUT file (beta + s_lut_heat_bath) from the product's builder."""
    beta = float(BETA_TEXT) if beta is None else beta
    out = np.zeros(4096, np.uint8)
    f = micsa.lib().micsa_build_lut
    f.argtypes = [C.c_double, C.c_void_p]
    f(beta, out.ctypes.data_as(C.c_void_p))
    return struct.pack("<d", beta) + out.tobytes()


def seeds_mc(cfg):
    return [cfg["seed_MC0"] + r for r in range(cfg["nr"])]


def write_inputs(d, cfg):
    """input.in / times.in / beta.in / lut.bin for one run, in directory d."""
    os.makedirs(d, exist_ok=True)
    lines = ["./", str(cfg["maxtime"]), "0", str(len(cfg["times"])), str(cfg["nterm"]),
             str(cfg["nc"]), str(cfg["nr"]), str(cfg["L"]), str(cfg.get("flag", 1)),
             str(cfg["seed_J"]), str(cfg["seed_u"])] + [str(s) for s in seeds_mc(cfg)]
    with open(os.path.join(d, "input.in"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(d, "times.in"), "w") as f:
        f.write("\n".join(str(t) for t in cfg["times"]) + "\n")
    with open(os.path.join(d, "beta.in"), "w") as f:
        f.write(BETA_TEXT + "\n")
    with open(os.path.join(d, "lut.bin"), "wb") as f:
        f.write(lut_bytes())
    argv = [str(cfg.get("isample", 0)), str(cfg["nbits"]), "beta.in", "input.in", "lut.bin",
            "times.in", "0"]
    if cfg.get("list_samples"):
        with open(os.path.join(d, "samples.in"), "w") as f:
            f.write("\n".join(str(s) for s in cfg["list_samples"]) + "\n")
        argv += ["0", "samples.in"]
    return argv


def conf_layout(L, nr):
    data = 40 + 8 * (2 + nr)
    spin_off = data + 8 + 2080 + 48 + 1
    return spin_off, L ** 3 // 8


def collect(outdir, cfg, measured_times):
    """Summary of a finished run whose sample tree is outdir (= .../I000/)."""
    L, nr, nbits = cfg["L"], cfg["nr"], cfg["nbits"]
    samples = cfg.get("list_samples") or list(range(nbits))
    spin_off, nsb = conf_layout(L, nr)
    res = {"evol": {}, "seeds_in": {}, "conf_Js": {}, "times": {}, "walkers": {}}
    with open(os.path.join(outdir, "master_seedJ.in")) as f:
        res["master_seedJ"] = f.read()
    for b, s in enumerate(samples):
        sd = os.path.join(outdir, "BIT%03d" % s)
        ev = {}
        for k in ("E_spins", "E_walkers", "T_walkers"):
            with open(os.path.join(sd, "evol_%s.txt" % k)) as f:
                ev[k] = f.read()
        res["evol"][str(b)] = ev
        with open(os.path.join(sd, "seeds.in")) as f:
            res["seeds_in"][str(b)] = f.read()
        with open(os.path.join(sd, "conf_Js"), "rb") as f:
            res["conf_Js"][str(b)] = sha(f.read())
        for t in measured_times:
            spins, confs, en = [], [], []
            for r in range(nr):
                with open(os.path.join(sd, "R%02d" % r, "conf.%016d" % t), "rb") as f:
                    c = f.read()
                confs.append(c)
                spins.append(c[spin_off:spin_off + nsb])
                en.append(struct.unpack("<i", c[spin_off + nsb:spin_off + nsb + 4])[0])
            res["times"].setdefault(str(t), {})[str(b)] = {
                "spins": sha(b"".join(spins)), "conf": sha(b"".join(confs)), "energies": en}
        with open(os.path.join(sd, "walkers"), "rb") as f:
            w = f.read()
        hdr = 40 + nr * (2080 + 48)
        res["walkers"][str(b)] = {"file": sha(w), "demons": sha(w[hdr:])}
    return res


def measured(cfg):
    return [t for t in cfg["times"] if t <= cfg["maxtime"]]


def run_program(exe, cfg, workdir, timeout=3600, env=None, exit_race_ok=False):
    """Run the reference (or micsa_run) with the reference argv in workdir.

    exit_race_ok: the reference frees its demon buffers at exit while the
    last detached demon-generation thread may still write them (main.cu:
    191-192 vs 372), which can crash the process after every output file is
    complete; such an exit is accepted once the completion line is printed."""
    argv = write_inputs(workdir, cfg)
    p = subprocess.run([exe] + argv, cwd=workdir, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=timeout, env=env)
    finished = "finished at iteration" in p.stdout
    if p.returncode != 0 and not (exit_race_ok and finished):
        raise RuntimeError("%s exited %d:\n%s" % (exe, p.returncode, p.stdout[-4000:]))
    # the reference formats "{dir}I%03d/" with overlapping sprintf buffers and
    # under glibc's fortified sprintf ends up with "I%03d/"; the product uses
    # the intended "{dir}I%03d/" -- with dir = "./" both are the same folder.
    return collect(os.path.join(workdir, "I%03d" % cfg.get("isample", 0)), cfg, measured(cfg)), p.stdout


# --------------------------------------------------------------- oracle run
def _evol_line(t, a, b):
    return "%d %14.10g %14.10g\n" % (t, a, b)


def _stats(vals, nr):
    a = s = 0.0
    for v in vals:
        a += v
        s += v * v
    a /= float(nr)
    s /= float(nr)
    s -= a * a
    s /= float(nr) - 1
    return a, math.sqrt(s)


def data_record(cfg, now, seed_J, seed_u, seed_MC, flag=1):
    return (struct.pack("<QQ6i", cfg["maxtime"], now, len(cfg["times"]), cfg["nterm"], cfg["nc"],
                        cfg["nr"], cfg["L"], flag)
            + struct.pack("<%dQ" % (2 + cfg["nr"]), seed_J, seed_u, *seed_MC))


class OracleEngine:
    """Sweeps on the CPU oracle, state in the reference layouts."""

    def __init__(self, cfg, hm, lut, nthreads=8):
        import oracle
        self.o, self.cfg, self.nthreads, self.lut = oracle, cfg, nthreads, lut
        self.even = [hm.spins[b][0].copy() for b in range(cfg["nbits"])]
        self.odd = [hm.spins[b][1].copy() for b in range(cfg["nbits"])]
        self.J = hm.J
        self.w0 = [None] * cfg["nbits"]
        self.w1 = [None] * cfg["nbits"]

    def metropolis(self, te0, te1, keys):
        c = self.cfg
        for b in range(c["nbits"]):
            self.o.metropolis_iteration(c["L"], c["nr"], self.J[b], self.even[b], self.odd[b],
                                        te0, te1, keys, self.lut)

    def set_demons(self, b, w0, w1):
        self.w0[b], self.w1[b] = w0.copy(), w1.copy()

    def iterate(self, n):
        c = self.cfg
        for _ in range(n):
            for b in range(c["nbits"]):
                self.o.micsa_iteration(c["L"], c["nr"], c["nc"], self.J[b], self.even[b],
                                       self.odd[b], self.w0[b], self.w1[b], self.nthreads)

    def state(self, b):
        return self.even[b], self.odd[b], self.w0[b], self.w1[b]

    def energies(self, b):
        c = self.cfg
        return (self.o.energy(c["L"], c["nr"], self.J[b], self.even[b], self.odd[b]),
                self.o.demon_energy(c["L"], c["nr"], c["nc"], self.w0[b], self.w1[b]))


class GpuEngine:
    """Sweeps on the GPU through the C ABI (libmicsa)."""

    def __init__(self, cfg, hm, lut, device=0):
        c = cfg
        self.cfg = cfg
        self.ctx = micsa.Context(c["L"], c["nr"], c["nbits"], c["nc"], device)
        self.ctx.set_lut(lut)
        for b in range(c["nbits"]):
            self.ctx.upload_couplings(b, hm.J[b])
            self.ctx.upload_spins(b, hm.spins[b][0], hm.spins[b][1])
        self._meas = None

    def metropolis(self, te0, te1, keys):
        self.ctx.monte_carlo(0, np.concatenate([te0, te1]), keys)

    def set_demons(self, b, w0, w1):
        self.ctx.upload_demons(b, w0, w1)

    def iterate(self, n):
        self.ctx.iterate(n)
        self._meas = None

    def state(self, b):
        e, o = self.ctx.download_spins(b)
        w0, w1 = self.ctx.download_demons(b)
        return e, o, w0, w1

    def energies(self, b):
        if self._meas is None:
            self._meas = self.ctx.measure(spin=True, demon=True)
        return self._meas["e_spin"][b], self._meas["e_demon"][b]

    def close(self):
        self.ctx.close()


def model_run(cfg, engine="oracle", nthreads=8, on_state=None, device=0):
    """The reference main loop (main.cu:121-180) with product host init and
    sweeps on `engine` ("oracle" or "gpu"); returns a run summary."""
    L, nr, nc, nbits = cfg["L"], cfg["nr"], cfg["nc"], cfg["nbits"]
    samples = cfg.get("list_samples") or list(range(nbits))
    jobid = cfg.get("isample", 0)
    hm = micsa.HostModel(L, nr, nc, cfg["seed_J"], cfg["seed_u"], seeds_mc(cfg), samples,
                         beta=float(BETA_TEXT), nthreads=nthreads)
    lut = lut_bytes()[8:]
    eng = OracleEngine(cfg, hm, lut, nthreads) if engine == "oracle" else GpuEngine(cfg, hm, lut, device)
    V = L ** 3
    res = {"evol": {str(b): {"E_spins": "", "E_walkers": "", "T_walkers": ""} for b in range(nbits)},
           "seeds_in": {}, "conf_Js": {}, "times": {}, "walkers": {},
           "master_seedJ": "%d\n" % hm.seed_J}
    for b in range(nbits):
        res["seeds_in"][str(b)] = "%d %d %s %d\n" % (hm.seeds_J[b], hm.seed_u,
                                                      " ".join(str(s) for s in hm.seed_MC),
                                                      hm.Jsite[b][3])
        bits = b"".join(np.packbits(hm.Jsite[b][k], bitorder="little").tobytes() for k in range(3))
        res["conf_Js"][str(b)] = sha(bits)
    # thermalisation (main.cu:126-128)
    for t in range(cfg["nterm"]):
        te0 = hm.fill_bits(2 * t, 0, jobid)
        te1 = hm.fill_bits(2 * t + 1, 1, jobid)
        eng.metropolis(te0, te1, hm.keys)
    snap = [None] * nbits
    times = measured(cfg)
    it, i, prev_t = 0, 0, 0
    while it < cfg["maxtime"] and i < len(times):
        if not (it & (it - 1)):
            for b in range(nbits):
                w0, w1 = hm.draw_demons(b)
                eng.set_demons(b, w0, w1)
                snap[b] = (bytes(hm.prc_C[b]), bytes(hm.xo_C[b]))
        # run to the next refresh or measurement
        nxt, p2 = times[i], 1
        while p2 <= it:
            p2 <<= 1
        nxt = min(nxt, p2, cfg["maxtime"])
        if on_state:
            nxt = it + 1
        eng.iterate(nxt - it)
        it = nxt
        if on_state:
            on_state(it, eng)
        if it == times[i]:
            for b in range(nbits):
                e, ed = eng.energies(b)
                even, odd, w0, w1 = eng.state(b)
                es_m, es_s = _stats([float(-int(x)) / V for x in e], nr)
                ec_m, ec_s = _stats([float(int(x)) / (float(V) * nc) for x in ed], nr)
                ev = res["evol"][str(b)]
                ev["E_spins"] += _evol_line(it, es_m, es_s)
                ev["E_walkers"] += _evol_line(it, ec_m, ec_s)
                ev["T_walkers"] += "%d %14.10g \n" % (it, 1.0 / (0.25 * math.log(1.0 + 1.0 / ec_m)))
                uu = micsa.unpack_spins(L, nr, even, odd).reshape(nr, V)
                spins, confs = [], []
                drec = data_record(cfg, it, JANUS_SEED, hm.seed_u, hm.seed_MC)
                for r in range(nr):
                    sb = np.packbits(uu[r], bitorder="little").tobytes()
                    spins.append(sb)
                    confs.append(drec + struct.pack("<d", float(BETA_TEXT)) + bytes(hm.prc[r])
                                 + bytes(hm.xo[r]) + b"\x00" + sb + struct.pack("<i", int(e[r])))
                res["times"].setdefault(str(it), {})[str(b)] = {
                    "spins": sha(b"".join(spins)), "conf": sha(b"".join(confs)),
                    "energies": [int(x) for x in e]}
                icds = struct.pack("<6IQd", 0, b, nr, nc, L, 0,
                                   int(hm.seeds_C[samples[b]]), float(BETA_TEXT))
                dem = w0.tobytes() + w1.tobytes()
                res["walkers"][str(b)] = {"file": sha(icds + snap[b][0] + snap[b][1] + dem),
                                          "demons": sha(dem)}
            prev_t = it
            i += 1
    res["final_time"] = prev_t
    if hasattr(eng, "close"):
        eng.close()
    return res


def oracle_run(cfg, nthreads=8):
    return model_run(cfg, "oracle", nthreads)


def compare(got, want, what="run"):
    """Assert two run summaries agree; returns the list of compared keys."""
    keys = []
    assert got["master_seedJ"] == want["master_seedJ"], "%s: master_seedJ" % what
    for b, ev in want["evol"].items():
        for k, text in ev.items():
            assert got["evol"][b][k] == text, "%s: evol_%s.txt of sample %s differs:\n%s\nvs\n%s" % (
                what, k, b, got["evol"][b][k], text)
            keys.append("evol_%s[%s]" % (k, b))
        assert got["seeds_in"][b] == want["seeds_in"][b], "%s: seeds.in %s" % (what, b)
        assert got["conf_Js"][b] == want["conf_Js"][b], "%s: conf_Js %s" % (what, b)
    for t, per in want["times"].items():
        for b, v in per.items():
            g = got["times"][t][b]
            assert g["energies"] == v["energies"], "%s: energies t=%s sample %s" % (what, t, b)
            assert g["spins"] == v["spins"], "%s: spins t=%s sample %s" % (what, t, b)
            assert g["conf"] == v["conf"], "%s: conf records t=%s sample %s" % (what, t, b)
            keys.append("conf[t=%s,%s]" % (t, b))
    for b, v in want["walkers"].items():
        assert got["walkers"][b]["demons"] == v["demons"], "%s: final demons of sample %s" % (what, b)
        assert got["walkers"][b]["file"] == v["file"], "%s: walkers file of sample %s" % (what, b)
        keys.append("walkers[%s]" % b)
    return keys
