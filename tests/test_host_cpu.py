"""CPU tests of the host library and of the oracle's own consistency."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import micsa
import oracle
import runs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_abi_exports_every_declared_symbol():
    """libmicsa loads without a GPU and exports every function declared in
    include/micsa.h."""
    hdr = open(os.path.join(ROOT, "include", "micsa.h")).read()
    declared = set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(micsa_\w+)\s*\(", hdr, flags=re.M))
    assert declared == set(micsa.ABI_SYMBOLS)
    lib = micsa.lib()
    for name in declared:
        assert hasattr(lib, name), name


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cfg = micsa.Config(0, 16, 32, 1, 6)
    h = C.c_void_p()
    rc = micsa.lib().micsa_create(C.byref(cfg), C.byref(h))
    assert rc in (2, 3) and not h.value  # ERR_CUDA / ERR_NOMEM, no context, no exit


def test_invalid_configs_rejected_before_cuda():
    for bad in [(0, 12, 32, 1, 6), (0, 16, 48, 1, 6), (0, 16, 32, 0, 6), (0, 16, 32, 1, 0),
                (0, 16, 32, 4097, 6), (0, 16, 32, 1, 7)]:
        cfg = micsa.Config(*bad)
        assert micsa.lib().micsa_footprint_bytes(C.byref(cfg)) == -1
        h = C.c_void_p()
        assert micsa.lib().micsa_create(C.byref(cfg), C.byref(h)) in (1, 5)


def test_footprint_headline():
    cfg = micsa.Config(0, 160, 64, 2, 6)
    b = micsa.lib().micsa_footprint_bytes(C.byref(cfg))
    # spins 65.5 MB, demons 2 x 393 MB, random words 49 MB, staging 197 MB
    assert 1.0e9 < b < 1.2e9


def test_isi_algebra_is_the_integer_demon_rule():
    """The ISI boolean algebra (main.cu:1037-1074) equals: with u unsatisfied
    bonds, accept iff 0 <= D + u - 3 <= 3 and then D <- D + u - 3 -- over the
    whole truth table, each case in its own bit of one word."""
    j = [0, 0, 0, 0]
    d0 = d1 = 0
    cases = []
    bit = 0
    for a in range(4):
        for b in range(4):
            for D in range(4):
                for k, v in enumerate((a & 1, a >> 1, b & 1, b >> 1)):
                    j[k] |= v << bit
                d0 |= (D & 1) << bit
                d1 |= (D >> 1) << bit
                cases.append((a + b, D))
                bit += 1
    flip, n0, n1 = oracle.isi_word(j[0], j[1], j[2], j[3], d0, d1)
    for i, (u, D) in enumerate(cases):
        nd, f = oracle.scalar_rule(u, D)
        assert (flip >> i) & 1 == f
        assert ((n0 >> i) & 1) + 2 * ((n1 >> i) & 1) == nd


def test_metropolis_rule_depends_only_on_total_unsatisfied():
    """The Metropolis acceptance expression of the reference (main.cu:950-957)
    is a function of u = (j1 + 2 j2) + (j3 + 2 j4) and the random bits only;
    with the ISI check above this is why the GPU sweep may put either
    x-neighbour into either bond group."""
    seen = {}
    for a in range(4):
        for b in range(4):
            for r in range(8):
                j1, j2, j3, j4 = a & 1, a >> 1, b & 1, b >> 1
                b0, b1, b2 = r & 1, (r >> 1) & 1, (r >> 2) & 1
                b1 &= b0
                b2 &= b1
                id2, id1, j24 = b1, (b0 ^ b1) | b2, j2 | j4
                f = (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2))
                assert seen.setdefault((a + b, r), f) == f


@pytest.mark.parametrize("L", [8, 16, 24, 40])
def test_pack_unpack_roundtrip(L):
    """check_packing (ini.c:397-423)."""
    nr = 32
    rng = np.random.default_rng(L)
    uu = rng.integers(0, 2, size=nr * L ** 3, dtype=np.uint8)
    e, o = micsa.pack_spins(L, nr, uu)
    assert np.array_equal(micsa.unpack_spins(L, nr, e, o), uu)


@pytest.mark.parametrize("L", [8, 16, 24])
def test_energy_equals_scalar_energy(L):
    """d_computeEne vs calculate_scalar_energy (the reference's resume check,
    io.c:186-196) on random states."""
    nr = 32
    rng = np.random.default_rng(L + 1)
    V = L ** 3
    uu = rng.integers(0, 2, size=nr * V, dtype=np.uint8)
    Jx, Jy, Jz = (rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3))
    e, o = micsa.pack_spins(L, nr, uu)
    J = micsa.pack_couplings(L, Jx, Jy, Jz)
    en = oracle.energy(L, nr, J, e, o)
    for r in range(nr):
        assert en[r] == oracle.scalar_energy(L, uu[r * V:(r + 1) * V], Jx, Jy, Jz)


@pytest.mark.parametrize("L", [8, 16, 24, 40])
def test_oracle_coupling_packer_equals_product_packer(L):
    """The oracle's packing_J restatement (used by the CPU arms of bench.py,
    which must not load the product library) and the product's host packer
    give the same coupling words."""
    rng = np.random.default_rng(L + 17)
    Jx, Jy, Jz = (rng.integers(0, 2, size=L ** 3, dtype=np.uint8) for _ in range(3))
    assert np.array_equal(oracle.pack_couplings(L, Jx, Jy, Jz), micsa.pack_couplings(L, Jx, Jy, Jz))


def test_walk_is_a_translation():
    """After k walks (d_Walk), the colour-p demon of plane ic sits at
    x + sgn*2k*e_axis of where it started (sgn = +1 iff (p == 0) == (ic < 3)):
    the fact that lets the GPU replace the walk by an address offset."""
    L, nr, nc = 16, 32, 6
    H, V = (L // 4) ** 3 // 2, L ** 3
    rng = np.random.default_rng(2)
    n = 2 * nc * H * nr
    w0 = rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64, endpoint=True)
    w1 = w0.copy()

    def real(w):
        out = np.zeros((2, nc, nr, L, L, L), np.uint8)
        for p in range(2):
            for ic in range(nc):
                words = w[(p * nc + ic) * H * nr:(p * nc + ic + 1) * H * nr]
                z = np.zeros_like(words)
                e, o = (words, z) if p == 0 else (z, words)
                out[p, ic] = micsa.unpack_spins(L, nr, e, o).reshape(nr, L, L, L)
        return out
    before = real(w0)
    k = 3
    for _ in range(k):
        oracle.walk(L, nr, nc, w0, w1)
    after = real(w0)
    s = np.arange(L)
    colour = (s[:, None, None] + s[None, :, None] + s[None, None, :]) & 1
    for p in range(2):
        for ic in range(nc):
            axis = ic % 3
            sgn = 1 if (p == 0) == (ic < 3) else -1
            shift = [0, 0, 0]
            shift[2 - axis] = sgn * 2 * k  # arrays are [z][y][x]
            pred = np.roll(before[p, ic], shift=shift, axis=(1, 2, 3))
            m = colour == p
            assert np.array_equal(after[p, ic][:, m], pred[:, m])


def test_thresholds_and_demon_distribution():
    """get_thresholds (ini.c:680-710): P(D=k) ~ e^{-4 beta k}; the draws of
    InitWalkers follow it within 5 sigma."""
    beta = float(runs.BETA_TEXT)
    thr = micsa.thresholds(beta)
    f = np.exp(-4 * beta)
    p = np.array([1, f, f * f, f ** 3])
    p /= p.sum()
    assert abs(int(thr[0]) / 2 ** 64 - p[3]) < 1e-15
    assert abs(int(thr[2]) / 2 ** 64 - (1 - p[0])) < 1e-15
    hm = micsa.HostModel(8, 64, 6, 1, 2, list(range(3, 67)), [0])
    w0, w1 = hm.draw_demons(0)
    bits = np.unpackbits(w0.view(np.uint8)).astype(np.int64) + 2 * np.unpackbits(w1.view(np.uint8))
    n = bits.size
    for k in range(4):
        c = int((bits == k).sum())
        assert abs(c - n * p[k]) < 5 * np.sqrt(n * p[k] * (1 - p[k])) + 1


def test_philox_bits_density():
    """The Philox4x32-10 + LUT generator gives i.i.d. Bernoulli(e^{-4 beta})
    bits (the check of input/LUT/bits-random.cu: densities within 4 sigma)."""
    L, nr = 16, 64
    lut = runs.lut_bytes()[8:]
    rng = np.random.default_rng(0)
    te = rng.integers(0, 2 ** 32, size=4 * nr, dtype=np.uint32)
    keys = rng.integers(0, 2 ** 32, size=nr, dtype=np.uint32)
    out = oracle.gen_rndbits(L, nr, te, keys, lut)
    bits = np.unpackbits(out.view(np.uint8))
    p = np.exp(-4 * float(runs.BETA_TEXT))
    n = bits.size
    assert abs(bits.sum() - n * p) < 4 * np.sqrt(n * p * (1 - p))


def test_seed_fanout_paranoia_constant():
    """generate_seeds_from_one always skips 109 outputs (random_generator.cu:
    215-231): the fan-out is a pure function of the seed."""
    a = micsa.seeds_from_one(12345, 8)[1]
    b = micsa.seeds_from_one(12345, 8)[1]
    assert np.array_equal(a, b) and len(set(a.tolist())) == 8


def test_every_environment_variable_is_documented():
    """Every MICSA_* variable the library reads is listed in the public
    header, and every one the command-line driver reads in the driver's
    usage comment."""
    import glob
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkg = os.path.join(root, "micsa-ea-mc_gb300")
    read = lambda fs: set().union(*(re.findall(r'getenv\("(MICSA_[A-Z_]+)"\)', open(f).read())
                                    for f in fs))
    drv = os.path.join(pkg, "host", "micsa_driver.c")
    lib_names = read(glob.glob(os.path.join(pkg, "csrc", "*.cu")) +
                     [f for f in glob.glob(os.path.join(pkg, "host", "*.c")) if f != drv])
    drv_names = read([drv])
    header = open(os.path.join(root, "include", "micsa.h")).read()
    usage = open(drv).read().split("*/", 1)[0]
    assert lib_names and drv_names
    assert not [n for n in sorted(lib_names) if n not in header]
    assert not [n for n in sorted(drv_names) if n not in usage]


def test_noalloc_entry_point_checks_its_arguments_before_any_device_work():
    """micsa_energy_noalloc rejects impossible sizes and missing row tables
    before it touches a device, so these calls need no GPU; they also check
    that the binding's argument list matches the declaration."""
    err = C.create_string_buffer(256)
    f = micsa.lib().micsa_energy_noalloc
    dummy = (C.c_void_p * 64)(*([16] * 64))
    assert f(16, micsa.NOALLOC_MAX_REPLICAS, 2, dummy, dummy, C.c_void_p(16), None, err, 256) == 1
    assert b"exceeds" in err.value
    assert f(micsa.NOALLOC_MAX_L + 8, 32, 1, dummy, dummy, C.c_void_p(16), None, err, 256) == 1
    assert b"888" in err.value
    assert f(16, 32, 1, None, dummy, C.c_void_p(16), None, err, 256) == 1
    nulls = (C.c_void_p * 24)()
    assert f(16, 32, 1, dummy, nulls, C.c_void_p(16), None, err, 256) == 1
    assert b"coupling row 0" in err.value
