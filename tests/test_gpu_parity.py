"""CUDA path (libmicsa through its C ABI) against the oracle and the golden
outputs of the reference.  Integer/bitwise work: every comparison is exact.
"""
import numpy as np
import pytest

import micsa
import oracle
import runs
from conftest import golden_cases

pytestmark = pytest.mark.gpu

LUT = runs.lut_bytes()[8:]


def random_state(rng, L, nr, nc, ns, consistent=True):
    """Random spins, demons and couplings in the reference layouts.  With
    consistent=False the 12 coupling words are independent random words (a
    bond then has different values seen from its two ends), which checks that
    the GPU consumes each word exactly as the reference kernel does."""
    H = (L // 4) ** 3 // 2
    V = L ** 3
    st = []
    for _ in range(ns):
        Jx, Jy, Jz = (rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3))
        if consistent:
            J = micsa.pack_couplings(L, Jx, Jy, Jz)
        else:
            J = rng.integers(0, 2 ** 64 - 1, size=12 * H, dtype=np.uint64, endpoint=True)
        e = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        o = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        n = 2 * H * nc * nr
        # demons in 0..3 with a nonuniform mix of levels
        w0 = rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64, endpoint=True)
        w1 = rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64, endpoint=True) & \
            rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64, endpoint=True)
        st.append([J, e, o, w0, w1, (Jx, Jy, Jz)])
    return st


@pytest.mark.parametrize("golden", golden_cases())
def test_gpu_reproduces_reference(golden):
    """Full runs (thermalisation, refreshes, walks, measurements) on the GPU
    give the reference program's files bit for bit."""
    got = runs.model_run(golden["cfg"], engine="gpu", nthreads=16)
    runs.compare(got, golden, golden["cfg"])


@pytest.mark.parametrize("L,nr,nc,ns,iters", [
    (8, 32, 6, 1, 9), (8, 64, 2, 3, 5), (16, 32, 6, 2, 17), (16, 96, 3, 1, 4),
    (24, 32, 6, 1, 13), (32, 64, 6, 2, 3), (40, 32, 4, 1, 21), (48, 128, 6, 1, 2),
    (64, 64, 6, 1, 2), (64, 64, 6, 8, 3), (96, 32, 6, 2, 2), (56, 64, 5, 3, 4),
    (24, 256, 3, 1, 5),   # two word groups of four-word vectors
    (24, 160, 2, 2, 4),   # five word groups of one word
])
def test_gpu_matches_oracle_random_state(L, nr, nc, ns, iters):
    """Arbitrary states (not reachable from seeds), many iterations so the
    demon walk wraps around the lattice more than once for small L."""
    rng = np.random.default_rng(L * 1000 + nr + nc)
    st = random_state(rng, L, nr, nc, ns, consistent=(ns > 1))
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ctx.iterate(iters)
        ctx.synchronize()
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            for _ in range(iters):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 8)
            ge, go = ctx.download_spins(s)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(ge, e) and np.array_equal(go, o), "spins differ, sample %d" % s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), "demons differ, sample %d" % s
        m = ctx.measure(spin=True, demon=True)
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            assert np.array_equal(m["e_spin"][s], oracle.energy(L, nr, J, e, o))
            assert np.array_equal(m["e_demon"][s], oracle.demon_energy(L, nr, nc, w0, w1))


def test_gpu_monte_carlo_step_equals_iterate():
    """micsa_monte_carlo(flag=1) (direct launches) and micsa_iterate (graph
    replay) are the same step."""
    L, nr, nc = 16, 64, 6
    rng = np.random.default_rng(5)
    (J, e, o, w0, w1, _), = random_state(rng, L, nr, nc, 1)
    out = []
    for use_graph in (False, True):
        with micsa.Context(L, nr, 1, nc) as ctx:
            ctx.upload_couplings(0, J)
            ctx.upload_spins(0, e, o)
            ctx.upload_demons(0, w0, w1)
            for _ in range(7):
                if use_graph:
                    ctx.iterate(1)
                else:
                    ctx.monte_carlo(1)
            out.append(ctx.download_spins(0) + ctx.download_demons(0))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("L,nr,ns", [(8, 32, 1), (16, 64, 2), (24, 96, 1), (32, 32, 3)])
def test_gpu_metropolis_matches_oracle(L, nr, ns):
    """Philox4x32-10 heat-bath bits + Metropolis sweeps, random counters."""
    rng = np.random.default_rng(L + nr)
    st = random_state(rng, L, nr, 1, ns)
    keys = rng.integers(0, 2 ** 32, size=nr, dtype=np.uint32)
    with micsa.Context(L, nr, ns, 1) as ctx:
        ctx.set_lut(LUT)
        for s, (J, e, o, *_r) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
        for t in range(3):
            te = rng.integers(0, 2 ** 32, size=8 * nr, dtype=np.uint32)
            ctx.monte_carlo(0, te, keys)
            for s, (J, e, o, *_r) in enumerate(st):
                oracle.metropolis_iteration(L, nr, J, e, o, te[:4 * nr].copy(), te[4 * nr:].copy(),
                                            keys, LUT)
        for s, (J, e, o, *_r) in enumerate(st):
            ge, go = ctx.download_spins(s)
            assert np.array_equal(ge, e) and np.array_equal(go, o)


@pytest.mark.parametrize("L,nr,ns", [(8, 32, 1), (16, 64, 2), (24, 32, 1)])
def test_gpu_overlap_c4_matches_scalar_oracle(L, nr, ns):
    rng = np.random.default_rng(3 * L + nr)
    st = random_state(rng, L, nr, 1, ns)
    with micsa.Context(L, nr, ns, 1) as ctx:
        for s, (J, e, o, *_r) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
        m = ctx.measure(spin=True, demon=False, overlap=True)
        for s, (J, e, o, _a, _b, (Jx, Jy, Jz)) in enumerate(st):
            uu = micsa.unpack_spins(L, nr, e, o)
            q, c4 = oracle.overlap_c4(L, nr, uu)
            assert np.array_equal(m["q"][s], q)
            assert np.array_equal(m["c4"][s], c4)
            V = L ** 3
            for r in range(nr):
                assert m["e_spin"][s][r] == oracle.scalar_energy(L, uu[r * V:(r + 1) * V], Jx, Jy, Jz)


def test_gpu_roundtrip_and_errors():
    L, nr, nc = 16, 64, 3
    rng = np.random.default_rng(11)
    (J, e, o, w0, w1, _), = random_state(rng, L, nr, nc, 1)
    with micsa.Context(L, nr, 2, nc) as ctx:
        with pytest.raises(micsa.MicsaError, match="ERR_STATE"):
            ctx.iterate(1)
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            ctx.upload_spins(2, e, o)
        with pytest.raises(micsa.MicsaError, match="ERR_STATE"):
            ctx.monte_carlo(0, np.zeros(8 * nr, np.uint32), np.zeros(nr, np.uint32))
        for s in range(2):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ge, go = ctx.download_spins(1)
        g0, g1 = ctx.download_demons(1)
        assert np.array_equal(ge, e) and np.array_equal(go, o)
        assert np.array_equal(g0, w0) and np.array_equal(g1, w1)
    for bad in [dict(L=12), dict(nr=16), dict(nc=7), dict(nsamples=0)]:
        kw = dict(L=16, nr=32, nsamples=1, nc=6)
        kw.update(bad)
        with pytest.raises(micsa.MicsaError):
            micsa.Context(kw["L"], kw["nr"], kw["nsamples"], kw["nc"])


def test_gpu_full_size_headline_properties():
    """L=160, 2 samples x 64 replicas, 6 demons: one iteration equals the
    oracle; between refreshes E_spin + 4*E_demon is conserved per replica
    (the microcanonical invariant) and the demon walk conserves demons."""
    L, nr, nc, ns = 160, 64, 6, 2
    rng = np.random.default_rng(160)
    st = random_state(rng, L, nr, nc, ns)
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        m0 = ctx.measure()
        ctx.iterate(1)
        s = 0
        J, e, o, w0, w1, _ = st[s]
        oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 32)
        ge, go = ctx.download_spins(s)
        assert np.array_equal(ge, e) and np.array_equal(go, o)
        g0, g1 = ctx.download_demons(s)
        assert np.array_equal(g0, w0) and np.array_equal(g1, w1)
        inv0 = m0["e_spin"].astype(np.int64) - 4 * m0["e_demon"].astype(np.int64)
        for _ in range(3):
            ctx.iterate(7)
            m = ctx.measure()
            inv = m["e_spin"].astype(np.int64) - 4 * m["e_demon"].astype(np.int64)
            assert np.array_equal(inv, inv0)
            assert not np.array_equal(m["e_spin"], m0["e_spin"])
