"""The sweep with TMA-staged demon tiles (cp.async.bulk.tensor into shared
memory, completing on mbarriers), pinned on, against the oracle: over more
iterations than half the lattice side, so every walk shift -- odd ones that
start a tile 8 bytes off a 16-byte boundary, and tiles that wrap around the
lattice and keep the global loads -- is met, with one launch for all samples
and sample-major launches."""
import os

import numpy as np
import pytest

import micsa
import oracle
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


def _pinned(env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    return old


def _restore(old):
    for k, v in old.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v


@pytest.mark.parametrize("L,nr,nc,ns,split", [(32, 64, 6, 2, 0), (32, 32, 4, 1, 0), (64, 128, 6, 2, 1),
                                              (96, 64, 6, 2, 1), (64, 64, 3, 3, 0)])
def test_staged_sweep_matches_oracle(L, nr, nc, ns, split):
    old = _pinned({"MICSA_SWEEP_ZC": "4", "MICSA_SWEEP_PD": "0", "MICSA_SWEEP_TMA": "1",
                   "MICSA_SWEEP_SPLIT": str(split), "MICSA_SWEEP_OCC": "4", "MICSA_RESIDENT": "0"})
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "load=tma" in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(L + nr + ns)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ctx.iterate(iters)
        ctx.synchronize()  # also reports any staged load that timed out
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            for _ in range(iters):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 8)
            ge, go = ctx.download_spins(s)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nc,ns,split,occ", [(32, 6, 2, 0, 4), (40, 3, 1, 0, 3), (64, 6, 2, 1, 4),
                                               (96, 5, 2, 1, 3)])
def test_async_staged_sweep_matches_oracle(L, nc, ns, split, occ):
    """The cp.async double-buffered sweep (64 replicas, one 8-byte vector per
    site), pinned on, against the oracle over every walk shift."""
    nr = 64
    old = _pinned({"MICSA_SWEEP_ZC": "4", "MICSA_SWEEP_PD": "0", "MICSA_SWEEP_ASYNC": "1",
                   "MICSA_SWEEP_SPLIT": str(split), "MICSA_SWEEP_OCC": str(occ),
                   "MICSA_RESIDENT": "0"})
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "load=async" in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(7 * L + ns)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
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
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nr,nc,ns,split,occ,zc,pd", [(32, 64, 6, 2, 0, 3, 4, 2), (40, 32, 3, 1, 0, 2, 8, 0),
                                                       (64, 128, 6, 2, 1, 3, 8, 4),
                                                       (96, 64, 5, 2, 1, 2, 16, 2),
                                                       (48, 96, 2, 3, 0, 3, 1, 0)])
def test_pipelined_sweep_matches_oracle(L, nr, nc, ns, split, occ, zc, pd):
    """The sweep with each z step's loads issued one step ahead, pinned on,
    against the oracle over every walk shift (32, 64, 96 and 128 replicas:
    one, two, three-of-one and four-word vectors)."""
    old = _pinned({"MICSA_SWEEP_ZC": str(zc), "MICSA_SWEEP_PD": str(pd), "MICSA_SWEEP_PIPE": "1",
                   "MICSA_SWEEP_SPLIT": str(split), "MICSA_SWEEP_OCC": str(occ),
                   "MICSA_RESIDENT": "0"})
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "load=pipe" in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(11 * L + ns)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
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
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nr,nc,ns,split,pipe", [(40, 64, 6, 2, 0, 0), (96, 64, 6, 2, 1, 0),
                                                   (56, 32, 3, 1, 0, 1), (96, 128, 2, 2, 0, 1)])
def test_whole_row_blocks_match_oracle(L, nr, nc, ns, split, pipe):
    """Sweep blocks spanning whole rows along x (tile=row; L/4 threads per
    row, the last y tile partly empty), direct and pipelined loads, against
    the oracle over every walk shift."""
    old = _pinned({"MICSA_SWEEP_ZC": "4", "MICSA_SWEEP_PD": "2", "MICSA_SWEEP_PIPE": str(pipe),
                   "MICSA_SWEEP_TILE": "row", "MICSA_SWEEP_SPLIT": str(split),
                   "MICSA_SWEEP_OCC": "3", "MICSA_RESIDENT": "0"})
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "tile=row" in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(13 * L + ns + pipe)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
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
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nc,ns,split,occ,zc,pd,tile", [(32, 6, 2, 0, 4, 4, 2, None),
                                                        (40, 3, 1, 0, 3, 8, 0, None),
                                                        (96, 5, 2, 1, 4, 4, 2, "row"),
                                                        (24, 2, 3, 0, 3, 2, 0, None),
                                                        (64, 6, 2, 1, 3, 8, 4, "row")])
def test_four_site_threads_match_oracle(L, nc, ns, split, occ, zc, pd, tile):
    """32 replicas (one word per site) with four sites per thread (load=quad:
    16-byte loads; demon words loaded one by one when the walk's x shift is
    not a multiple of four x/2 steps), against the oracle over every walk
    shift, with rows of 3 to 12 four-site groups."""
    nr = 32
    env = {"MICSA_SWEEP_ZC": str(zc), "MICSA_SWEEP_PD": str(pd), "MICSA_SWEEP_QUAD": "1",
           "MICSA_SWEEP_SPLIT": str(split), "MICSA_SWEEP_OCC": str(occ), "MICSA_RESIDENT": "0"}
    if tile:
        env["MICSA_SWEEP_TILE"] = tile
    old = _pinned(env)
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "load=quad" in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(19 * L + ns)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
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
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nr,nc,ns,split,quad", [(32, 64, 4, 5, 2, 0), (24, 32, 3, 3, 2, 1),
                                                   (40, 64, 2, 4, 3, 0)])
def test_sample_groups_match_oracle(L, nr, nc, ns, split, quad):
    """Half-sweep launches per group of `split` samples (group-major; the last
    group shorter), with a sample frozen for a while, against the oracle over
    every walk shift."""
    old = _pinned({"MICSA_SWEEP_ZC": "4", "MICSA_SWEEP_PD": "2", "MICSA_SWEEP_SPLIT": str(split),
                   "MICSA_SWEEP_QUAD": str(quad), "MICSA_SWEEP_OCC": "4", "MICSA_RESIDENT": "0"})
    try:
        ctx = micsa.Context(L, nr, ns, nc)
        assert "split=%d" % split in ctx.tuning(), ctx.tuning()
    finally:
        _restore(old)
    rng = np.random.default_rng(23 * L + ns)
    st = random_state(rng, L, nr, nc, ns)
    frozen = ns - 2
    a, b, c = 3, L // 2, 2
    with ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ctx.iterate(a)
        ctx.set_active([0 if s == frozen else 1 for s in range(ns)])
        ctx.iterate(b)
        ctx.set_active(None)
        ctx.iterate(c)
        ctx.synchronize()
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            for _ in range(a + c + (0 if s == frozen else b)):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 8)
            ge, go = ctx.download_spins(s)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(ge, e) and np.array_equal(go, o), s
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s
