"""The dataflow sweep -- all 2*nc half-sweeps of an iteration in one launch,
one block per tile, tiles ordered by per-slab completion counters instead of
launch boundaries -- pinned on, against the oracle: over more iterations
than half the lattice side (every walk shift, and the counters reset by
every launch), with 32, 64, 96 and 128 replicas, one, two, three slabs and
many, default and whole-row blocks, both register budgets, tiles taken
sample-major and half-sweep-major, frozen samples, and the headline shape."""
import os

import numpy as np
import pytest

import micsa
import oracle
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


def _context(L, nr, ns, nc, zc, pd=0, occ=3, tile=None, split=1, fit=1, pers=0, half=0, xs=0):
    env = {"MICSA_SWEEP_ZC": str(zc), "MICSA_SWEEP_PD": str(pd), "MICSA_SWEEP_FLOW": "1",
           "MICSA_SWEEP_OCC": str(occ), "MICSA_SWEEP_SPLIT": str(split), "MICSA_RESIDENT": "0",
           "MICSA_FLOW_ITERS": str(fit), "MICSA_SWEEP_PERS": str(pers), "MICSA_FLOW_HALF": str(half),
           "MICSA_FLOW_XS": str(xs)}
    if tile:
        env["MICSA_SWEEP_TILE"] = tile
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        ctx = micsa.Context(L, nr, ns, nc)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    assert ("load=pflow" if pers else "load=flow") in ctx.tuning(), ctx.tuning()
    return ctx


def _upload(ctx, st):
    for s, (J, e, o, w0, w1, _) in enumerate(st):
        ctx.upload_couplings(s, J)
        ctx.upload_spins(s, e, o)
        ctx.upload_demons(s, w0, w1)


def _check(ctx, st, L, nr, nc, iters, samples=None):
    for s, (J, e, o, w0, w1, _) in enumerate(st):
        if samples is not None and s not in samples:
            continue
        for _ in range(iters):
            oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 8)
        ge, go = ctx.download_spins(s)
        g0, g1 = ctx.download_demons(s)
        assert np.array_equal(ge, e) and np.array_equal(go, o), s
        assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s


@pytest.mark.parametrize("L,nr,nc,ns,zc,pd,occ,tile,split", [
    (32, 64, 6, 2, 4, 2, 4, None, 1),     # 8 slabs, the headline replica count
    (32, 64, 6, 3, 4, 2, 4, None, 0),
    (64, 128, 6, 2, 8, 4, 3, None, 1),    # four-word vectors
    (40, 96, 3, 3, 8, 0, 4, None, 0),     # three word groups of one word, 5 slabs
    (96, 64, 5, 2, 2, 0, 4, "row", 1),    # whole-row blocks, 48 slabs
    (24, 32, 2, 2, 8, 0, 3, None, 0),     # 3 slabs: every slab depends on every slab
    (16, 64, 6, 1, 16, 0, 3, None, 1),    # one slab
    (32, 32, 1, 4, 16, 0, 4, None, 0),    # nc = 1, 2 slabs
    (40, 96, 3, 3, 2, 0, 3, None, 1),
    (96, 64, 5, 2, 4, 2, 3, "row", 0),
    (32, 256, 6, 1, 4, 0, 3, None, 1),    # two word groups of four-word vectors
])
def test_flow_sweep_matches_oracle(L, nr, nc, ns, zc, pd, occ, tile, split):
    ctx = _context(L, nr, ns, nc, zc, pd, occ, tile, split)
    rng = np.random.default_rng(17 * L + nr + ns + zc)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
        _upload(ctx, st)
        ctx.iterate(iters)
        ctx.synchronize()  # also reports any dependency wait that timed out
        _check(ctx, st, L, nr, nc, iters)


@pytest.mark.parametrize("occ,split", [(3, 1), (4, 0)])
def test_flow_sweep_frozen_sample_untouched(occ, split):
    """micsa_set_active with the dataflow sweep: a frozen sample's tiles are
    skipped (its counters still advance, so later tiles do not wait on it)
    and its state stays as it was; after it is unfrozen it continues like
    the oracle."""
    L, nr, nc, ns = 32, 64, 4, 3
    ctx = _context(L, nr, ns, nc, 4, 2, occ, split=split)
    rng = np.random.default_rng(23 + occ)
    st = random_state(rng, L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(5)
        ctx.set_active([1, 0, 1])
        ctx.iterate(7)
        ctx.set_active(None)
        ctx.iterate(4)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 16, samples=(0, 2))
        _check(ctx, st, L, nr, nc, 9, samples=(1,))


def test_flow_sweep_headline_shape():
    """L=160, 2 samples x 64 replicas, nc=6 (the benchmark's shape, with its
    whole-row blocks and 8-plane slabs), two iterations against the oracle."""
    L, nr, nc, ns = 160, 64, 6, 2
    ctx = _context(L, nr, ns, nc, 8, 2, 3, "row")
    rng = np.random.default_rng(160)
    st = random_state(rng, L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(2)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 2)


def test_dataflow_wait_that_runs_out_is_reported_and_the_gpu_stays_usable():
    """The dataflow sweep's dependency waits are bounded.  With every wait's
    target raised out of reach (a count nothing produces) and a 1 ms limit,
    the first wait runs out, every later wait of the launch gives up at once,
    the launch finishes, and micsa_synchronize turns the count into an error
    with a message; nothing faults or hangs.  With the waits restored, a new
    context on the same GPU runs bit-exact against the oracle."""
    import torch
    L, nr, nc, ns = 32, 64, 6, 2
    st = random_state(np.random.default_rng(71), L, nr, nc, ns)
    with _context(L, nr, ns, nc, zc=4, pd=2, occ=4) as ctx:
        _upload(ctx, st)
        lib = micsa.lib()
        assert lib.micsa_debug_flow_waits(ctx.h, 1000000, 1) == micsa.MICSA_OK
        try:
            ctx.iterate(1)
            rc = lib.micsa_synchronize(ctx.h)
            msg = lib.micsa_last_error(ctx.h).decode()
        finally:
            assert lib.micsa_debug_flow_waits(ctx.h, 0, 0) == micsa.MICSA_OK
        assert rc == micsa.MICSA_ERR_CUDA and "timed out" in msg, (rc, msg)
        assert lib.micsa_synchronize(ctx.h) == micsa.MICSA_OK  # reported once, then cleared
    torch.cuda.synchronize()  # the context of the device still answers
    st = random_state(np.random.default_rng(72), L, nr, nc, ns)
    with _context(L, nr, ns, nc, zc=4, pd=2, occ=4) as ctx:
        _upload(ctx, st)
        ctx.iterate(3)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 3)


@pytest.mark.parametrize("L,nr,nc,ns,zc,fit,iters,split", [
    (32, 64, 6, 2, 4, 4, 21, 1),    # 5 launches of 4 iterations and one of 1; walks wrap
    (24, 32, 2, 2, 8, 16, 37, 0),   # 3 slabs, 16 iterations per launch
    (16, 64, 6, 1, 16, 4, 9, 1),    # one slab
    (40, 96, 3, 3, 8, 16, 23, 0),   # three word groups
])
def test_flow_sweep_several_iterations_per_launch(L, nr, nc, ns, zc, fit, iters, split):
    """The dataflow sweep carrying several iterations per launch: half-sweep
    j of the launch is half-sweep j % 2nc of iteration j / 2nc, ordered by the
    same per-slab rule (which also orders the demon words the walk moves from
    one iteration to the next); the remainder runs as one launch of the
    remaining iterations, and micsa_monte_carlo stays one iteration."""
    ctx = _context(L, nr, ns, nc, zc, 0, 3, None, split, fit)
    assert "fit=%d" % fit in ctx.tuning(), ctx.tuning()
    rng = np.random.default_rng(5 * L + fit + ns)
    st = random_state(rng, L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(iters - 1)
        ctx.monte_carlo(1)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, iters)


def test_flow_sweep_several_iterations_frozen_and_headline():
    """16 iterations per launch with a frozen sample, then the headline
    shape (L=160, 2 x 64 replicas, whole-row blocks, 8-plane slabs) over one
    launch of 16 iterations and one more."""
    L, nr, nc, ns = 32, 64, 4, 3
    ctx = _context(L, nr, ns, nc, 4, 2, 3, split=1, fit=16)
    st = random_state(np.random.default_rng(41), L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(16)
        ctx.set_active([1, 0, 1])
        ctx.iterate(16)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 32, samples=(0, 2))
        _check(ctx, st, L, nr, nc, 16, samples=(1,))
    L, nr, nc, ns = 160, 64, 6, 2
    ctx = _context(L, nr, ns, nc, 8, 2, 3, "row", fit=16)
    st = random_state(np.random.default_rng(1600), L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(17)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 17)


@pytest.mark.parametrize("L,nr,nc,ns,zc,occ,fit,split,tile", [
    (32, 64, 6, 2, 4, 3, 1, 1, None),
    (32, 64, 6, 3, 4, 4, 4, 0, None),      # 4-block register budget, half-sweep-major
    (24, 32, 2, 2, 8, 3, 16, 0, None),     # 3 slabs
    (64, 128, 6, 2, 8, 3, 4, 1, None),     # four-word vectors
    (40, 96, 3, 3, 8, 3, 16, 1, None),     # three word groups
    (96, 64, 5, 2, 4, 3, 16, 1, "row"),    # whole-row blocks
])
def test_persistent_flow_sweep_matches_oracle(L, nr, nc, ns, zc, occ, fit, split, tile):
    """The persistent form of the dataflow sweep (blocks loop over tickets,
    each taking its next ticket during its current tile): same tiles, same
    order rule, same results -- with one and several iterations per launch,
    remainders as one launch of the remaining iterations, frozen samples."""
    ctx = _context(L, nr, ns, nc, zc, 2 if zc > 2 else 0, occ, tile, split, fit, pers=1)
    rng = np.random.default_rng(11 * L + nr + fit)
    st = random_state(rng, L, nr, nc, ns)
    iters = L // 2 + 3
    with ctx:
        _upload(ctx, st)
        ctx.iterate(iters - 2)
        ctx.set_active([0] + [1] * (ns - 1))
        ctx.iterate(2)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, iters, samples=range(1, ns))
        _check(ctx, st, L, nr, nc, iters - 2, samples=(0,))


def test_persistent_flow_sweep_headline_shape():
    L, nr, nc, ns = 160, 64, 6, 2
    ctx = _context(L, nr, ns, nc, 8, 2, 3, "row", fit=16, pers=1)
    st = random_state(np.random.default_rng(1601), L, nr, nc, ns)
    with ctx:
        _upload(ctx, st)
        ctx.iterate(17)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, 17)


@pytest.mark.parametrize("L,nr,nc,ns,zc,occ,fit,split,tile", [
    (32, 64, 6, 2, 4, 3, 4, 1, None),
    (40, 96, 3, 3, 8, 4, 1, 0, None),
    (96, 64, 5, 2, 4, 3, 16, 1, "row"),    # whole-row blocks of 3 rows
])
def test_flow_sweep_half_height_tiles(L, nr, nc, ns, zc, occ, fit, split, tile):
    """Half-height dataflow tiles (blocks of about 128 threads, twice as many
    per SM): the same rule over twice the tiles, same results as the oracle."""
    ctx = _context(L, nr, ns, nc, zc, 0, occ, tile, split, fit, half=1)
    assert "/2" in ctx.tuning(), ctx.tuning()
    st = random_state(np.random.default_rng(7 * L + fit + occ), L, nr, nc, ns)
    iters = L // 2 + 1
    with ctx:
        _upload(ctx, st)
        ctx.iterate(iters)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, iters)


@pytest.mark.parametrize("L,nr,nc,ns,zc,occ,fit,split,tile", [
    (32, 64, 6, 2, 4, 3, 4, 1, None),      # x blocks narrower than a row: block edges
    (40, 96, 3, 3, 8, 4, 1, 0, None),      # one-word groups; rows past L in the last tile
    (96, 64, 5, 2, 4, 3, 16, 1, "row"),    # 24 threads a row: rows straddle warps
    (64, 128, 6, 2, 8, 3, 4, 1, "row"),    # four-word vectors, 16 threads a row
    (24, 32, 2, 2, 8, 3, 2, 0, "row"),     # 6 threads a row, one word
])
def test_flow_sweep_x_halo_by_shuffle(L, nr, nc, ns, zc, occ, fit, split, tile):
    """The dataflow sweep taking the remaining x-neighbour word from the
    adjacent lane (warp shuffle) and loading it only at row ends, the periodic
    wrap and warp boundaries: same results as the oracle."""
    ctx = _context(L, nr, ns, nc, zc, 0, occ, tile, split, fit, xs=1)
    assert "+xs" in ctx.tuning(), ctx.tuning()
    st = random_state(np.random.default_rng(11 * L + fit + occ), L, nr, nc, ns)
    iters = L // 2 + 1
    with ctx:
        _upload(ctx, st)
        ctx.iterate(iters)
        ctx.synchronize()
        _check(ctx, st, L, nr, nc, iters)
