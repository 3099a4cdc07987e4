"""The mixed-lattice launch (micsa_multi_*): one dataflow launch per
iteration over the samples of several contexts of different L, against the
oracle -- every group's spins and demons bit-exact after more iterations
than half the smallest lattice side (every walk shift), with frozen samples
inside and at the end of a group's running prefix, a group with fewer
demon planes, and the shape pinned as well as tuned."""
import os

import numpy as np
import pytest

import micsa
import oracle
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


def _groups(shapes, seed):
    rng = np.random.default_rng(seed)
    ctxs, states = [], []
    for L, nr, nc, ns in shapes:
        ctxs.append(micsa.Context(L, nr, ns, nc))
        states.append(random_state(rng, L, nr, nc, ns, consistent=True))
    return ctxs, states


def _upload(ctx, st):
    for s, (J, e, o, w0, w1, _) in enumerate(st):
        ctx.upload_couplings(s, J)
        ctx.upload_spins(s, e, o)
        ctx.upload_demons(s, w0, w1)


def _check(ctx, st, L, nr, nc, iters, frozen=()):
    for s, (J, e, o, w0, w1, _) in enumerate(st):
        if s not in frozen:
            for _ in range(iters):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 16)
        ge, go = ctx.download_spins(s)
        g0, g1 = ctx.download_demons(s)
        assert np.array_equal(ge, e) and np.array_equal(go, o), (L, s)
        assert np.array_equal(g0, w0) and np.array_equal(g1, w1), (L, s)


@pytest.mark.parametrize("shapes,iters,pin", [
    # the batched stream's sizes, 64 replicas; tuned shape (L <= 16 on their resident kernel)
    ([(8, 64, 6, 3), (16, 64, 6, 2), (24, 64, 6, 2), (32, 64, 6, 1), (48, 64, 6, 1)], 13, {}),
    # every group in the launch, several samples per tile at L = 8 and 16, 4 iterations per
    # launch (9 = one launch of 4 and remainders of 3 and 2), walks wrapping inside a launch
    ([(8, 64, 6, 3), (16, 64, 6, 2), (24, 64, 6, 2), (32, 64, 6, 1)], 9,
     {"MICSA_MULTI_RESIDENT": "0", "MICSA_MULTI_ITERS": "4", "MICSA_MULTI_ZC": "4"}),
    # 32 replicas, a group with 3 demon planes, pinned slab depth 2, in the launch
    ([(8, 32, 6, 2), (16, 32, 3, 2), (40, 32, 6, 1)], 9,
     {"MICSA_MULTI_ZC": "2", "MICSA_MULTI_RESIDENT": "0"}),
    # 128 replicas (two word groups of 64), slab depth 4, 16 iterations per launch
    ([(16, 128, 6, 2), (24, 128, 6, 1)], 7,
     {"MICSA_MULTI_ZC": "4", "MICSA_MULTI_ITERS": "16", "MICSA_MULTI_RESIDENT": "0"}),
])
def test_mixed_launch_matches_oracle(shapes, iters, pin):
    old = {k: os.environ.get(k) for k in pin}
    os.environ.update(pin)
    try:
        ctxs, states = _groups(shapes, seed=sum(s[0] for s in shapes))
        multi = micsa.Multi(ctxs)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    with multi:
        rep = multi.report()
        assert rep.startswith("occ="), rep
        for ctx, st in zip(ctxs, states):
            _upload(ctx, st)
        # freeze sample 0 of the first group (inside the running prefix)
        # and the last sample of the second (the prefix shrinks)
        f0 = [0] + [1] * (shapes[0][3] - 1)
        ctxs[0].set_active(f0)
        f1 = [1] * (shapes[1][3] - 1) + [0]
        ctxs[1].set_active(f1)
        multi.iterate(iters - 2)
        multi.iterate(2)
        multi.synchronize()
        assert multi.kernel_launches() > 0
        for k, (ctx, st, (L, nr, nc, ns)) in enumerate(zip(ctxs, states, shapes)):
            frozen = {0} if k == 0 else ({ns - 1} if k == 1 else set())
            _check(ctx, st, L, nr, nc, iters, frozen)
            # measurements on the contexts are ordered after the mixed launches
            m = ctx.measure(spin=True, demon=True)
            for s, (J, e, o, w0, w1, _) in enumerate(st):
                if s not in frozen:
                    assert np.array_equal(m["e_spin"][s], oracle.energy(L, nr, J, e, o))
    for c in ctxs:
        c.close()


def test_mixed_launch_interleaves_with_per_context_iterations():
    """micsa_iterate on one context and the mixed launch over both, in any
    order, give the oracle's states (the launch waits for each context's
    queued work, and the contexts' later work waits for it)."""
    shapes = [(16, 64, 6, 2), (32, 64, 6, 1)]
    ctxs, states = _groups(shapes, seed=5)
    with micsa.Multi(ctxs) as multi:
        for ctx, st in zip(ctxs, states):
            _upload(ctx, st)
        ctxs[0].iterate(3)
        multi.iterate(2)
        ctxs[1].iterate(1)
        multi.iterate(1)
        ctxs[0].synchronize()
        ctxs[1].synchronize()
        _check(ctxs[0], states[0], 16, 64, 6, 6)
        _check(ctxs[1], states[1], 32, 64, 6, 4)
    for c in ctxs:
        c.close()


def test_mixed_launch_refuses_mismatched_contexts():
    a = micsa.Context(16, 32, 1, 6)
    b = micsa.Context(16, 64, 1, 6)
    with pytest.raises(micsa.MicsaError, match="replica words"):
        micsa.Multi([a, b])
    with pytest.raises(micsa.MicsaError, match="twice"):
        micsa.Multi([a, a])
    a.close()
    b.close()
