"""Small lattices (L = 8, 16) run whole iterations in shared memory
(k_resident).  Its results must equal those of the per-half-sweep kernels
(the path every other L takes, MICSA_RESIDENT=0) bit for bit: spins, demons
in the frame of the walk, and energies, across a launch-chunk boundary."""
import os

import numpy as np
import pytest

import micsa
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


def _ctx(L, nr, ns, nc, resident, st):
    old = os.environ.get("MICSA_RESIDENT")
    os.environ["MICSA_RESIDENT"] = "1" if resident else "0"
    try:
        ctx = micsa.Context(L, nr, ns, nc)
    finally:
        if old is None:
            del os.environ["MICSA_RESIDENT"]
        else:
            os.environ["MICSA_RESIDENT"] = old
    for s, (J, e, o, w0, w1, _) in enumerate(st):
        ctx.upload_couplings(s, J)
        ctx.upload_spins(s, e, o)
        ctx.upload_demons(s, w0, w1)
    return ctx


@pytest.mark.parametrize("L,nr,nc,ns", [(8, 32, 6, 3), (8, 96, 1, 2), (16, 64, 6, 2), (16, 32, 3, 1)])
def test_resident_equals_half_sweep_kernels(L, nr, nc, ns):
    rng = np.random.default_rng(L * 100 + nr + nc)
    st = random_state(rng, L, nr, nc, ns)
    a = _ctx(L, nr, ns, nc, True, st)
    b = _ctx(L, nr, ns, nc, False, st)
    for n in (1, 6, 1030):
        a.iterate(n)
        b.iterate(n)
        ma, mb = a.measure(), b.measure()
        assert np.array_equal(ma["e_spin"], mb["e_spin"]), n
        assert np.array_equal(ma["e_demon"], mb["e_demon"]), n
        for s in range(ns):
            for x, y in zip(a.download_spins(s) + a.download_demons(s),
                            b.download_spins(s) + b.download_demons(s)):
                assert np.array_equal(x, y), (n, s)
    a.close()
    b.close()


@pytest.mark.parametrize("L", [8, 24])
def test_frozen_sample_keeps_state_and_others_advance(L):
    """micsa_set_active: a frozen sample is untouched by iterations (both the
    resident and the per-half-sweep paths), measures as 0, and the running
    samples evolve exactly as in a context without it."""
    nr, nc, ns = 32, 3, 3
    rng = np.random.default_rng(L)
    st = random_state(rng, L, nr, nc, ns)
    a = _ctx(L, nr, ns, nc, True, st)
    before = a.download_spins(1) + a.download_demons(1)
    a.set_active([1, 0, 1])
    a.iterate(7)
    m = a.measure()
    assert (m["e_spin"][1] == 0).all() and (m["e_demon"][1] == 0).all()
    for x, y in zip(before, a.download_spins(1) + a.download_demons(1)):
        assert np.array_equal(x, y)
    b = _ctx(L, nr, 2, nc, True, [st[0], st[2]])
    b.iterate(7)
    mb = b.measure()
    assert np.array_equal(m["e_spin"][[0, 2]], mb["e_spin"])
    assert np.array_equal(m["e_demon"][[0, 2]], mb["e_demon"])
    for sa, sb in ((0, 0), (2, 1)):
        for x, y in zip(a.download_spins(sa) + a.download_demons(sa),
                        b.download_spins(sb) + b.download_demons(sb)):
            assert np.array_equal(x, y)
    a.set_active(None)
    a.iterate(1)
    a.close()
    b.close()
