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
