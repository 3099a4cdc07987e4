"""Downloads into page-locked, mapped host buffers (converted straight into
them by the device) equal downloads into ordinary buffers (converted into a
device staging buffer, then copied), after iterations that move the walk."""
import ctypes as C

import numpy as np
import pytest

import micsa
import oracle
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


def _pinned(n):
    import torch
    t = torch.zeros(n, dtype=torch.int64, pin_memory=True)
    return t, t.numpy().view(np.uint64)


@pytest.mark.parametrize("L,nr,nc,ns,iters", [(16, 64, 6, 2, 5), (24, 32, 3, 1, 7), (32, 128, 2, 2, 3)])
def test_download_into_mapped_buffers_equals_staged(L, nr, nc, ns, iters):
    st = random_state(np.random.default_rng(3 * L + nr), L, nr, nc, ns)
    H = (L // 4) ** 3 // 2
    p64 = lambda v: v.ctypes.data_as(C.POINTER(C.c_uint64))
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ctx.iterate(iters)
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ge, go = ctx.download_spins(s)
            g0, g1 = ctx.download_demons(s)
            bufs = [_pinned(H * nr), _pinned(H * nr), _pinned(2 * H * nc * nr), _pinned(2 * H * nc * nr)]
            v = [b[1] for b in bufs]
            micsa.check(ctx.h, micsa.lib().micsa_download_spins(ctx.h, s, p64(v[0]), p64(v[1])), "spins")
            micsa.check(ctx.h, micsa.lib().micsa_download_demons(ctx.h, s, p64(v[2]), p64(v[3])), "demons")
            assert np.array_equal(v[0], ge) and np.array_equal(v[1], go), s
            assert np.array_equal(v[2], g0) and np.array_equal(v[3], g1), s
            for _ in range(iters):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 8)
            assert np.array_equal(v[0], e) and np.array_equal(v[1], o), s
            assert np.array_equal(v[2], w0) and np.array_equal(v[3], w1), s
