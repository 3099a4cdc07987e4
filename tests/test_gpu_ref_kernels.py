"""The reference's own CUDA kernels (d_oneMCstepBN_multisample, d_Walk of
PROGRAM/src/main.cu, compiled unmodified for sm_103a by
oracle/ref_gpu/build_ref_gpu.sh and driven by oracle/ref_gpu's harness as
Monte_Carlo drives them) on the GB300: they reproduce the oracle bit for
bit, and so does this library's sweep from the same state.  Skipped where
the cubins were not built (they need the reference sources)."""
import numpy as np
import pytest

import micsa
import oracle
from test_gpu_parity import random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L,nr,ns,nc,iters", [(16, 64, 2, 6, 5), (32, 64, 2, 4, 3)])
def test_reference_kernels_equal_oracle_and_this_library(L, nr, ns, nc, iters):
    cubin = oracle.ref_gpu_cubin(L, nr, 2)
    if cubin is None:
        pytest.skip("reference kernels not built (no reference sources where build() ran)")
    st = random_state(np.random.default_rng(L + 3 * nc), L, nr, nc, ns, consistent=True)
    ref = oracle.RefGPU(cubin, L, nr, ns, nc)
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            ref.upload(s, J, e, o, w0, w1)
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
            ctx.upload_demons(s, w0, w1)
        ref.iterate(iters)
        ctx.iterate(iters)
        for s, (J, e, o, w0, w1, _) in enumerate(st):
            for _ in range(iters):
                oracle.micsa_iteration(L, nr, nc, J, e, o, w0, w1, 16)
            got_ref = ref.download(s)
            got = ctx.download_spins(s) + ctx.download_demons(s)
            for name, a, b, c in zip(("even", "odd", "w0", "w1"), got_ref, got, (e, o, w0, w1)):
                assert np.array_equal(a, c), "reference kernels vs oracle: %s, sample %d" % (name, s)
                assert np.array_equal(b, c), "this library vs oracle: %s, sample %d" % (name, s)
    ref.close()
