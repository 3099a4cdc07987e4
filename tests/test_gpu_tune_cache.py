"""Launch-shape choices reused across contexts of one shape in a process:
the second context takes the first one's choice and table without timing,
MICSA_TUNE_CACHE=0 times again, and the reused shape runs bit-exact."""
import numpy as np
import pytest

import micsa

pytestmark = pytest.mark.gpu


def _run(L, nr, ns, nc, seed):
    rng = np.random.default_rng(seed)
    H, V = (L // 4) ** 3 // 2, L ** 3
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s in range(ns):
            J = micsa.pack_couplings(L, *(rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, *(rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64,
                                               endpoint=True) for _ in range(2)))
            n = 2 * H * nc * nr
            ctx.upload_demons(s, *(rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64,
                                                endpoint=True) for _ in range(2)))
        ctx.iterate(3)
        return ctx.tuning(), [ctx.download_spins(s) for s in range(ns)]


def test_second_context_of_a_shape_reuses_the_choice(monkeypatch):
    monkeypatch.delenv("MICSA_TUNE_CACHE", raising=False)
    for k in ("ZC", "PD", "SPLIT", "OCC", "TMA", "ASYNC"):
        monkeypatch.delenv("MICSA_SWEEP_" + k, raising=False)
    L, nr, ns, nc = 40, 64, 2, 5  # a shape no other test creates
    t1, s1 = _run(L, nr, ns, nc, 1)
    t2, s2 = _run(L, nr, ns, nc, 1)
    head1, tab1 = t1.split("|")
    head2, tab2 = t2.split("|")
    assert "cached" not in head1 and head2.split() == head1.split() + ["cached"], (t1, t2)
    assert tab1 == tab2 and tab1.strip(), t2
    for a, b in zip(s1, s2):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    monkeypatch.setenv("MICSA_TUNE_CACHE", "0")
    t3, s3 = _run(L, nr, ns, nc, 1)
    assert "cached" not in t3.split("|")[0] and t3.split("|")[1].strip(), t3
    for a, b in zip(s1, s3):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
