"""Serving (micsa_serve): requests arriving over time are continuously
batched into per-shape slot pools.  Each request's measurements must be the
same in the mix as alone (micsa_run_batch of that one job), bit for bit,
also when few slots force requests to wait and reuse freed slots."""
import numpy as np
import pytest

import micsa

pytestmark = pytest.mark.gpu

BETA = 0.9090909090909


def _trace(n, seed):
    rng = np.random.default_rng(seed)
    shapes = [(8, 32), (16, 64), (24, 32), (16, 32)]
    t, out = 0.0, []
    for k in range(n):
        t += rng.exponential(0.004)
        L, nr = shapes[rng.integers(len(shapes))]
        out.append(dict(arrival=t, L=L, nr=nr, nc=3, iterations=int(rng.integers(3, 80)),
                        seed_J=int(rng.integers(1, 2 ** 62)), seed_u=int(rng.integers(1, 2 ** 62)),
                        beta=BETA))
    return out


@pytest.mark.parametrize("slots_max,chunk", [(2, 0), (64, 5)])
def test_served_results_equal_alone(slots_max, chunk):
    reqs = _trace(14, 7 + slots_max)
    es, ed, times, sec = micsa.serve(reqs, slots_max=slots_max, chunk=chunk)
    assert sec > 0
    for j, r in enumerate(reqs):
        job = {k: r[k] for k in ("L", "nr", "nc", "iterations", "seed_J", "seed_u", "beta")}
        e1, d1, _ = micsa.run_batch([job])
        assert np.array_equal(es[j], e1[0]) and np.array_equal(ed[j], d1[0]), j
        prepared, admitted, finished = times[j]
        assert r["arrival"] <= prepared <= admitted <= finished, (j, r["arrival"], times[j])
