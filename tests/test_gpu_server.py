"""The long-lived server (micsa_server_create / micsa_submit / micsa_poll):
jobs submitted from the caller's loop, including while earlier ones run and
after the pools went idle, give the same measurements as the job run alone;
shapes the server does not serve and unknown ids are refused."""
import time

import numpy as np
import pytest

import micsa

pytestmark = pytest.mark.gpu

BETA = 0.9090909090909


def _job(L, nr, nc, it, seed, beta_end=0.0):
    return dict(L=L, nr=nr, nc=nc, iterations=it, seed_J=1000 + seed, seed_u=2000 + seed,
                beta=BETA, beta_end=beta_end)


def _alone(j):
    e, d, _ = micsa.run_batch([j])
    return e[0], d[0]


def test_submitted_jobs_equal_alone_in_waves():
    jobs = [_job(16, 64, 3, 40 + 7 * k, k) for k in range(5)] + \
           [_job(24, 32, 2, 20 + 3 * k, 10 + k) for k in range(3)] + [_job(16, 64, 3, 33, 20, 1.4)]
    with micsa.Server([(16, 64, 3, 3), (24, 32, 2)], slots_max=4, chunk=16) as sv:
        ids = [sv.submit(j) for j in jobs[:6]]
        got = {}
        # a second wave while the first runs
        ids += [sv.submit(j) for j in jobs[6:]]
        deadline = time.time() + 120
        while len(got) < len(ids) and time.time() < deadline:
            for i in ids:
                if i not in got:
                    r = sv.poll(i, timeout=0.05)
                    if r is not None:
                        got[i] = r
        assert len(got) == len(ids)
        # a third wave after the pools went idle
        late = _job(24, 32, 2, 17, 30)
        i = sv.submit(late)
        r = sv.poll(i, timeout=60.0)
        assert r is not None
        got[i] = r
        ids.append(i)
        jobs.append(late)
    for i, j in zip(ids, jobs):
        e, d, (prep, adm, fin) = got[i]
        e1, d1 = _alone(j)
        assert np.array_equal(e, e1) and np.array_equal(d, d1), (i, j)
        assert 0 <= prep <= adm <= fin, (i, prep, adm, fin)


def test_server_refuses_unserved_shapes_and_unknown_ids():
    with micsa.Server([(8, 32, 2)]) as sv:
        with pytest.raises(micsa.MicsaError, match="ERR_UNSUPPORTED"):
            sv.submit(_job(16, 32, 2, 5, 1))
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            sv.submit(_job(8, 32, 2, 0, 1))  # no iterations
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            sv.poll(12345)
        i = sv.submit(_job(8, 32, 2, 9, 2))
        assert sv.poll(i, timeout=60.0) is not None
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            sv.poll(i)  # released once polled done


def test_server_destroy_drains_unpolled_jobs():
    sv = micsa.Server([(16, 32, 2)], slots_max=2)
    for k in range(4):
        sv.submit(_job(16, 32, 2, 25, 40 + k))
    sv.close()  # returns once every submitted job has finished
