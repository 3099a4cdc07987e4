"""Batched runs (micsa_run_batch): many independent reference runs of one
shape share one context.  Each job's energies must equal (a) those of the
same job run alone and (b) the oracle running that job on the reference's
schedule (refresh at t = 0 and powers of two, measurements at powers of two
and at the end), with the job's host initialisation."""
import numpy as np
import pytest

import micsa
import oracle

pytestmark = pytest.mark.gpu

BETA = 0.9090909090909


@pytest.fixture(params=["groups", "multi"])
def batch_mode(request, monkeypatch):
    """groups: each shape group on its own stream and host thread; multi:
    all groups in lockstep, their iterations as mixed-lattice launches."""
    monkeypatch.setenv("MICSA_BATCH", request.param)
    return request.param


def _jobs(n, L, nr, nc, iters, base):
    return [dict(L=L, nr=nr, nc=nc, iterations=iters, seed_J=base + 101 * j + 1,
                 seed_u=base + 7 * j + 3, beta=BETA) for j in range(n)]


@pytest.mark.parametrize("L,nr,nc,iters,n", [(8, 32, 6, 37, 6), (16, 64, 3, 16, 3), (24, 32, 2, 9, 4)])
def test_batch_equals_jobs_run_alone(L, nr, nc, iters, n):
    jobs = _jobs(n, L, nr, nc, iters, 1000 * L)
    es, ed, _ = micsa.run_batch(jobs)
    assert es[0].shape == (micsa.lib().micsa_job_measurements(iters), nr)
    for j in range(n):
        e1, d1, _ = micsa.run_batch([jobs[j]])
        assert np.array_equal(es[j], e1[0]) and np.array_equal(ed[j], d1[0]), j
    assert not np.array_equal(es[0], es[1])  # distinct seeds, distinct runs


def _oracle_job(job):
    L, nr, nc = job["L"], job["nr"], job["nc"]
    hm = micsa.HostModel(L, nr, nc, 1, job["seed_u"], [1] * nr, [0], beta=job["beta"])
    Jx, Jy, Jz, _ = micsa.couplings_janus(job["seed_J"], L)
    J = micsa.pack_couplings(L, Jx, Jy, Jz)
    even, odd = hm.spins[0][0].copy(), hm.spins[0][1].copy()
    out_s, out_d = [], []
    t, w0, w1 = 0, None, None
    while t < job["iterations"]:
        if t & (t - 1) == 0:
            w0, w1 = hm.draw_demons(0)
        nxt = 1
        while nxt <= t:
            nxt <<= 1
        nxt = min(nxt, job["iterations"])
        for _ in range(nxt - t):
            oracle.micsa_iteration(L, nr, nc, J, even, odd, w0, w1, 8)
        t = nxt
        if t & (t - 1) == 0 or t == job["iterations"]:
            out_s.append(oracle.energy(L, nr, J, even, odd))
            out_d.append(oracle.demon_energy(L, nr, nc, w0, w1))
    return np.array(out_s), np.array(out_d)


def test_batch_job_equals_oracle_on_reference_schedule(batch_mode):
    jobs = _jobs(3, 8, 32, 6, 21, 77)
    es, ed, _ = micsa.run_batch(jobs)
    for j in range(3):
        os_, od = _oracle_job(jobs[j])
        assert np.array_equal(es[j], os_.astype(np.int32)), j
        assert np.array_equal(ed[j], od.astype(np.uint64)), j


def test_batch_mixed_shapes_and_lengths_equal_alone(batch_mode, monkeypatch):
    """Uneven L, replica counts and iteration counts in one call: shape
    groups run concurrently (or in lockstep through the mixed-lattice
    launch), jobs finish at their own lengths; each job equals the job run
    alone in the other mode as well."""
    shapes = [(8, 32, 37), (16, 64, 64), (24, 32, 20), (8, 32, 5), (16, 64, 9), (24, 32, 64),
              (8, 32, 64), (40, 32, 3)]
    jobs = [dict(L=L, nr=nr, nc=4, iterations=it, seed_J=900 + 17 * k, seed_u=55 + 3 * k, beta=BETA)
            for k, (L, nr, it) in enumerate(shapes)]
    es, ed, _ = micsa.run_batch(jobs)
    monkeypatch.setenv("MICSA_BATCH", "groups" if batch_mode == "multi" else "multi")
    for j, job in enumerate(jobs):
        e1, d1, _ = micsa.run_batch([job])
        assert es[j].shape == (micsa.lib().micsa_job_measurements(job["iterations"]), job["nr"])
        assert np.array_equal(es[j], e1[0]) and np.array_equal(ed[j], d1[0]), j


def test_batch_rejects_invalid_job():
    jobs = _jobs(2, 8, 32, 6, 4, 5)
    jobs[1]["L"] = 12
    with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
        micsa.run_batch(jobs)


def test_batch_512_samples_headline_batched_shape():
    """512 samples at L=16, 64 replicas, 2^10 iterations: the batched
    configuration, spot-checked against single runs of three jobs."""
    jobs = _jobs(512, 16, 64, 6, 1024, 20260101)
    es, ed, sec = micsa.run_batch(jobs)
    assert sec > 0 and len(es) == 512 and es[0].shape == (11, 64)
    for j in (0, 255, 511):
        e1, d1, _ = micsa.run_batch([jobs[j]])
        assert np.array_equal(es[j], e1[0]) and np.array_equal(ed[j], d1[0]), j


def test_batch_beta_schedule_equals_alone_and_oracle(batch_mode):
    """Linear beta schedule (an extension: the reference has one beta): each
    refresh draws the demons at beta(t); the batch equals the jobs alone and
    the oracle with the thresholds recomputed at every refresh."""
    jobs = [dict(L=8, nr=32, nc=6, iterations=it, seed_J=31 + k, seed_u=41 + k, beta=0.1,
                 beta_end=1.5) for k, it in enumerate((40, 17, 40))]
    es, ed, _ = micsa.run_batch(jobs)
    for j, job in enumerate(jobs):
        e1, d1, _ = micsa.run_batch([job])
        assert np.array_equal(es[j], e1[0]) and np.array_equal(ed[j], d1[0]), j
    job = jobs[0]
    L, nr, nc = job["L"], job["nr"], job["nc"]
    hm = micsa.HostModel(L, nr, nc, 1, job["seed_u"], [1] * nr, [0], beta=job["beta"])
    J = micsa.pack_couplings(L, *micsa.couplings_janus(job["seed_J"], L)[:3])
    even, odd = hm.spins[0][0].copy(), hm.spins[0][1].copy()
    out, t = [], 0
    while t < job["iterations"]:
        if t & (t - 1) == 0:
            b = job["beta"] + (job["beta_end"] - job["beta"]) * t / job["iterations"]
            hm.thr = micsa.thresholds(b)
            w0, w1 = hm.draw_demons(0)
        nxt = 1
        while nxt <= t:
            nxt <<= 1
        nxt = min(nxt, job["iterations"])
        for _ in range(nxt - t):
            oracle.micsa_iteration(L, nr, nc, J, even, odd, w0, w1, 8)
        t = nxt
        if t & (t - 1) == 0 or t == job["iterations"]:
            out.append(oracle.demon_energy(L, nr, nc, w0, w1))
    assert np.array_equal(ed[0], np.array(out).astype(np.uint64))
