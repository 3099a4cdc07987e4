"""Host-side observables and schedules beyond the reference: the integral
estimators of the correlation length from C4 (I_k = sum r^k C4(r),
xi_{k,k+1} = I_{k+1}/I_k), and the linear beta schedule of a job."""
import ctypes as C

import numpy as np

import micsa


def test_correlation_lengths_match_numpy():
    L, npairs = 16, 5
    nd = L // 2 + 1
    rng = np.random.default_rng(4)
    r = np.arange(nd)
    base = np.exp(-r / 2.5) * L ** 3
    c4 = np.rint(base[None, None, :] * rng.uniform(0.8, 1.2, size=(npairs, 3, nd))).astype(np.int64)
    C4r, x12, x23 = micsa.correlation_lengths(L, c4)
    want = c4.sum(axis=(0, 1)) / (L ** 3 * 3.0 * npairs)
    assert np.allclose(C4r, want, rtol=1e-15, atol=0)
    I1, I2, I3 = (r * want).sum(), ((r ** 2) * want).sum(), ((r ** 3) * want).sum()
    assert abs(x12 - I2 / I1) < 1e-12 * x12 and abs(x23 - I3 / I2) < 1e-12 * x23
    assert 1.0 < x12 < x23  # a decaying correlation: xi23 > xi12


def test_correlation_length_of_uncorrelated_field_is_zero():
    L = 8
    c4 = np.zeros((2, 3, L // 2 + 1), np.int64)
    c4[:, :, 0] = L ** 3  # only the r = 0 term
    _, x12, x23 = micsa.correlation_lengths(L, c4)
    assert x12 == 0.0 and x23 == 0.0


def test_job_beta_schedule():
    f = micsa.lib().micsa_job_beta
    j = micsa.Job(16, 32, 6, 4096, 1, 2, 0.1, 1.5)
    assert f(C.byref(j), 0) == 0.1 and abs(f(C.byref(j), 4096) - 1.5) < 1e-15
    assert abs(f(C.byref(j), 1024) - (0.1 + 1.4 / 4)) < 1e-15
    const = micsa.Job(16, 32, 6, 4096, 1, 2, 0.9, 0.0)
    assert f(C.byref(const), 2048) == 0.9
