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


def _numpy_xi(L, c4, kappa, rmax=0):
    """The cut-off estimator restated in numpy: per-pair axis averages / V,
    their mean and standard error over pairs, integrals over r < r_cut."""
    nd = L // 2 + 1
    per_pair = c4.sum(axis=1) / (3.0 * L ** 3)  # [pairs, nd]
    C4 = per_pair.mean(axis=0)
    err = per_pair.std(axis=0, ddof=1) / np.sqrt(per_pair.shape[0])
    cut = nd if rmax <= 0 else min(nd, rmax + 1)
    for d in range(1, cut):
        if kappa > 0 and C4[d] < kappa * err[d]:
            cut = d
            break
    r = np.arange(cut)
    I1, I2, I3 = (((r ** k) * C4[:cut]).sum() for k in (1, 2, 3))
    return C4, err, I2 / I1, I3 / I2, cut


def test_correlation_lengths_stop_where_c4_sinks_into_its_noise():
    """A decaying C4 with pair-to-pair noise: the integrals stop at the first
    r where C4 < 3 x its standard error over the pairs; the tail beyond it,
    pure noise with large r^k weights, no longer moves xi.  Checked against
    a numpy restatement, and xi with the cut differs from the whole-range
    sum when the tail is noisy."""
    L, npairs = 32, 16
    nd = L // 2 + 1
    rng = np.random.default_rng(11)
    r = np.arange(nd)
    signal = np.exp(-r / 2.0) * L ** 3
    noise = rng.normal(0.0, 0.02 * L ** 3, size=(npairs, 3, nd))
    c4 = np.rint(signal[None, None, :] + noise).astype(np.int64)
    C4r, x12, x23, cut, err = micsa.correlation_lengths(L, c4, kappa=3.0, with_cut=True)
    wC4, werr, w12, w23, wcut = _numpy_xi(L, c4, 3.0)
    assert np.allclose(C4r, wC4, rtol=1e-13, atol=0) and np.allclose(err, werr, rtol=1e-9)
    assert cut == wcut and 2 <= cut < nd
    assert C4r[cut] < 3.0 * err[cut] and all(C4r[d] >= 3.0 * err[d] for d in range(1, cut))
    assert abs(x12 - w12) < 1e-12 * x12 and abs(x23 - w23) < 1e-12 * x23
    _, a12, _ = micsa.correlation_lengths(L, c4)  # whole range
    assert abs(a12 - x12) > 1e-3 * x12
    # an explicit r_max caps the range as well
    _, _, _, cut2, _ = micsa.correlation_lengths(L, c4, rmax=3, with_cut=True)
    assert cut2 == 4
    _, _, b12, _, _ = _numpy_xi(L, c4, 0.0, rmax=3)
    assert abs(micsa.correlation_lengths(L, c4, rmax=3)[1] - b12) < 1e-12 * b12


def test_correlation_length_cut_needs_two_pairs():
    """One replica pair gives no error estimate: the whole range is summed."""
    L = 16
    c4 = np.zeros((1, 3, L // 2 + 1), np.int64)
    c4[0, :, :4] = [L ** 3, L ** 3 // 2, L ** 3 // 4, L ** 3 // 8]
    _, x12, _, cut, _ = micsa.correlation_lengths(L, c4, kappa=3.0, with_cut=True)
    assert cut == L // 2 + 1 and x12 == micsa.correlation_lengths(L, c4)[1]
