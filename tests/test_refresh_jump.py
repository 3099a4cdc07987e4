"""Jump-ahead of the demon-refresh streams (host/micsa_jump.c) against plain
sequential stepping of the reference's generators: the stream structs after
n draws must match byte for byte, and the demons drawn segment by segment
(what one GPU lane does) must equal InitWalkers' sequential draw
(micsa_draw_demons, ini.c:712-781)."""
import ctypes as C

import numpy as np
import pytest

import micsa


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _streams(seeds):
    prc, xo = (micsa.PRC * len(seeds))(), (micsa.Xoshiro * len(seeds))()
    for i, s in enumerate(seeds):
        k = C.c_uint32()
        micsa.lib().micsa_init_cpu_generators(C.byref(prc[i]), C.byref(xo[i]), C.byref(k), s)
    return prc, xo


def test_xoshiro_characteristic_polynomial_has_degree_256():
    p = np.zeros(5, np.uint64)
    micsa.lib().micsa_xoshiro_charpoly(_p(p))
    assert int(p[4]) == 1 and int(p[0]) & 1 == 1  # monic of degree 256, X does not divide it


@pytest.mark.parametrize("n", [1, 61, 300, 512, 513, 1000, 3072, 98304, 1234567])
def test_advance_equals_sequential_steps(n):
    lib = micsa.lib()
    (a, b), (c, d) = _streams([0xABC + n]), _streams([0xABC + n])
    left = n
    while left:  # up to 512 draws at a time are plain steps
        s = min(left, 512)
        lib.micsa_streams_advance(C.byref(a[0]), C.byref(b[0]), s)
        left -= s
    lib.micsa_streams_advance(C.byref(c[0]), C.byref(d[0]), n)
    assert bytes(a) == bytes(c) and bytes(b) == bytes(d)


def test_lcg_jump_composes():
    lib = micsa.lib()
    m, a = C.c_uint64(), C.c_uint64()
    lib.micsa_lcg_jump(1000, C.byref(m), C.byref(a))
    z = z0 = 0x0123456789ABCDEF
    for _ in range(1000):
        z = (z * 3202034522624059733 + 1) % 2 ** 64
    assert (m.value * z0 + a.value) % 2 ** 64 == z


@pytest.mark.parametrize("L,nc,wps", [(8, 6, 1), (8, 1, 3), (16, 6, 7), (16, 3, 32), (24, 5, 5)])
def test_segments_equal_sequential_refresh(L, nc, wps):
    lib = micsa.lib()
    thr = micsa.thresholds(0.9090909090909)
    H = lib.micsa_half_words(L)
    nw, nr = 2 * H * nc, 32
    plan = micsa.RefreshPlan()
    assert lib.micsa_refresh_plan_make(nw, wps, C.byref(plan)) == 0
    try:
        for r in (0, 13, 31):
            (a, b), (c, d) = _streams([77 + r]), _streams([77 + r])
            w0, w1 = np.zeros(nw * nr, np.uint64), np.zeros(nw * nr, np.uint64)
            lib.micsa_draw_demons(C.byref(a[0]), C.byref(b[0]), _p(thr), L, nr, nc, r, _p(w0), _p(w1))
            rec = np.zeros(micsa.STREAM_REC, np.uint64)
            assert lib.micsa_stream_record(C.byref(c[0]), C.byref(d[0]), _p(rec)) == 0
            v0, v1 = np.zeros_like(w0), np.zeros_like(w1)
            for g in range(plan.nseg):
                lib.micsa_draw_segment(C.byref(plan), g, _p(rec), _p(thr), nr, r, _p(v0), _p(v1))
            assert np.array_equal(v0, w0) and np.array_equal(v1, w1)
            lib.micsa_streams_advance_plan(C.byref(plan), C.byref(c[0]), C.byref(d[0]))
            assert bytes(a) == bytes(c) and bytes(b) == bytes(d)
    finally:
        lib.micsa_refresh_plan_free(C.byref(plan))


def test_stream_record_rejects_foreign_ring_pointers():
    prc, xo = _streams([5])
    prc[0].ip1 = (prc[0].ip1 + 1) % 256
    rec = np.zeros(micsa.STREAM_REC, np.uint64)
    assert micsa.lib().micsa_stream_record(C.byref(prc[0]), C.byref(xo[0]), _p(rec)) == -1
