"""Demon refresh drawn on the GPU (micsa_refresh_demons) against the host
restatement of InitWalkers (ini.c:712-781, micsa_draw_demons_all, itself
pinned to the reference through the golden runs): every demon word and every
byte of the advanced stream structs must be equal."""
import ctypes as C

import numpy as np
import pytest

import micsa

pytestmark = pytest.mark.gpu

BETA = 0.9090909090909


def _streams(n, base):
    prc, xo = (micsa.PRC * n)(), (micsa.Xoshiro * n)()
    for i in range(n):
        k = C.c_uint32()
        micsa.lib().micsa_init_cpu_generators(C.byref(prc[i]), C.byref(xo[i]), C.byref(k),
                                              base + 7919 * i)
    return prc, xo


def _copy(arr, typ):
    out = (typ * len(arr))()
    C.memmove(out, arr, C.sizeof(arr))
    return out


def _host_draw(L, nr, nc, prc, xo, s, thr):
    """InitWalkers on the host for sample s of [ns][nr] stream arrays."""
    n = 2 * ((L // 4) ** 3 // 2) * nc * nr
    w0, w1 = np.zeros(n, np.uint64), np.zeros(n, np.uint64)
    sl_p = (micsa.PRC * nr).from_buffer(prc, s * nr * C.sizeof(micsa.PRC))
    sl_x = (micsa.Xoshiro * nr).from_buffer(xo, s * nr * C.sizeof(micsa.Xoshiro))
    p64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint64))
    assert micsa.lib().micsa_draw_demons_all(sl_p, sl_x, p64(thr), L, nr, nc, p64(w0), p64(w1), 16) == 0
    return w0, w1


@pytest.mark.parametrize("L,nr,nc,ns", [(8, 32, 6, 1), (16, 64, 3, 2), (24, 96, 5, 3), (40, 32, 6, 2),
                                        (16, 32, 1, 4)])
def test_gpu_refresh_equals_host_draw_twice(L, nr, nc, ns):
    thr = micsa.thresholds(BETA)
    prc, xo = _streams(ns * nr, 1000 + L)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    with micsa.Context(L, nr, ns, nc) as ctx:
        for rnd in range(2):  # the second refresh continues the streams
            ctx.refresh_demons(0, prc, xo, thr)
            for s in range(ns):
                w0, w1 = _host_draw(L, nr, nc, hp, hx, s, thr)
                g0, g1 = ctx.download_demons(s)
                assert np.array_equal(g0, w0) and np.array_equal(g1, w1), (rnd, s)
            assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx), rnd


@pytest.mark.parametrize("order", [(2, 1, 0), (1, 0, 2), (0, 0, 1)])
def test_gpu_refresh_thresholds_in_any_order(order):
    """The kernel counts the thresholds above each draw as InitWalkers does,
    so thresholds that are not ascending (no beta gives them) still give
    InitWalkers' demons."""
    L, nr, nc, ns = 16, 64, 2, 2
    t = micsa.thresholds(BETA)
    thr = np.array([t[i] for i in order], dtype=np.uint64)
    prc, xo = _streams(ns * nr, 2024)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    with micsa.Context(L, nr, ns, nc) as ctx:
        ctx.refresh_demons(0, prc, xo, thr)
        for s in range(ns):
            w0, w1 = _host_draw(L, nr, nc, hp, hx, s, thr)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s
    assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx)


@pytest.mark.parametrize("wps", ["3", "128"])
def test_gpu_refresh_segment_lengths(monkeypatch, wps):
    """Pinned segment lengths (MICSA_REFRESH_WPS) change only the launch."""
    monkeypatch.setenv("MICSA_REFRESH_WPS", wps)
    L, nr, nc, ns = 32, 64, 3, 1
    thr = micsa.thresholds(BETA)
    prc, xo = _streams(ns * nr, 555)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    with micsa.Context(L, nr, ns, nc) as ctx:
        for rnd in range(2):
            ctx.refresh_demons(0, prc, xo, thr)
            w0, w1 = _host_draw(L, nr, nc, hp, hx, 0, thr)
            g0, g1 = ctx.download_demons(0)
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), rnd
            assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx), rnd


def test_gpu_refresh_part_of_the_samples_after_walks():
    """A refresh of samples [1, 3) resets their walk and leaves sample 0."""
    L, nr, nc, ns = 16, 32, 6, 3
    thr = micsa.thresholds(BETA)
    rng = np.random.default_rng(3)
    H, V = (L // 4) ** 3 // 2, L ** 3
    prc, xo = _streams(ns * nr, 99)
    with micsa.Context(L, nr, ns, nc) as ctx:
        for s in range(ns):
            J = micsa.pack_couplings(L, *(rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, *(rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64,
                                               endpoint=True) for _ in range(2)))
        ctx.refresh_demons(0, prc, xo, thr)
        ctx.iterate(5)  # walk = 5 on every sample
        keep0 = ctx.download_demons(0)
        part_p = (micsa.PRC * (2 * nr)).from_buffer(prc, nr * C.sizeof(micsa.PRC))
        part_x = (micsa.Xoshiro * (2 * nr)).from_buffer(xo, nr * C.sizeof(micsa.Xoshiro))
        hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
        ctx.refresh_demons(1, part_p, part_x, thr)
        g = ctx.download_demons(0)
        assert np.array_equal(g[0], keep0[0]) and np.array_equal(g[1], keep0[1])
        for s in (1, 2):
            w0, w1 = _host_draw(L, nr, nc, hp, hx, s, thr)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s
        ctx.iterate(1)
        ctx.synchronize()


def test_gpu_refresh_rejects_bad_arguments_without_change():
    L, nr, nc = 8, 32, 2
    thr = micsa.thresholds(BETA)
    prc, xo = _streams(nr, 5)
    before = bytes(prc)
    with micsa.Context(L, nr, 1, nc) as ctx:
        prc[3].ip2 = (prc[3].ip2 + 1) % 256
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            ctx.refresh_demons(0, prc, xo, thr)
        prc[3].ip2 = (prc[3].ip2 - 1) % 256
        assert bytes(prc) == before
        with pytest.raises(micsa.MicsaError, match="ERR_ARG"):
            ctx.refresh_demons(1, prc, xo, thr)


def test_gpu_refresh_full_size_headline_shape():
    """L=160, 2 samples x 64 replicas, 6 demons per site: 24.6 M draws per
    stream, cut into segments."""
    L, nr, nc, ns = 160, 64, 6, 2
    thr = micsa.thresholds(BETA)
    prc, xo = _streams(ns * nr, 0x5EED0000)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    with micsa.Context(L, nr, ns, nc) as ctx:
        ctx.refresh_demons(0, prc, xo, thr)
        for s in range(ns):
            w0, w1 = _host_draw(L, nr, nc, hp, hx, s, thr)
            g0, g1 = ctx.download_demons(s)
            assert np.array_equal(g0, w0) and np.array_equal(g1, w1), s
        assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx)


def test_gpu_refresh_async_overlaps_and_matches():
    """micsa_refresh_demons_async: iterations queued right after it run while
    the host advances the streams; after refresh_wait the structs and the
    demons equal those of the synchronous call."""
    L, nr, nc, ns = 16, 64, 6, 2
    thr = micsa.thresholds(BETA)
    rng = np.random.default_rng(11)
    H, V = (L // 4) ** 3 // 2, L ** 3
    prc, xo = _streams(ns * nr, 321)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    out = []
    for asyn, (p_, x_) in ((True, (prc, xo)), (False, (hp, hx))):
        r2 = np.random.default_rng(5)
        with micsa.Context(L, nr, ns, nc) as ctx:
            for s in range(ns):
                J = micsa.pack_couplings(L, *(r2.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
                ctx.upload_couplings(s, J)
                ctx.upload_spins(s, *(r2.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64,
                                                  endpoint=True) for _ in range(2)))
            for rnd in range(3):
                if asyn:
                    ctx.refresh_demons_async(0, p_, x_, thr)
                else:
                    ctx.refresh_demons(0, p_, x_, thr)
                ctx.iterate(3)
            ctx.refresh_wait()
            out.append([ctx.download_demons(s) for s in range(ns)] + [ctx.download_spins(s) for s in range(ns)])
    assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("mode", ["1", "0"])
def test_gpu_refresh_ahead_equals_in_place(monkeypatch, mode):
    """Refreshes asked for ahead -- drawn on the side stream while iterations
    run (MICSA_REFRESH_AHEAD=1), or recorded and drawn in place at the commit
    (0, the form for contexts on the dataflow sweep) -- then committed, give
    the demons, spins and stream structs of in-place refreshes at the same
    points; committing with nothing pending fails."""
    monkeypatch.setenv("MICSA_REFRESH_AHEAD", mode)
    L, nr, nc, ns = 16, 64, 3, 2
    thr = micsa.thresholds(BETA)
    H, V = (L // 4) ** 3 // 2, L ** 3
    prc, xo = _streams(ns * nr, 4242)
    hp, hx = _copy(prc, micsa.PRC), _copy(xo, micsa.Xoshiro)
    out = []
    for ahead, (p_, x_) in ((True, (prc, xo)), (False, (hp, hx))):
        r2 = np.random.default_rng(9)
        with micsa.Context(L, nr, ns, nc) as ctx:
            for s in range(ns):
                J = micsa.pack_couplings(L, *(r2.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
                ctx.upload_couplings(s, J)
                ctx.upload_spins(s, *(r2.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64,
                                                  endpoint=True) for _ in range(2)))
            if ahead:
                with pytest.raises(micsa.MicsaError, match="ERR_STATE"):
                    ctx.refresh_commit()
                ctx.refresh_demons(0, p_, x_, thr)
                ctx.refresh_demons_ahead(0, p_, x_, thr)
                for _ in range(3):
                    ctx.iterate(2)
                    ctx.refresh_commit()
                    ctx.refresh_demons_ahead(0, p_, x_, thr)
                ctx.iterate(2)
            else:
                ctx.refresh_demons(0, p_, x_, thr)
                for _ in range(3):
                    ctx.iterate(2)
                    ctx.refresh_demons(0, p_, x_, thr)
                ctx.iterate(2)
                ctx.refresh_demons(0, p_, x_, thr)  # the draw the other run left pending
            ctx.refresh_wait()
            out.append([ctx.download_spins(s) for s in range(ns)] + [ctx.measure()["e_demon"]])
    assert bytes(prc) == bytes(hp) and bytes(xo) == bytes(hx)
    for a, b in zip(out[0][:ns], out[1][:ns]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
