"""ctypes binding of libmicsa (include/micsa.h) for tests and benchmarks.

The product is the C ABI; this module only loads the in-tree shared library
and wraps numpy arrays.  Loading fails loudly when the library has not been
built -- there is no fallback implementation.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmicsa.so")
DRIVER_PATH = os.path.join(PKG, "bin", "micsa_run")

MICSA_OK = 0
MICSA_ERR_ARG = 1
MICSA_ERR_CUDA = 2
MICSA_ERR_NOMEM = 3
MICSA_ERR_STATE = 4
MICSA_ERR_UNSUPPORTED = 5
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NOMEM", 4: "ERR_STATE", 5: "ERR_UNSUPPORTED"}

# symbols declared in include/micsa.h (checked by the CPU test suite)
ABI_SYMBOLS = [
    "micsa_create", "micsa_destroy", "micsa_last_error", "micsa_footprint_bytes",
    "micsa_set_lut", "micsa_upload_couplings", "micsa_upload_spins", "micsa_upload_demons",
    "micsa_refresh_demons", "micsa_refresh_demons_async", "micsa_refresh_wait",
    "micsa_refresh_demons_ahead", "micsa_refresh_commit",
    "micsa_monte_carlo", "micsa_iterate", "micsa_measure", "micsa_download_spins",
    "micsa_download_demons", "micsa_profile", "micsa_tuning_report", "micsa_energy_noalloc",
    "micsa_synchronize", "micsa_kernel_launches", "micsa_stream", "micsa_job_measurements",
    "micsa_run_batch", "micsa_set_active", "micsa_serve", "micsa_job_beta",
    "micsa_server_create", "micsa_submit", "micsa_poll", "micsa_server_destroy",
    "micsa_debug_flow_waits", "micsa_multi_create", "micsa_multi_iterate",
    "micsa_multi_synchronize", "micsa_multi_destroy", "micsa_multi_last_error",
    "micsa_multi_kernel_launches", "micsa_multi_report",
]
NOALLOC_MAX_REPLICAS = 8192
NOALLOC_MAX_L = 888

_lib = None


class MicsaError(RuntimeError):
    pass


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("L", C.c_int), ("nr", C.c_int),
                ("nsamples", C.c_int), ("nc", C.c_int)]


class PRC(C.Structure):
    """micsa_prc_t: the reference's s_aleatorio_HQ_64bits (2080 bytes)."""
    _fields_ = [("ira", C.c_uint64 * 256), ("pr", C.c_uint64), ("zseed", C.c_uint64),
                ("out", C.c_uint64), ("ip", C.c_ubyte), ("ip1", C.c_ubyte), ("ip2", C.c_ubyte),
                ("ip3", C.c_ubyte), ("pad", C.c_ubyte * 4)]


class Xoshiro(C.Structure):
    """micsa_xoshiro_t: the reference's s_xoshiro256pp (48 bytes)."""
    _fields_ = [("s", C.c_uint64 * 4), ("t", C.c_uint64), ("out", C.c_uint64)]


class Job(C.Structure):
    """micsa_job (include/micsa.h): one reference run of one sample."""
    _fields_ = [("L", C.c_int), ("nr", C.c_int), ("nc", C.c_int), ("iterations", C.c_int64),
                ("seed_J", C.c_uint64), ("seed_u", C.c_uint64), ("beta", C.c_double),
                ("beta_end", C.c_double)]


class Request(C.Structure):
    _fields_ = [("arrival", C.c_double), ("job", Job)]


class RequestResult(C.Structure):
    _fields_ = [("prepared", C.c_double), ("admitted", C.c_double), ("finished", C.c_double)]


class ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_int64), ("slots_max", C.c_int),
                ("chunk", C.c_int64), ("prep_threads", C.c_int)]


class PoolShape(C.Structure):
    """micsa_pool_shape: one shape a server serves (slots 0 = from the budget)."""
    _fields_ = [("L", C.c_int), ("nr", C.c_int), ("nc", C.c_int), ("slots", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_int64), ("slots_max", C.c_int),
                ("chunk", C.c_int64), ("prep_threads", C.c_int),
                ("shapes", C.POINTER(PoolShape)), ("nshapes", C.c_int)]


class RefreshPlan(C.Structure):
    """micsa_refresh_plan (host/micsa_jump.h): jump tables of one refresh shape."""
    _fields_ = [("nwords", C.c_int64), ("words_per_seg", C.c_int64), ("nseg", C.c_int64),
                ("lcg", C.POINTER(C.c_uint64)), ("xo", C.POINTER(C.c_uint64)),
                ("fib", C.POINTER(C.c_uint64)), ("adv_lcg", C.c_uint64 * 2),
                ("adv_xo", C.c_uint64 * 4), ("adv_fib", C.c_uint64 * 55)]


STREAM_REC = 120  # words of one stream's start record (micsa_stream_record)


def _ptr(a, ctype):
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.POINTER(ctype))


def lib():
    """Load libmicsa.so (build it first with micsa-ea-mc_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MicsaError("libmicsa.so is not built (%s); run build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    u64p, u32p, i32p, i64p, u8p = (C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_uint8))
    sig = {
        "micsa_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
        "micsa_destroy": (C.c_int, [C.c_void_p]),
        "micsa_last_error": (C.c_char_p, [C.c_void_p]),
        "micsa_footprint_bytes": (C.c_int64, [C.POINTER(Config)]),
        "micsa_set_lut": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
        "micsa_upload_couplings": (C.c_int, [C.c_void_p, C.c_int, u64p]),
        "micsa_upload_spins": (C.c_int, [C.c_void_p, C.c_int, u64p, u64p]),
        "micsa_upload_demons": (C.c_int, [C.c_void_p, C.c_int, u64p, u64p]),
        "micsa_refresh_demons": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(PRC),
                                           C.POINTER(Xoshiro), u64p]),
        "micsa_refresh_demons_async": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(PRC),
                                                 C.POINTER(Xoshiro), u64p]),
        "micsa_refresh_wait": (C.c_int, [C.c_void_p]),
        "micsa_refresh_demons_ahead": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(PRC),
                                                 C.POINTER(Xoshiro), u64p]),
        "micsa_refresh_commit": (C.c_int, [C.c_void_p]),
        "micsa_monte_carlo": (C.c_int, [C.c_void_p, C.c_int, u32p, u32p]),
        "micsa_iterate": (C.c_int, [C.c_void_p, C.c_int64]),
        "micsa_measure": (C.c_int, [C.c_void_p, i32p, u64p, i64p, i64p]),
        "micsa_download_spins": (C.c_int, [C.c_void_p, C.c_int, u64p, u64p]),
        "micsa_download_demons": (C.c_int, [C.c_void_p, C.c_int, u64p, u64p]),
        "micsa_profile": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]),
        "micsa_tuning_report": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
        # (L, nr, nsamples, spin_rows, J_rows, e_spin, stream, err, errlen)
        "micsa_energy_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]),
        "micsa_synchronize": (C.c_int, [C.c_void_p]),
        "micsa_kernel_launches": (C.c_int64, [C.c_void_p]),
        "micsa_stream": (C.c_void_p, [C.c_void_p]),
        "micsa_job_measurements": (C.c_int64, [C.c_int64]),
        "micsa_set_active": (C.c_int, [C.c_void_p, u8p]),
        "micsa_debug_flow_waits": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int]),
        "micsa_multi_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p),
                                         C.c_char_p, C.c_size_t]),
        "micsa_multi_iterate": (C.c_int, [C.c_void_p, C.c_int64]),
        "micsa_multi_synchronize": (C.c_int, [C.c_void_p]),
        "micsa_multi_destroy": (C.c_int, [C.c_void_p]),
        "micsa_multi_last_error": (C.c_char_p, [C.c_void_p]),
        "micsa_multi_kernel_launches": (C.c_int64, [C.c_void_p]),
        "micsa_multi_report": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
        "micsa_job_beta": (C.c_double, [C.POINTER(Job), C.c_int64]),
        "micsa_serve": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(Request), C.c_int,
                                  C.POINTER(RequestResult), i32p, u64p, C.POINTER(C.c_double),
                                  C.c_char_p, C.c_size_t]),
        "micsa_run_batch": (C.c_int, [C.c_int, C.POINTER(Job), C.c_int, i32p, u64p,
                                      C.POINTER(C.c_double), C.c_char_p, C.c_size_t]),
        "micsa_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p),
                                          C.c_char_p, C.c_size_t]),
        "micsa_submit": (C.c_int, [C.c_void_p, C.POINTER(Job), C.POINTER(C.c_int64)]),
        "micsa_poll": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_int), i32p,
                                 u64p, C.POINTER(RequestResult)]),
        "micsa_server_destroy": (C.c_int, [C.c_void_p]),
        # host side (micsa-ea-mc_gb300/host/micsa_host.h)
        "micsa_check_seed": (C.c_uint64, [C.c_uint64]),
        "micsa_init_cpu_generators": (None, [C.POINTER(PRC), C.POINTER(Xoshiro), u32p, C.c_uint64]),
        "micsa_init_rand_hq": (None, [C.POINTER(PRC), C.c_uint64]),
        "micsa_seeds_from_one": (None, [u64p, u64p, C.c_int]),
        "micsa_half_words": (C.c_int64, [C.c_int]),
        "micsa_pack_spins": (None, [C.c_int, C.c_int, u8p, u64p, u64p]),
        "micsa_unpack_spins": (None, [C.c_int, C.c_int, u64p, u64p, u8p]),
        "micsa_pack_couplings": (None, [C.c_int, u8p, u8p, u8p, u64p]),
        "micsa_init_spins": (C.c_int, [C.POINTER(PRC), C.c_int, C.c_int, C.c_int, i32p, C.c_int, u8p]),
        "micsa_init_couplings_janus": (C.c_int, [C.c_uint64, C.c_int, u8p, u8p, u8p]),
        "micsa_thresholds": (None, [C.c_double, u64p]),
        "micsa_draw_demons_all": (C.c_int, [C.POINTER(PRC), C.POINTER(Xoshiro), u64p, C.c_int,
                                            C.c_int, C.c_int, u64p, u64p, C.c_int]),
        "micsa_fill_bits": (None, [C.POINTER(PRC), C.POINTER(Xoshiro), C.c_int, C.c_uint64,
                                   C.c_int, C.c_uint32, u32p]),
        "micsa_correlation_lengths": (None, [C.c_int, C.c_int, i64p, C.c_double, C.c_int,
                                             C.POINTER(C.c_double), C.POINTER(C.c_double),
                                             C.POINTER(C.c_double), C.POINTER(C.c_double),
                                             C.POINTER(C.c_int)]),
        "micsa_draw_demons": (None, [C.POINTER(PRC), C.POINTER(Xoshiro), u64p, C.c_int, C.c_int,
                                     C.c_int, C.c_int, u64p, u64p]),
        # jump-ahead of the refresh streams (micsa-ea-mc_gb300/host/micsa_jump.h)
        "micsa_lcg_jump": (None, [C.c_uint64, u64p, u64p]),
        "micsa_fib_jump": (None, [C.c_uint64, u64p]),
        "micsa_xoshiro_charpoly": (None, [u64p]),
        "micsa_xoshiro_jump_poly": (None, [C.c_uint64, u64p]),
        "micsa_xoshiro_apply": (None, [u64p, u64p]),
        "micsa_streams_advance": (None, [C.POINTER(PRC), C.POINTER(Xoshiro), C.c_uint64]),
        "micsa_refresh_plan_make": (C.c_int, [C.c_int64, C.c_int64, C.POINTER(RefreshPlan)]),
        "micsa_refresh_plan_free": (None, [C.POINTER(RefreshPlan)]),
        "micsa_stream_record": (C.c_int, [C.POINTER(PRC), C.POINTER(Xoshiro), u64p]),
        "micsa_streams_advance_plan": (None, [C.POINTER(RefreshPlan), C.POINTER(PRC),
                                              C.POINTER(Xoshiro)]),
        "micsa_draw_segment": (None, [C.POINTER(RefreshPlan), C.c_int64, u64p, u64p, C.c_int,
                                      C.c_int, u64p, u64p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(ctx, rc, what):
    if rc != MICSA_OK:
        msg = lib().micsa_last_error(ctx) if ctx else b""
        raise MicsaError("%s failed: %s %s" % (what, STATUS.get(rc, rc), (msg or b"").decode()))


class Context:
    """One libmicsa context (device state of nsamples x nr replicas)."""

    def __init__(self, L, nr, nsamples=1, nc=6, device=0):
        self.L, self.nr, self.ns, self.nc = L, nr, nsamples, nc
        self.H = (L // 4) ** 3 // 2
        self.cfg = Config(device, L, nr, nsamples, nc)
        h = C.c_void_p()
        rc = lib().micsa_create(C.byref(self.cfg), C.byref(h))
        if rc != MICSA_OK:
            raise MicsaError("micsa_create failed: %s" % STATUS.get(rc, rc))
        self.h = h

    def close(self):
        if self.h:
            lib().micsa_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_lut(self, lut):
        b = np.ascontiguousarray(np.frombuffer(bytes(lut), dtype=np.uint8))
        check(self.h, lib().micsa_set_lut(self.h, b.ctypes.data_as(C.c_void_p), b.size), "set_lut")

    def upload_couplings(self, s, J):
        J = np.ascontiguousarray(J, dtype=np.uint64)
        check(self.h, lib().micsa_upload_couplings(self.h, s, _ptr(J, C.c_uint64)), "upload_couplings")

    def upload_spins(self, s, even, odd):
        e = np.ascontiguousarray(even, dtype=np.uint64)
        o = np.ascontiguousarray(odd, dtype=np.uint64)
        check(self.h, lib().micsa_upload_spins(self.h, s, _ptr(e, C.c_uint64), _ptr(o, C.c_uint64)),
              "upload_spins")

    def upload_demons(self, s, w0, w1):
        a = np.ascontiguousarray(w0, dtype=np.uint64)
        b = np.ascontiguousarray(w1, dtype=np.uint64)
        check(self.h, lib().micsa_upload_demons(self.h, s, _ptr(a, C.c_uint64), _ptr(b, C.c_uint64)),
              "upload_demons")

    def refresh_demons(self, first, prc, xo, thr):
        """Demon refresh on the GPU for samples first .. first+len(prc)/nr-1;
        prc/xo (ctypes arrays of PRC / Xoshiro, [count][nr]) are advanced in
        place as InitWalkers would advance them."""
        count, rem = divmod(len(prc), self.nr)
        if rem or len(xo) != len(prc):
            raise ValueError("need count*nr streams of each generator")
        t = np.ascontiguousarray(thr, dtype=np.uint64)
        check(self.h, lib().micsa_refresh_demons(self.h, first, count, prc, xo, _ptr(t, C.c_uint64)),
              "refresh_demons")

    def refresh_demons_async(self, first, prc, xo, thr):
        """As refresh_demons; prc/xo are advanced in the background until
        refresh_wait (keep them alive and untouched until then)."""
        count, rem = divmod(len(prc), self.nr)
        if rem or len(xo) != len(prc):
            raise ValueError("need count*nr streams of each generator")
        self._thr = np.ascontiguousarray(thr, dtype=np.uint64)
        check(self.h, lib().micsa_refresh_demons_async(self.h, first, count, prc, xo,
                                                       _ptr(self._thr, C.c_uint64)),
              "refresh_demons_async")

    def set_active(self, flags):
        """Per-sample run flags (None: all samples run)."""
        a = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
        check(self.h, lib().micsa_set_active(self.h, _ptr(a, C.c_uint8)), "set_active")

    def refresh_demons_ahead(self, first, prc, xo, thr):
        """Draw the next refresh into the back buffer on the side stream
        (prc/xo advanced in the background, as refresh_demons_async)."""
        count, rem = divmod(len(prc), self.nr)
        if rem or len(xo) != len(prc):
            raise ValueError("need count*nr streams of each generator")
        self._thr_a = np.ascontiguousarray(thr, dtype=np.uint64)
        check(self.h, lib().micsa_refresh_demons_ahead(self.h, first, count, prc, xo,
                                                       _ptr(self._thr_a, C.c_uint64)),
              "refresh_demons_ahead")

    def refresh_commit(self):
        check(self.h, lib().micsa_refresh_commit(self.h), "refresh_commit")

    def refresh_wait(self):
        check(self.h, lib().micsa_refresh_wait(self.h), "refresh_wait")

    def monte_carlo(self, flag, te=None, keys=None):
        t = None if te is None else np.ascontiguousarray(te, dtype=np.uint32)
        k = None if keys is None else np.ascontiguousarray(keys, dtype=np.uint32)
        check(self.h, lib().micsa_monte_carlo(self.h, flag, _ptr(t, C.c_uint32), _ptr(k, C.c_uint32)),
              "monte_carlo")

    def iterate(self, n):
        check(self.h, lib().micsa_iterate(self.h, n), "iterate")

    def synchronize(self):
        check(self.h, lib().micsa_synchronize(self.h), "synchronize")

    def measure(self, spin=True, demon=True, overlap=False):
        ns, nr, nd = self.ns, self.nr, self.L // 2 + 1
        es = np.zeros(ns * nr, np.int32) if spin else None
        ed = np.zeros(ns * nr, np.uint64) if demon else None
        q = np.zeros(ns * (nr // 2), np.int64) if overlap else None
        c4 = np.zeros(ns * (nr // 2) * 3 * nd, np.int64) if overlap else None
        check(self.h, lib().micsa_measure(self.h, _ptr(es, C.c_int32), _ptr(ed, C.c_uint64),
                                          _ptr(q, C.c_int64), _ptr(c4, C.c_int64)), "measure")
        out = {}
        if spin:
            out["e_spin"] = es.reshape(ns, nr)
        if demon:
            out["e_demon"] = ed.reshape(ns, nr)
        if overlap:
            out["q"] = q.reshape(ns, nr // 2)
            out["c4"] = c4.reshape(ns, nr // 2, 3, nd)
        return out

    def download_spins(self, s):
        e = np.zeros(self.H * self.nr, np.uint64)
        o = np.zeros(self.H * self.nr, np.uint64)
        check(self.h, lib().micsa_download_spins(self.h, s, _ptr(e, C.c_uint64), _ptr(o, C.c_uint64)),
              "download_spins")
        return e, o

    def download_demons(self, s):
        n = 2 * self.H * self.nc * self.nr
        a = np.zeros(n, np.uint64)
        b = np.zeros(n, np.uint64)
        check(self.h, lib().micsa_download_demons(self.h, s, _ptr(a, C.c_uint64), _ptr(b, C.c_uint64)),
              "download_demons")
        return a, b

    def profile(self, n):
        """(mean half-sweep launch ms, mean iteration ms) over n iterations."""
        a, b = C.c_double(), C.c_double()
        check(self.h, lib().micsa_profile(self.h, n, C.byref(a), C.byref(b)), "profile")
        return a.value, b.value

    def tuning(self):
        """The autotuner's choice and timings, as a text line."""
        buf = C.create_string_buffer(16384)
        check(self.h, lib().micsa_tuning_report(self.h, buf, 16384), "tuning_report")
        return buf.value.decode()

    def kernel_launches(self):
        return lib().micsa_kernel_launches(self.h)

    def stream(self):
        return lib().micsa_stream(self.h)


# ------------------------------------------------------------------ host side
class Multi:
    """Mixed-lattice launches over several contexts (micsa_multi_*)."""

    def __init__(self, contexts):
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h for c in self.contexts])
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().micsa_multi_create(arr, len(self.contexts), C.byref(h), err, 512)
        if rc != MICSA_OK:
            raise MicsaError("micsa_multi_create failed (%d): %s" % (rc, err.value.decode()))
        self.h = h

    def _check(self, rc, what):
        if rc != MICSA_OK:
            raise MicsaError("%s failed (%d): %s" % (what, rc,
                                                    lib().micsa_multi_last_error(self.h).decode()))

    def iterate(self, n):
        self._check(lib().micsa_multi_iterate(self.h, n), "micsa_multi_iterate")

    def synchronize(self):
        self._check(lib().micsa_multi_synchronize(self.h), "micsa_multi_synchronize")

    def report(self):
        b = C.create_string_buffer(8192)
        lib().micsa_multi_report(self.h, b, 8192)
        return b.value.decode()

    def kernel_launches(self):
        return lib().micsa_multi_kernel_launches(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().micsa_multi_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Streams:
    """Host generator state of one run (the reference's globals of ini.c)."""


def check_seed(seed):
    return lib().micsa_check_seed(seed)


def seeds_from_one(seed, n):
    s = C.c_uint64(seed)
    out = np.zeros(n, np.uint64)
    lib().micsa_seeds_from_one(C.byref(s), _ptr(out, C.c_uint64), n)
    return s.value, out


def init_cpu_generators(seed):
    p, x, k = PRC(), Xoshiro(), C.c_uint32()
    lib().micsa_init_cpu_generators(C.byref(p), C.byref(x), C.byref(k), seed)
    return p, x, k.value


def init_rand_hq(seed):
    p = PRC()
    lib().micsa_init_rand_hq(C.byref(p), seed)
    return p


def thresholds(beta):
    t = np.zeros(3, np.uint64)
    lib().micsa_thresholds(beta, _ptr(t, C.c_uint64))
    return t


def couplings_janus(seed, L):
    V = L ** 3
    Jx, Jy, Jz = (np.zeros(V, np.uint8) for _ in range(3))
    count = lib().micsa_init_couplings_janus(seed, L, _ptr(Jx, C.c_uint8), _ptr(Jy, C.c_uint8),
                                             _ptr(Jz, C.c_uint8))
    return Jx, Jy, Jz, count


def pack_couplings(L, Jx, Jy, Jz):
    H = (L // 4) ** 3 // 2
    J = np.zeros(12 * H, np.uint64)
    lib().micsa_pack_couplings(L, _ptr(Jx, C.c_uint8), _ptr(Jy, C.c_uint8), _ptr(Jz, C.c_uint8),
                               _ptr(J, C.c_uint64))
    return J


def pack_spins(L, nr, uu):
    H = (L // 4) ** 3 // 2
    e = np.zeros(H * nr, np.uint64)
    o = np.zeros(H * nr, np.uint64)
    uu = np.ascontiguousarray(uu, dtype=np.uint8)
    lib().micsa_pack_spins(L, nr, _ptr(uu, C.c_uint8), _ptr(e, C.c_uint64), _ptr(o, C.c_uint64))
    return e, o


def unpack_spins(L, nr, even, odd):
    uu = np.zeros(nr * L ** 3, np.uint8)
    e = np.ascontiguousarray(even, dtype=np.uint64)
    o = np.ascontiguousarray(odd, dtype=np.uint64)
    lib().micsa_unpack_spins(L, nr, _ptr(e, C.c_uint64), _ptr(o, C.c_uint64), _ptr(uu, C.c_uint8))
    return uu


class HostModel:
    """The reference's host initialisation (ini.c Init) for one run:
    seeds, Metropolis streams, spins, couplings, demon streams."""

    MAXNSAMPLES = 2

    def __init__(self, L, nr, nc, seed_J, seed_u, seed_MC, list_samples=(0,), beta=0.9090909090909,
                 nthreads=8):
        Lb = lib()
        self.L, self.nr, self.nc, self.beta = L, nr, nc, beta
        self.nbits = len(list_samples)
        self.list_samples = list(list_samples)
        self.V = L ** 3
        self.H = (L // 4) ** 3 // 2
        self.nthreads = nthreads
        # get_seeds (io.c:794-799): the Janus build uses one fixed coupling seed
        self.seed_J, _ = seeds_from_one(seed_J, self.MAXNSAMPLES)
        self.seeds_J = [9164166177945067407] * self.nbits
        # Init_Random (ini.c:34-60)
        self.seed_u = check_seed(seed_u)
        self.seed_MC = [check_seed(s) for s in seed_MC]
        self.random_u = init_rand_hq(self.seed_u)
        self.prc = (PRC * nr)()
        self.xo = (Xoshiro * nr)()
        self.keys = np.zeros(nr, np.uint32)
        for r in range(nr):
            k = C.c_uint32()
            Lb.micsa_init_cpu_generators(C.byref(self.prc[r]), C.byref(self.xo[r]), C.byref(k),
                                         self.seed_MC[r])
            self.keys[r] = k.value
        self.seed_u, self.seeds_C = seeds_from_one(self.seed_u, self.MAXNSAMPLES * nr)
        self.prc_C, self.xo_C = [], []
        for b in range(self.nbits):
            pa, xa = (PRC * nr)(), (Xoshiro * nr)()
            for r in range(nr):
                k = C.c_uint32()
                Lb.micsa_init_cpu_generators(C.byref(pa[r]), C.byref(xa[r]), C.byref(k),
                                             int(self.seeds_C[b * nr + r]))
            self.prc_C.append(pa)
            self.xo_C.append(xa)
        # Init_u (ini.c:275-299)
        self.uu = np.zeros(self.nbits * nr * self.V, np.uint8)
        ls = np.array(self.list_samples + [0] * (self.MAXNSAMPLES + 1 - self.nbits), np.int32)
        rc = Lb.micsa_init_spins(C.byref(self.random_u), L, nr, self.MAXNSAMPLES,
                                 _ptr(ls, C.c_int32), self.nbits, _ptr(self.uu, C.c_uint8))
        if rc:
            raise MicsaError("Problems generating spins")
        self.uu = self.uu.reshape(self.nbits, nr, self.V)
        self.spins = [pack_spins(L, nr, self.uu[b]) for b in range(self.nbits)]
        # Init_J / packing_J (ini.c:425-578)
        self.Jsite, self.J = [], []
        for b in range(self.nbits):
            Jx, Jy, Jz, count = couplings_janus(self.seeds_J[b], L)
            self.Jsite.append((Jx, Jy, Jz, count))
            self.J.append(pack_couplings(L, Jx, Jy, Jz))
        self.thr = thresholds(beta)

    def draw_demons(self, b):
        """InitWalkers (ini.c:712-781) for sample b: CPUwalker0/1 words."""
        n = 2 * self.H * self.nc * self.nr
        w0 = np.zeros(n, np.uint64)
        w1 = np.zeros(n, np.uint64)
        rc = lib().micsa_draw_demons_all(self.prc_C[b], self.xo_C[b], _ptr(self.thr, C.c_uint64),
                                         self.L, self.nr, self.nc, _ptr(w0, C.c_uint64),
                                         _ptr(w1, C.c_uint64), self.nthreads)
        if rc:
            raise MicsaError("demon draw failed")
        return w0, w1

    def fill_bits(self, it, parity, jobid):
        """_fill_bits (fill_bits.h:47-68): Philox counters of one call."""
        te = np.zeros(4 * self.nr, np.uint32)
        lib().micsa_fill_bits(self.prc, self.xo, self.nr, it, parity, jobid, _ptr(te, C.c_uint32))
        return te


def run_batch(jobs, device=0):
    """micsa_run_batch over a list of dicts (L, nr, nc, iterations, seed_J,
    seed_u, beta); returns ([e_spin [m, nr] per job], [e_demon ...], seconds)."""
    n = len(jobs)
    arr = (Job * n)(*[Job(j["L"], j["nr"], j["nc"], j["iterations"], j["seed_J"], j["seed_u"],
                          j["beta"], j.get("beta_end", 0.0)) for j in jobs])
    nms = [lib().micsa_job_measurements(j["iterations"]) for j in jobs]
    sizes = [nm * j["nr"] for nm, j in zip(nms, jobs)]
    es = np.zeros(sum(sizes), np.int32)
    ed = np.zeros(sum(sizes), np.uint64)
    sec = C.c_double()
    err = C.create_string_buffer(512)
    rc = lib().micsa_run_batch(device, arr, n, _ptr(es, C.c_int32), _ptr(ed, C.c_uint64),
                               C.byref(sec), err, 512)
    if rc != MICSA_OK:
        raise MicsaError("micsa_run_batch: %s %s" % (STATUS.get(rc, rc), err.value.decode()))
    cut = np.cumsum([0] + sizes)
    outs = [(es[a:b].reshape(nm, j["nr"]), ed[a:b].reshape(nm, j["nr"]))
            for a, b, nm, j in zip(cut[:-1], cut[1:], nms, jobs)]
    return [o[0] for o in outs], [o[1] for o in outs], sec.value


def serve(requests, device=0, hbm_budget=0, slots_max=0, chunk=0, prep_threads=0):
    """micsa_serve over a list of dicts (arrival + the job fields); returns
    (e_spin per request, e_demon per request, [(prepared, admitted,
    finished)], seconds)."""
    n = len(requests)
    arr = (Request * n)(*[Request(r["arrival"], Job(r["L"], r["nr"], r["nc"], r["iterations"],
                                                    r["seed_J"], r["seed_u"], r["beta"],
                                                    r.get("beta_end", 0.0)))
                          for r in requests])
    nms = [lib().micsa_job_measurements(r["iterations"]) for r in requests]
    sizes = [nm * r["nr"] for nm, r in zip(nms, requests)]
    es = np.zeros(sum(sizes), np.int32)
    ed = np.zeros(sum(sizes), np.uint64)
    res = (RequestResult * n)()
    cfg = ServeConfig(device, hbm_budget, slots_max, chunk, prep_threads)
    sec = C.c_double()
    err = C.create_string_buffer(512)
    rc = lib().micsa_serve(C.byref(cfg), arr, n, res, _ptr(es, C.c_int32), _ptr(ed, C.c_uint64),
                           C.byref(sec), err, 512)
    if rc != MICSA_OK:
        raise MicsaError("micsa_serve: %s %s" % (STATUS.get(rc, rc), err.value.decode()))
    cut = np.cumsum([0] + sizes)
    e_s = [es[a:b].reshape(nm, r["nr"]) for a, b, nm, r in zip(cut[:-1], cut[1:], nms, requests)]
    e_d = [ed[a:b].reshape(nm, r["nr"]) for a, b, nm, r in zip(cut[:-1], cut[1:], nms, requests)]
    return e_s, e_d, [(x.prepared, x.admitted, x.finished) for x in res], sec.value


class Server:
    """A micsa_server: pools for the given shapes [(L, nr, nc) or (L, nr, nc,
    slots)], jobs submitted as dicts (the micsa_job fields), results polled."""

    def __init__(self, shapes, device=0, hbm_budget=0, slots_max=0, chunk=0, prep_threads=0):
        sh = [tuple(x) + (0,) * (4 - len(x)) for x in shapes]
        self._shapes = (PoolShape * len(sh))(*[PoolShape(*x) for x in sh])
        cfg = ServerConfig(device, hbm_budget, slots_max, chunk, prep_threads, self._shapes, len(sh))
        self.h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().micsa_server_create(C.byref(cfg), C.byref(self.h), err, 512)
        if rc != MICSA_OK:
            raise MicsaError("micsa_server_create: %s %s" % (STATUS.get(rc, rc), err.value.decode()))
        self._jobs = {}

    def submit(self, j):
        job = Job(j["L"], j["nr"], j["nc"], j["iterations"], j["seed_J"], j["seed_u"], j["beta"],
                  j.get("beta_end", 0.0))
        i = C.c_int64()
        rc = lib().micsa_submit(self.h, C.byref(job), C.byref(i))
        if rc != MICSA_OK:
            raise MicsaError("micsa_submit: %s" % STATUS.get(rc, rc))
        self._jobs[i.value] = j
        return i.value

    def poll(self, i, timeout=0.0):
        """None while request i runs; then (e_spin [m, nr], e_demon [m, nr],
        (prepared, admitted, finished) seconds after its submission)."""
        j = self._jobs.get(i)
        nm = lib().micsa_job_measurements(j["iterations"]) if j else 0
        nr = j["nr"] if j else 0
        es = np.zeros(max(1, nm * nr), np.int32)
        ed = np.zeros(max(1, nm * nr), np.uint64)
        done, t = C.c_int(), RequestResult()
        rc = lib().micsa_poll(self.h, i, timeout, C.byref(done), _ptr(es, C.c_int32),
                              _ptr(ed, C.c_uint64), C.byref(t))
        if rc != MICSA_OK:
            self._jobs.pop(i, None)
            raise MicsaError("micsa_poll: %s" % STATUS.get(rc, rc))
        if not done.value:
            return None
        del self._jobs[i]
        return (es[:nm * nr].reshape(nm, nr), ed[:nm * nr].reshape(nm, nr),
                (t.prepared, t.admitted, t.finished))

    def close(self):
        if self.h:
            lib().micsa_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


XI_KAPPA = 3.0  # the noise cut-off of the driver's evol_xi.txt


def correlation_lengths(L, c4, kappa=0.0, rmax=0, with_cut=False):
    """(C4(r) averaged over pairs and axes / V, xi12, xi23) from one sample's
    c4 array [pairs, 3, L/2+1] (micsa_measure's layout).  kappa > 0 stops the
    integrals at the first r >= 1 where C4(r) < kappa x its standard error
    over the pairs, rmax > 0 at r = rmax; with_cut=True also returns that
    cut and the errors."""
    c = np.ascontiguousarray(c4, dtype=np.int64)
    npairs = c.size // (3 * (L // 2 + 1))
    out = np.zeros(L // 2 + 1, np.float64)
    err = np.zeros(L // 2 + 1, np.float64)
    x12, x23, cut = C.c_double(), C.c_double(), C.c_int()
    lib().micsa_correlation_lengths(L, npairs, _ptr(c, C.c_int64), kappa, rmax,
                                    _ptr(out, C.c_double), _ptr(err, C.c_double), C.byref(x12),
                                    C.byref(x23), C.byref(cut))
    if with_cut:
        return out, x12.value, x23.value, cut.value, err
    return out, x12.value, x23.value
