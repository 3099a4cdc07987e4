"""TEST INFRASTRUCTURE ONLY: build and ctypes binding of the CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product (libmicsa, micsa_run) never links or calls it.
"""
import ctypes as C
import os
import platform
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# the reference sources, where a copy exists (never on the GPU host); unset:
# the live reference build is skipped and the committed golden fixtures pin
# the oracle alone
REFERENCE = os.environ.get("MICSA_REFERENCE_DIR", "")

_lib = None


def build(force=False):
    src = os.path.join(HERE, "micsa_oracle.c")
    hdr = os.path.join(HERE, "micsa_oracle.h")
    os.makedirs(LIBDIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    subprocess.run(["gcc", "-O3", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-Wall",
                    src, "-o", LIB], check=True)
    return LIB


def reference_available():
    return bool(REFERENCE) and os.path.exists(os.path.join(REFERENCE, "PROGRAM", "src", "main.cu"))


def build_reference(L, nr, ms=2):
    """Reference program compiled for the CPU (oracle/ref_cpu/build_ref.sh);
    only possible where the reference sources are present."""
    exe = os.path.join(REF_DIR, "micsa_ref_L%d_NR%d_MS%d" % (L, nr, ms))
    if os.path.exists(exe):
        return exe
    if not reference_available() or platform.machine() not in ("x86_64", "AMD64"):
        return None
    subprocess.run(["sh", os.path.join(HERE, "ref_cpu", "build_ref.sh"), str(L), str(nr), str(ms)],
                   check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return exe


REF_GPU_LIB = os.path.join(LIBDIR, "libref_gpu.so")


def build_ref_gpu_harness(force=False):
    """The host side that drives the reference's own CUDA kernels
    (ref_gpu/ref_gpu_harness.cu; our code, test infrastructure)."""
    src = os.path.join(HERE, "ref_gpu", "ref_gpu_harness.cu")
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(REF_GPU_LIB) and os.path.getmtime(REF_GPU_LIB) >= os.path.getmtime(src):
        return REF_GPU_LIB
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    stubs = "/usr/local/cuda/lib64/stubs"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src, "-o", REF_GPU_LIB,
                    "-L" + stubs, "-lcuda"], check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return REF_GPU_LIB


def ref_gpu_cubin(L, nr, ms=2, build=False):
    """The reference's device code for (L, NR, MAXNSAMPLES) compiled for
    sm_103a (ref_gpu/build_ref_gpu.sh); built only where the reference
    sources are present, else whatever was built there before."""
    path = os.path.join(REF_DIR, "micsa_ref_gpu_L%d_NR%d_MS%d.cubin" % (L, nr, ms))
    if os.path.exists(path) or not build or not reference_available():
        return path if os.path.exists(path) else None
    subprocess.run(["sh", os.path.join(HERE, "ref_gpu", "build_ref_gpu.sh"), str(L), str(nr), str(ms)],
                   check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return path


class RefGPU:
    """The reference's CUDA kernels for ns samples of one (L, nr) build, on
    device 0, laid out and launched as the reference's main.cu does."""

    def __init__(self, cubin, L, nr, ns, nc):
        self.lib = C.CDLL(build_ref_gpu_harness())
        self.lib.rg_error.restype = C.c_char_p
        self.L, self.nr, self.ns, self.nc = L, nr, ns, nc
        neig, rot = tables(L)
        neig = np.ascontiguousarray(neig.reshape(-1))
        rot = np.ascontiguousarray(rot.reshape(-1))
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = self.lib.rg_create(cubin.encode(), L, nr, ns, nc, _p(neig, I32), _p(rot, U8), C.byref(h),
                                err, 512)
        if rc:
            raise RuntimeError("reference kernels: %s" % err.value.decode())
        self.h = h

    def _ck(self, rc, what):
        if rc:
            raise RuntimeError("%s: %s" % (what, self.lib.rg_error(self.h).decode()))

    def upload(self, s, J, even, odd, w0, w1):
        self._ck(self.lib.rg_upload(self.h, s, None if J is None else _p(J, U64), _p(even, U64),
                                    _p(odd, U64), _p(w0, U64), _p(w1, U64)), "rg_upload")

    def download(self, s):
        H = (self.L // 4) ** 3 // 2
        e = np.zeros(H * self.nr, np.uint64)
        o = np.zeros(H * self.nr, np.uint64)
        w0 = np.zeros(2 * H * self.nc * self.nr, np.uint64)
        w1 = np.zeros(2 * H * self.nc * self.nr, np.uint64)
        self._ck(self.lib.rg_download(self.h, s, _p(e, U64), _p(o, U64), _p(w0, U64), _p(w1, U64)),
                 "rg_download")
        return e, o, w0, w1

    def iterate(self, n):
        self._ck(self.lib.rg_iterate(self.h, C.c_int64(n)), "rg_iterate")

    def time(self, warm, n):
        ms = C.c_double()
        self._ck(self.lib.rg_time(self.h, C.c_int64(warm), C.c_int64(n), C.byref(ms)), "rg_time")
        return ms.value

    def launch_shape(self):
        a, b = C.c_int(), C.c_int()
        self.lib.rg_launch_shape(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.rg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        u64p, u32p, i32p, i64p, u8p = (C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_uint8))
        sig = {
            "oracle_tables": (None, [C.c_int, i32p, u8p]),
            "oracle_half_sweep": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, u64p, u64p,
                                         u64p, u64p, u64p, u64p, C.c_int, C.c_int]),
            "oracle_walk": (None, [C.c_int, C.c_int, C.c_int, u64p, u64p, C.c_int, C.c_int]),
            "oracle_micsa_iteration": (None, [C.c_int, C.c_int, C.c_int, u64p, u64p, u64p, u64p,
                                              u64p, C.c_int]),
            "oracle_gen_rndbits": (None, [C.c_int, C.c_int, u32p, u32p, C.c_void_p, u64p]),
            "oracle_metropolis_iteration": (None, [C.c_int, C.c_int, u64p, u64p, u64p, u32p, u32p,
                                                   u32p, C.c_void_p]),
            "oracle_energy": (None, [C.c_int, C.c_int, u64p, u64p, u64p, i32p]),
            "oracle_demon_energy": (None, [C.c_int, C.c_int, C.c_int, u64p, u64p, u64p]),
            "oracle_scalar_rule": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int)]),
            "oracle_isi_word": (C.c_uint64, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                             u64p, u64p]),
            "oracle_overlap_c4": (None, [C.c_int, C.c_int, u8p, i64p, i64p]),
            "oracle_scalar_energy": (C.c_int32, [C.c_int, u8p, u8p, u8p, u8p]),
            "oracle_pack_couplings": (None, [C.c_int, u8p, u8p, u8p, u64p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


U64, U32, I32, I64, U8 = C.c_uint64, C.c_uint32, C.c_int32, C.c_int64, C.c_uint8


def micsa_iteration(L, nr, nc, J, even, odd, w0, w1, nthreads=1):
    lib().oracle_micsa_iteration(L, nr, nc, _p(J, U64), _p(even, U64), _p(odd, U64), _p(w0, U64),
                                 _p(w1, U64), nthreads)


def half_sweep(L, nr, nc, p, ic, J, even, odd, w0, w1, rand=None, r0=0, r1=None):
    r1 = nr if r1 is None else r1
    lib().oracle_half_sweep(L, nr, nc, p, ic, _p(J, U64), _p(even, U64), _p(odd, U64),
                            None if w0 is None else _p(w0, U64), None if w1 is None else _p(w1, U64),
                            None if rand is None else _p(rand, U64), r0, r1)


def walk(L, nr, nc, w0, w1):
    lib().oracle_walk(L, nr, nc, _p(w0, U64), _p(w1, U64), 0, nr)


def gen_rndbits(L, nr, te, keys, lut):
    H = (L // 4) ** 3 // 2
    out = np.zeros(3 * H * nr, np.uint64)
    lb = np.frombuffer(bytes(lut), np.uint8).copy()
    lib().oracle_gen_rndbits(L, nr, _p(te, U32), _p(keys, U32), lb.ctypes.data_as(C.c_void_p),
                             _p(out, U64))
    return out


def metropolis_iteration(L, nr, J, even, odd, te0, te1, keys, lut):
    lb = np.frombuffer(bytes(lut), np.uint8).copy()
    lib().oracle_metropolis_iteration(L, nr, _p(J, U64), _p(even, U64), _p(odd, U64), _p(te0, U32),
                                      _p(te1, U32), _p(keys, U32), lb.ctypes.data_as(C.c_void_p))


def energy(L, nr, J, even, odd):
    e = np.zeros(nr, np.int32)
    lib().oracle_energy(L, nr, _p(J, U64), _p(even, U64), _p(odd, U64), _p(e, I32))
    return e


def demon_energy(L, nr, nc, w0, w1):
    e = np.zeros(nr, np.uint64)
    lib().oracle_demon_energy(L, nr, nc, _p(w0, U64), _p(w1, U64), _p(e, U64))
    return e


def overlap_c4(L, nr, uu):
    uu = np.ascontiguousarray(uu, np.uint8)
    nd = L // 2 + 1
    q = np.zeros(nr // 2, np.int64)
    c4 = np.zeros(nr // 2 * 3 * nd, np.int64)
    lib().oracle_overlap_c4(L, nr, _p(uu, U8), _p(q, I64), _p(c4, I64))
    return q, c4.reshape(nr // 2, 3, nd)


def scalar_rule(u, d):
    f = C.c_int()
    nd = lib().oracle_scalar_rule(u, d, C.byref(f))
    return nd, f.value


def isi_word(j1, j2, j3, j4, d0, d1):
    a, b = C.c_uint64(d0), C.c_uint64(d1)
    f = lib().oracle_isi_word(j1, j2, j3, j4, C.byref(a), C.byref(b))
    return f, a.value, b.value


def scalar_energy(L, u, Jx, Jy, Jz):
    return lib().oracle_scalar_energy(L, _p(np.ascontiguousarray(u, np.uint8), U8), _p(Jx, U8),
                                      _p(Jy, U8), _p(Jz, U8))


def pack_couplings(L, Jx, Jy, Jz):
    H = (L // 4) ** 3 // 2
    J = np.zeros(12 * H, np.uint64)
    src = [np.ascontiguousarray(a, np.uint8) for a in (Jx, Jy, Jz)]  # alive across the call
    lib().oracle_pack_couplings(L, *(_p(a, U8) for a in src), _p(J, U64))
    return J


def tables(L):
    H = (L // 4) ** 3 // 2
    neig = np.zeros(12 * H, np.int32)
    rot = np.zeros(2 * H, np.uint8)
    lib().oracle_tables(L, _p(neig, I32), _p(rot, U8))
    return neig.reshape(2, 6, H), rot.reshape(2, H)
