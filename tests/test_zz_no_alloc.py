"""micsa_energy_noalloc: spin energies for callers that cannot allocate
device memory when they measure (services that size their memory once,
real-time loops, processes whose device memory belongs to another allocator).
The caller owns every buffer; the entry point keeps its counters in a fixed
device array.  Its results must equal those of the context's measurement
(micsa_measure) exactly -- energies are integers -- on consecutive calls,
since the counter array is shared and reused by every call.
"""
import ctypes as C

import numpy as np
import pytest

import micsa

pytestmark = pytest.mark.gpu


def _state(rng, L, nr, ns):
    H = (L // 4) ** 3 // 2
    V = L ** 3
    out = []
    for _ in range(ns):
        J = micsa.pack_couplings(L, *(rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
        e = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        o = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        out.append((J, e, o))
    return out


def _context_energies(L, nr, ns, st):
    with micsa.Context(L, nr, ns, 1) as ctx:
        for s, (J, e, o) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
        return ctx.measure(spin=True, demon=False)["e_spin"].reshape(-1)


def _noalloc_energies(L, nr, ns, st):
    import torch
    dev = torch.device("cuda:0")
    as_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).to(dev)
    even = as_dev(np.concatenate([x[1] for x in st]))
    odd = as_dev(np.concatenate([x[2] for x in st]))
    J = as_dev(np.concatenate([x[0] for x in st]))
    out = torch.full((ns * nr,), -1, dtype=torch.int32, device=dev)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = micsa.lib().micsa_energy_noalloc(L, nr, ns, even.data_ptr(), odd.data_ptr(), J.data_ptr(),
                                          out.data_ptr(), stream, err, 256)
    assert rc == micsa.MICSA_OK, err.value.decode()
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


@pytest.mark.parametrize("L,nr,ns", [(16, 64, 2), (24, 32, 1), (40, 96, 3)])
def test_noalloc_energy_equals_context_measure_twice(L, nr, ns):
    rng = np.random.default_rng(L * 7 + nr)
    for call in range(2):  # consecutive calls reuse the shared counters
        st = _state(rng, L, nr, ns)
        want = _context_energies(L, nr, ns, st)
        got = _noalloc_energies(L, nr, ns, st)
        assert np.array_equal(got, want), "call %d" % call


def test_noalloc_rejects_more_replicas_than_counters():
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = micsa.lib().micsa_energy_noalloc(16, micsa.NOALLOC_MAX_REPLICAS, 2, dummy, dummy, dummy,
                                          dummy, None, err, 256)
    assert rc == 1 and b"exceeds" in err.value
