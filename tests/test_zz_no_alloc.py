"""micsa_energy_noalloc: spin energies for callers that cannot allocate
device memory when they measure (services that size their memory once,
real-time loops, processes whose device memory belongs to another allocator).
The caller owns every buffer and passes the reference's own row tables (one
device allocation per row, as mmcuda makes them); the entry point keeps its
counters in a fixed device array shared by every call.  Its results must
equal the oracle's energies and those of the context's measurement
(micsa_measure) exactly -- energies are integers -- on consecutive calls,
since the counter array is reused by every call.

This file is collected last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import micsa
import oracle

pytestmark = pytest.mark.gpu


def _state(rng, L, nr, ns):
    H = (L // 4) ** 3 // 2
    V = L ** 3
    out = []
    for _ in range(ns):
        J = oracle.pack_couplings(L, *(rng.integers(0, 2, size=V, dtype=np.uint8) for _ in range(3)))
        e = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        o = rng.integers(0, 2 ** 64 - 1, size=H * nr, dtype=np.uint64, endpoint=True)
        out.append((J, e, o))
    return out


def _oracle_energies(L, nr, st):
    return np.concatenate([oracle.energy(L, nr, J, e, o) for J, e, o in st])


def _context_energies(L, nr, ns, st):
    with micsa.Context(L, nr, ns, 1) as ctx:
        for s, (J, e, o) in enumerate(st):
            ctx.upload_couplings(s, J)
            ctx.upload_spins(s, e, o)
        return ctx.measure(spin=True, demon=False)["e_spin"].reshape(-1)


def _noalloc_energies(L, nr, ns, st):
    """One call through the C ABI with the reference's row tables: two spin
    rows and twelve coupling rows per sample, each its own device buffer."""
    import torch
    dev = torch.device("cuda:0")
    H = (L // 4) ** 3 // 2
    as_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).to(dev)
    keep = []
    spin_rows, J_rows = [], []
    for J, e, o in st:
        for row in (e, o):
            keep.append(as_dev(row))
            spin_rows.append(keep[-1].data_ptr())
        for k in range(12):
            keep.append(as_dev(J[k * H:(k + 1) * H]))
            J_rows.append(keep[-1].data_ptr())
    out = torch.full((ns * nr,), -1, dtype=torch.int32, device=dev)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = micsa.lib().micsa_energy_noalloc(L, nr, ns, (C.c_void_p * len(spin_rows))(*spin_rows),
                                          (C.c_void_p * len(J_rows))(*J_rows), out.data_ptr(),
                                          stream, err, 256)
    assert rc == micsa.MICSA_OK, err.value.decode()
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


@pytest.mark.parametrize("L,nr,ns", [(8, 32, 1), (16, 64, 2), (24, 32, 1), (40, 96, 3)])
def test_noalloc_energy_equals_oracle_and_context_measure_twice(L, nr, ns):
    rng = np.random.default_rng(L * 7 + nr)
    for call in range(2):  # consecutive calls reuse the shared counters
        st = _state(rng, L, nr, ns)
        got = _noalloc_energies(L, nr, ns, st)
        assert np.array_equal(got, _oracle_energies(L, nr, st)), "call %d vs oracle" % call
        assert np.array_equal(got, _context_energies(L, nr, ns, st)), "call %d vs context" % call


@pytest.mark.parametrize("L,nr,ns", [(8, 40, 2), (16, 7, 20)])
def test_noalloc_energy_any_replica_count_equals_oracle(L, nr, ns):
    """Replica counts the context does not take (not a multiple of 32), and
    more samples than one launch carries (16), against the oracle alone;
    L = 8 is the smallest lattice, where the +1 and -1 neighbours of a block
    coordinate are the same block."""
    rng = np.random.default_rng(L + nr)
    for call in range(2):
        st = _state(rng, L, nr, ns)
        assert np.array_equal(_noalloc_energies(L, nr, ns, st), _oracle_energies(L, nr, st)), call


def test_noalloc_rejects_more_replicas_than_counters():
    err = C.create_string_buffer(256)
    dummy = (C.c_void_p * 64)(*([16] * 64))  # never dereferenced: the size check comes first
    rc = micsa.lib().micsa_energy_noalloc(16, micsa.NOALLOC_MAX_REPLICAS, 2, dummy, dummy,
                                          C.c_void_p(16), None, err, 256)
    assert rc == micsa.MICSA_ERR_ARG and b"exceeds" in err.value


def test_noalloc_rejects_lattices_whose_energy_overflows_int32():
    err = C.create_string_buffer(256)
    dummy = (C.c_void_p * 24)(*([16] * 24))
    rc = micsa.lib().micsa_energy_noalloc(micsa.NOALLOC_MAX_L + 8, 32, 1, dummy, dummy,
                                          C.c_void_p(16), None, err, 256)
    assert rc == micsa.MICSA_ERR_ARG and b"888" in err.value
    assert 3 * micsa.NOALLOC_MAX_L ** 3 < 2 ** 31 <= 3 * (micsa.NOALLOC_MAX_L + 8) ** 3
