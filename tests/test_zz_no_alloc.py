"""The allocation-free sort entry point, for callers that cannot allocate device memory (device
memory owned by the host application's allocator or budget, frame loops that cannot stall on an
allocation).

akua_sort_pairs_noalloc runs the step's stable radix sort with its temporary storage in a fixed
device array inside the library.  These tests call it through the C ABI on the pre-sort cell
hashes of a real step and check that it reproduces the sorted hashes and order that akua_pbf_step
itself produced (integer data: exactly), on two calls in a row that share the array; they also
sort caller payloads and keys with bits above keyBits against a stable host sort of the masked
keys.  This file is collected last so that a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

import akuaengine_gb300 as ak
from akuaengine_gb300 import LambdaCorrParams, PBFConfig, PBFSolver, scene



def _step_sorted(sc, steps):
    """Runs akua_pbf_step and returns (pre-sort keys, sorted keys, order, key bits) of the last
    step's cell-hash sort."""
    cfg, corr = PBFConfig(), LambdaCorrParams()
    p = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr) as s:
        for _ in range(steps):
            s.step_host(p, sc.dt, sc.box_min, sc.box_max)
        hashes = s.read_debug(ak.DEBUG_HASHES)
        order = s.read_debug(ak.DEBUG_ORDER)
    pre = np.empty_like(hashes)
    pre[order] = hashes  # order[s] = pre-sort index of the particle now at s
    bits = int(cfg.maxNeighbours * sc.n - 1).bit_length()
    return pre, hashes, order, bits


def _noalloc(lib, torch, keys_host, bits, stream, vals_host=None):
    n = len(keys_host)
    keys_in = torch.from_numpy(keys_host.astype(np.uint32).view(np.int32)).cuda()
    vals_in = (None if vals_host is None else
               torch.from_numpy(vals_host.astype(np.uint32).view(np.int32)).cuda())
    keys_out = torch.empty(n, dtype=torch.int32, device="cuda")
    vals_out = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.akua_sort_pairs_noalloc(ctypes.c_void_p(keys_in.data_ptr()),
                                     None if vals_in is None else ctypes.c_void_p(vals_in.data_ptr()),
                                     ctypes.c_void_p(keys_out.data_ptr()),
                                     ctypes.c_void_p(vals_out.data_ptr()), n, bits,
                                     ctypes.c_void_p(stream))
    assert rc == 0, ak._abi.status_string(rc)
    torch.cuda.synchronize()
    return keys_out.cpu().numpy().view(np.uint32), vals_out.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_noalloc_sort_matches_step_sort_twice(cuda_lib):
    torch = pytest.importorskip("torch")
    sc = scene.workload("dam_break_27k", seed=3)
    for steps in (1, 2):  # two calls in a row; the second reuses the array's stale contents
        pre, hashes, order, bits = _step_sorted(sc, steps)
        keys, vals = _noalloc(cuda_lib, torch, pre, bits, 0)
        assert np.array_equal(keys, hashes)
        assert np.array_equal(vals, order)


@pytest.mark.gpu
def test_noalloc_sort_at_the_size_limit_and_beyond(cuda_lib):
    torch = pytest.importorskip("torch")
    n = 1 << 20  # AKUA_SORT_NOALLOC_MAX_PAIRS
    rng = np.random.default_rng(0)
    keys = rng.integers(0, 1 << 27, size=n, dtype=np.uint32)
    for _ in range(2):
        k, v = _noalloc(cuda_lib, torch, keys, 27, 0)
        ref = np.argsort(keys, kind="stable").astype(np.uint32)
        assert np.array_equal(v, ref) and np.array_equal(k, keys[ref])
    big = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    out = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    out2 = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    rc = cuda_lib.akua_sort_pairs_noalloc(ctypes.c_void_p(big.data_ptr()), None,
                                          ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(out2.data_ptr()), n + 1, 27, None)
    assert rc == ak.AKUA_ERR_TOO_LARGE


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [1, 4, 11, 12, 27, 32])
def test_noalloc_sort_ignores_key_bits_above_key_bits(cuda_lib, bits):
    """Keys carry random bits above keyBits; the order must be that of the masked keys, ties in
    input order, and the caller's payload must travel with its key (two calls in a row)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(bits)
    n = 70_001  # several tiles and a ragged last tile
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    payload = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    mask = np.uint32((1 << bits) - 1) if bits < 32 else np.uint32(0xFFFFFFFF)
    order = np.argsort(keys & mask, kind="stable")
    for _ in range(2):
        k, v = _noalloc(cuda_lib, torch, keys, bits, 0, vals_host=payload)
        assert np.array_equal(k, keys[order])
        assert np.array_equal(v, payload[order])


def test_noalloc_sort_rejects_overlapping_arrays(cuda_lib):
    """Outputs that share memory with an input or with each other are refused before any device
    work (the addresses below are never dereferenced, so this runs without a GPU)."""
    n = 1000
    a, b, c, d = 0x100000, 0x200000, 0x300000, 0x400000
    step = 4 * n
    call = cuda_lib.akua_sort_pairs_noalloc
    def rc(ki, vi, ko, vo):
        return call(ctypes.c_void_p(ki), None if vi is None else ctypes.c_void_p(vi),
                    ctypes.c_void_p(ko), ctypes.c_void_p(vo), n, 20, None)
    bad = ak.AKUA_ERR_INVALID_ARGUMENT
    assert rc(a, b, a, d) == bad               # keys in == keys out
    assert rc(a, b, c, a) == bad               # keys in == vals out
    assert rc(a, b, b, d) == bad               # vals in == keys out
    assert rc(a, b, c, b) == bad               # vals in == vals out
    assert rc(a, b, c, c) == bad               # keys out == vals out
    assert rc(a, None, c, c + step - 4) == bad  # partial overlap of the outputs
    assert rc(a, None, a + step - 4, d) == bad  # partial overlap of keys in and keys out
    assert call(ctypes.c_void_p(a), None, ctypes.c_void_p(c), ctypes.c_void_p(d), -1, 20,
                None) == bad
    assert call(ctypes.c_void_p(a), None, ctypes.c_void_p(c), ctypes.c_void_p(d), n, 33,
                None) == bad
