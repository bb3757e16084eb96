"""asph_sort_keys_noalloc: the Morton-key sort without any allocation.

Callers that must not call cudaMalloc/cudaFree (a latency-critical step
loop where cudaFree would synchronise the device, a host callback or a
foreign-language runtime that must not block in the allocator, an
application whose memory pool owns the device) get the step's stable key
sort with its scratch in a static device array.  This file checks, through
the C ABI, that two calls in a row give exactly the permutation and sorted
keys of the existing entry point (asph_sort_build), and that sizes above the
stated maximum are refused.  It is collected last and needs no state from
other tests.
"""
import ctypes

import numpy as np
import pytest

from sph_cuda_gb300 import Asph, abi
from statebuild import small_config, random_state

pytestmark = pytest.mark.gpu


def _key_bits(p):
    b = 1
    while (1 << b) < max(p.nx, p.ny, p.nz):
        b += 1
    return 3 * b


def _reference_sort(p, s):
    """Keys of state s and their sort through the existing entry point."""
    sim = Asph(p)
    sim.set_state(s)
    keys = sim.get_sort()["keys_in"].copy()
    sim.sort_build()
    out = sim.get_sort()
    sim.close()
    return keys, out["keys_sorted"], out["perm"]


def _noalloc(lib, torch, keys, key_bits):
    n = keys.size
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    ks = torch.empty(n, dtype=torch.int32, device="cuda")
    pm = torch.empty(n, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.asph_sort_keys_noalloc(ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(ks.data_ptr()),
                                    ctypes.c_void_p(pm.data_ptr()), n, key_bits, ctypes.c_void_p(st))
    assert rc == abi.ASPH_OK, lib.asph_last_error()
    return ks.cpu().numpy().view(np.uint32), pm.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_sort_build_twice():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    # two different states of different sizes, sorted back to back
    cases = []
    p1 = small_config(lat=(64, 64, 64), grid=(40, 40, 80), box=(8000.0, 8000.0, 4000.0))
    cases.append((p1, random_state(p1, 21, "uniform")))
    p2 = small_config(lat=(30, 28, 20))
    cases.append((p2, random_state(p2, 22, "cluster")))
    for p, s in cases:
        keys, ref_sorted, ref_perm = _reference_sort(p, s)
        got_sorted, got_perm = _noalloc(lib, torch, keys, _key_bits(p))
        assert np.array_equal(got_perm, ref_perm)
        assert np.array_equal(got_sorted, ref_sorted)


def test_noalloc_sort_at_the_size_limit():
    """n = ASPH_NOALLOC_MAX_KEYS, where the scratch buffers are full: random
    30-bit keys, twice in a row, against numpy's stable argsort."""
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    rng = np.random.default_rng(23)
    for _ in range(2):
        keys = rng.integers(0, 1 << 30, abi.NOALLOC_MAX_KEYS, dtype=np.uint32)
        keys[:1000] = keys[1000:2000]   # ties: stability matters
        got_sorted, got_perm = _noalloc(lib, torch, keys, 30)
        ref_perm = np.argsort(keys, kind="stable").astype(np.uint32)
        assert np.array_equal(got_perm, ref_perm)
        assert np.array_equal(got_sorted, keys[ref_perm])


def test_noalloc_sort_rejects_oversize():
    lib = abi.load_library()
    n = abi.NOALLOC_MAX_KEYS + 1
    rc = lib.asph_sort_keys_noalloc(ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1), n, 24, None)
    assert rc == abi.ASPH_ERR_ARG
    assert b"ASPH_NOALLOC_MAX_KEYS" in lib.asph_last_error()
