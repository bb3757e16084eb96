"""State exchange with host arrays: pinned arrays go through the direct
pack/unpack kernels, pageable arrays through the staged copies; both give
the same state, for full and partial field sets."""
import numpy as np
import pytest

from sph_cuda_gb300 import Asph, STATE_FIELDS
from statebuild import random_state, small_config


def _pinned_like(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.gpu
def test_pinned_and_pageable_state_exchange_agree():
    p = small_config(sort_every=1)
    s = random_state(p, seed=12)
    a = Asph(p)
    a.set_state(s)
    a.step(3)
    pageable = a.get_state()
    pinned_out = {k: _pinned_like(np.zeros(p.n_particles, np.float32)) for k in STATE_FIELDS}
    got = a.get_state(STATE_FIELDS, out=pinned_out)
    for k in STATE_FIELDS:
        assert np.array_equal(got[k], pageable[k]), k
    # a partial pinned read
    part = a.get_state(("th", "qc"), out={"th": _pinned_like(np.zeros(p.n_particles)),
                                         "qc": _pinned_like(np.zeros(p.n_particles))})
    assert np.array_equal(part["th"], pageable["th"]) and np.array_equal(part["qc"], pageable["qc"])
    # two fresh contexts set from the same values, pageable and pinned
    b, c = Asph(p), Asph(p)
    b.set_state(pageable)
    c.set_state({k: _pinned_like(v) for k, v in pageable.items()})
    sb, sc = b.get_state(), c.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sb[k], pageable[k]) and np.array_equal(sc[k], pageable[k]), k
    b.step(2)
    c.step(2)
    sb, sc = b.get_state(), c.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sb[k], sc[k]), k
    for sim in (a, b, c):
        sim.close()


def _pinned_offset(a, off):
    """A pinned copy of `a` that starts `off` floats into its allocation (off = 1:
    not 16-byte aligned)."""
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape[0] + 4, dtype=torch.float32, pin_memory=True).numpy()[off:off + a.shape[0]]
    t[...] = a
    return t


@pytest.mark.gpu
def test_pinned_exchange_ragged_count_and_unaligned_arrays():
    """A particle count that is not a multiple of 4, with 16-byte aligned
    pinned arrays and with arrays that start one float into their pinned
    allocation: set and get return the state they were given."""
    p = small_config(lat=(15, 15, 15), grid=(20, 20, 40))
    assert p.n_particles % 4 == 3
    s = {k: v for k, v in random_state(p, seed=5, layout="uniform").items()}
    ref = Asph(p)
    ref.set_state(s)
    want = ref.get_state()
    for off in (0, 1):
        sim = Asph(p)
        sim.set_state({k: _pinned_offset(np.asarray(v, np.float32), off) for k, v in want.items()})
        back = sim.get_state()
        out = {k: _pinned_offset(np.zeros(p.n_particles, np.float32), off) for k in STATE_FIELDS}
        got = sim.get_state(STATE_FIELDS, out=out)
        for k in STATE_FIELDS:
            assert np.array_equal(back[k], want[k]), (off, k)
            assert np.array_equal(got[k], want[k]), (off, k)
        sim.close()
    ref.close()
