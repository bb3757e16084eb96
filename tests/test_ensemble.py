"""Snapshots, restart files and the batched ensemble.

Parity bar: a member of the ensemble, a run resumed from a snapshot and a
run resumed from a restart file are bit-identical to the same parameters
run alone, because they launch the same kernels on the same data.
"""
import numpy as np
import pytest

import sph_cuda_gb300 as sph
from sph_cuda_gb300 import Asph, Ensemble, ensemble_members
from statebuild import small_config

FIELDS = ("x", "y", "z", "u", "v", "w", "th", "qv", "qc", "rho", "prs")


def _same(a, b):
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k


# ---- host logic (CPU) -------------------------------------------------------
def test_ensemble_members_follow_the_workload_description():
    m = ensemble_members(64, seed=7)
    n = np.array([p.n_particles for p in m])
    assert len(m) == 64
    assert n.min() >= 2 * 20 ** 3 and n.max() <= 524288
    assert n.sum() == sum(2 * p.lat_nx ** 3 for p in m)
    for p in m:
        sph.check_params(p)
        assert p.lat_nz == 2 * p.lat_nx
        # the small box's lattice spacing and cell size
        assert abs(p.nx * p.dx / p.lat_nx - 312.5) < 1e-3
        assert abs(p.nz * p.dz / p.lat_nz - 78.125) < 1e-3
        # cells per axis = floor(L / h), so the cell edge exceeds h by less than 1/31
        assert 200.0 <= p.dx < 200.0 * (1 + 1 / 31.0) and 50.0 <= p.dz < 50.0 * (1 + 1 / 62.0)
    # log-uniform: about half the members below the geometric mean of the bounds
    below = np.sum(n < np.sqrt(16384 * 524288))
    assert 20 <= below <= 44
    # deterministic in the seed
    assert [p.n_particles for p in ensemble_members(64, seed=7)] == list(n)


# ---- GPU ------------------------------------------------------------------------
def _members():
    return [small_config(lat=(12, 12, 24), grid=(16, 16, 40), box=(3200.0, 3200.0, 2000.0), seed=1),
            small_config(lat=(16, 16, 32), grid=(20, 20, 40), box=(4000.0, 4000.0, 2000.0), seed=2),
            small_config(lat=(10, 10, 20), grid=(12, 12, 30), box=(2400.0, 2400.0, 1500.0), seed=3, sort_every=2)]


@pytest.mark.gpu
def test_snapshot_restore_continues_bit_identically():
    p = small_config(sort_every=0)   # displacement-gated: the stale cell table is part of the state
    sim = Asph(p)
    sim.init()
    sim.step(3)
    snap = sim.snapshot()
    sim.step(4)
    a = sim.get_state()
    ca = sim.control()
    sim.restore(snap)
    sim.step(4)
    b = sim.get_state()
    cb = sim.control()
    _same(a, b)
    assert ca["step"] == cb["step"] == 7 and ca["simt"] == cb["simt"] and ca["sort_count"] == cb["sort_count"]
    ra, pa = sim.get_rain()
    snap.close()
    sim.close()


@pytest.mark.gpu
def test_restart_file_round_trip(tmp_path):
    p = small_config(sort_every=0)
    sim = Asph(p)
    sim.init()
    sim.step(3)
    sim.checkpoint_write(str(tmp_path / "r.bin"))
    sim.step(4)
    a = sim.get_state()
    ra = sim.get_rain()
    other = Asph(p)
    other.checkpoint_read(str(tmp_path / "r.bin"))
    assert other.control()["step"] == 3
    other.step(4)
    _same(a, other.get_state())
    assert np.array_equal(ra[0], other.get_rain()[0])
    # a context of another size refuses the file
    q = small_config(lat=(8, 8, 16))
    small = Asph(q)
    with pytest.raises(sph.AsphError):
        small.checkpoint_read(str(tmp_path / "r.bin"))
    for s in (sim, other, small):
        s.close()


@pytest.mark.gpu
def test_reinit_after_steps_sorts_like_a_fresh_context():
    """A second init on a used context: the radix look-back epoch keeps
    growing, so status words of the earlier run are never taken as current."""
    p = small_config(sort_every=1)
    a = Asph(p)
    a.init()
    a.step(5)
    a.init()
    a.step(2)
    b = Asph(p)
    b.init()
    b.step(2)
    _same(a.get_state(), b.get_state())
    assert np.array_equal(a.get_sort()["perm"], b.get_sort()["perm"])
    a.close()
    b.close()


@pytest.mark.gpu
def test_ensemble_members_equal_solo_runs():
    ms = _members()
    ens = Ensemble(ms)
    ens.init()
    ens.step(6)
    ens.sync()
    for k, p in enumerate(ms):
        solo = Asph(p)
        solo.init()
        solo.step(6)
        m = ens.member(k)
        _same(m.get_state(), solo.get_state())
        assert m.control()["step"] == 6
        assert np.array_equal(m.get_rain()[0], solo.get_rain()[0])
        solo.close()
    ens.close()


@pytest.mark.gpu
def test_ensemble_member_calls_are_ordered_after_queued_steps():
    ms = _members()[:2]
    ens = Ensemble(ms)
    ens.init()
    ens.step_async(3)
    st = ens.member(1).get_state()   # must see all three steps
    solo = Asph(ms[1])
    solo.init()
    solo.step(3)
    _same(st, solo.get_state())
    ens.close()
    solo.close()


@pytest.mark.gpu
def test_tuner_keeps_state_and_choices_reproduce_solo_runs():
    ms = _members()[:2]
    ens = Ensemble(ms)
    ens.init()
    ens.step(2)
    before = [ens.member(k).get_state() for k in range(2)]
    chosen = ens.tune(trial_steps=2, sort_choices=(1, 2))
    assert len(chosen) == 2
    for k, (shape, cad, tpt) in enumerate(chosen):
        assert shape in (-1, 0, 1, 2, 3) and cad in (1, 2) and tpt in (1, 2, 4)
        m = ens.member(k)
        _same(before[k], m.get_state())
        assert m.control()["step"] == 2
        assert m.sort_every() == cad and m.targets_per_thread() == tpt
    ens.step(3)
    for k, (shape, cad, tpt) in enumerate(chosen):
        solo = Asph(ms[k])
        solo.init()
        solo.step(2)
        if shape < 0:
            solo.set_pair_path(True)
        else:
            solo.set_pair_shape(shape)
        solo.set_sort_every(cad)
        solo.set_targets_per_thread(tpt)
        solo.step(3)
        _same(ens.member(k).get_state(), solo.get_state())
        solo.close()
    ens.close()


@pytest.mark.gpu
def test_pair_shape_option_validates():
    p = small_config()
    sim = Asph(p)
    with pytest.raises(sph.AsphError):
        sim.set_pair_shape(7)
    sim.set_pair_shape(-1)
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("tpt", [1, 4])
def test_momentum_targets_per_thread_do_not_change_results(tpt):
    """The momentum pass's targets per thread (the cells one warp covers)
    is a launch shape only: states are bit-identical to the default's."""
    p = small_config()
    a, b = Asph(p), Asph(p)
    a.init(); b.init()
    b.set_targets_per_thread(tpt)
    assert b.targets_per_thread() == tpt and a.targets_per_thread() == 2
    a.step(4); b.step(4)
    _same(a.get_state(), b.get_state())
    with pytest.raises(sph.AsphError):
        b.set_targets_per_thread(3)
    a.close(); b.close()
