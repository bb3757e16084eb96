"""Source-term hook: per-particle additive tendencies in the theta update,
attached to particles through sorts, settable from host arrays or a CUDA
tensor; the device state copy for a model reading the state."""
import numpy as np
import pytest

from sph_cuda_gb300 import Asph
from statebuild import random_state, small_config


def _pair(p, s):
    a, b = Asph(p), Asph(p)
    for sim in (a, b):
        sim.set_state(s)
        sim.sort_build()
        sim.set_time(0.0, 0.25, True)
    return a, b


@pytest.mark.gpu
def test_constant_tendencies_add_dt_times_source():
    p = small_config(sort_every=1)
    s = random_state(p, seed=2, speed=2.0)
    ref, hook = _pair(p, s)
    hook.enable_source(True)
    N = p.n_particles
    hook.set_source(np.full(N, 2e-3), np.full(N, 1e-7), np.full(N, 2e-7))
    ref.step(1)
    hook.step(1)
    a, b = ref.get_state(), hook.get_state()
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["u"], b["u"])
    dt = 0.25
    assert np.allclose(b["th"] - a["th"], dt * 2e-3, atol=4e-5)
    ok = a["qv"] > 0
    assert np.allclose((b["qv"] - a["qv"])[ok], dt * 1e-7, atol=2e-9)
    assert np.allclose(b["qc"] - a["qc"], dt * 2e-7, atol=2e-9)
    ref.close()
    hook.close()


@pytest.mark.gpu
def test_tendencies_follow_their_particles_through_the_sort():
    """Tendencies set on a shuffled state follow their particles through the
    sort that orders it and through the step's own sort."""
    p = small_config(sort_every=1)
    s = random_state(p, seed=4, speed=5.0)          # shuffled order
    N = p.n_particles
    S = np.linspace(0.0, 4e-3, N).astype(np.float32)     # one value per particle, shuffled order
    ref, hook = Asph(p), Asph(p)
    for sim in (ref, hook):
        sim.set_state(s)
    hook.enable_source(True)
    hook.set_source(S)
    for sim in (ref, hook):
        sim.sort_build()
        sim.set_time(0.0, 0.25, True)
    perm0 = hook.get_sort()["perm"]                      # sorted position -> shuffled position
    assert not np.array_equal(perm0, np.arange(N))
    ref.step(1)
    hook.step(1)
    perm1 = hook.get_sort()["perm"]                      # the step's own sort
    assert np.array_equal(perm1, ref.get_sort()["perm"])
    a, b = ref.get_state(), hook.get_state()
    assert np.allclose(b["th"] - a["th"], 0.25 * S[perm0[perm1]], atol=4e-5)
    ref.close()
    hook.close()


@pytest.mark.gpu
def test_device_state_and_tensor_source():
    torch = pytest.importorskip("torch")
    p = small_config(sort_every=1)
    s = random_state(p, seed=6)
    a, b = _pair(p, s)
    N = p.n_particles
    pos = torch.empty((N, 4), dtype=torch.float32, device="cuda")
    thq = torch.empty((N, 4), dtype=torch.float32, device="cuda")
    a.state_device(pos=pos, thq=thq)
    st = a.get_state()
    assert np.array_equal(pos[:, 0].cpu().numpy(), st["x"])
    assert np.array_equal(thq[:, 0].cpu().numpy(), st["th"])
    # a "model": tendencies computed on the GPU from the device state
    src = torch.zeros((N, 4), dtype=torch.float32, device="cuda")
    src[:, 0] = 1e-3 * torch.tanh(thq[:, 0] - 300.0)
    a.enable_source(True)
    b.enable_source(True)
    a.set_source_device(src)
    b.set_source(src[:, 0].cpu().numpy())
    a.step(2)
    b.step(2)
    assert np.array_equal(a.get_state()["th"], b.get_state()["th"])
    a.close()
    b.close()


@pytest.mark.gpu
def test_source_hook_off_by_default_and_detachable():
    p = small_config(sort_every=1)
    s = random_state(p, seed=8)
    ref, hook = _pair(p, s)
    hook.enable_source(True)
    hook.set_source(np.full(p.n_particles, 1e-2))
    hook.enable_source(False)
    ref.step(2)
    hook.step(2)
    assert np.array_equal(ref.get_state()["th"], hook.get_state()["th"])
    ref.close()
    hook.close()
