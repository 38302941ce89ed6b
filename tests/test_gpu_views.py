"""Zero-copy device views of a scene's state (capi.Scene.device_array, over
pbf_scene_device_field): a consumer of __cuda_array_interface__ (torch here)
sees the scene's own memory, equal to what pbf_scene_read copies out, and
later steps show through the same view."""
import numpy as np
import pytest

from novaphy_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_device_views_are_live_and_equal_the_copies():
    torch = pytest.importorskip("torch")
    w = workloads.dam_break_8k()
    sc = capi.Scene(capi.default_settings(**w.settings), w.x, w.v, mass=w.mass)
    sc.set_gravity(w.gravity)
    sc.step(w.dt, 1)
    views = {f: torch.as_tensor(sc.device_array(f), device="cuda")
             for f in (capi.FIELD_POSITIONS, capi.FIELD_VELOCITIES, capi.FIELD_DENSITIES,
                       capi.FIELD_LAMBDAS)}
    assert views[capi.FIELD_POSITIONS].shape == (w.n, 3)
    assert views[capi.FIELD_POSITIONS].stride() == (4, 1)
    assert views[capi.FIELD_DENSITIES].shape == (w.n,)
    for _ in range(2):
        for f, t in views.items():
            got = t.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), sc.read(f).view(np.uint32)), f
        sc.step(w.dt, 1)  # the same tensors follow the scene
        sc.sync()
    x = views[capi.FIELD_POSITIONS]
    assert x.data_ptr() == sc.device_field(capi.FIELD_POSITIONS)


def test_fluid_world_pinned_and_device_views():
    """FluidWorld.fluid_arrays(): read-only numpy views of page-locked host
    memory, equal to the copying fluid_state accessors and rewritten in place
    after the next step; FluidWorld.fluid_device_arrays(): the device memory
    itself through __cuda_array_interface__."""
    torch = pytest.importorskip("torch")
    import warnings

    import novaphy_gb300 as nv

    spec = workloads.coupled_pool()
    lower, upper, _ = spec["block"]
    # A small corner of the pool, with one sphere in it, stands for a demo world.
    mb = nv.ModelBuilder()
    mb.add_shape(nv.CollisionShape.make_plane([0.0, 0.0, 1.0], 0.0))
    bi = mb.add_body(nv.RigidBody.from_sphere(5.0, 0.05),
                     nv.Transform.from_translation([0.7, 0.7, 0.12]))
    mb.add_shape(nv.CollisionShape.make_sphere(0.05, bi))
    blk = nv.FluidBlockDef()
    blk.lower = list(lower)
    blk.upper = [lower[0] + 0.2, lower[1] + 0.2, 0.2]
    blk.particle_spacing = 0.02
    st = nv.PBFSettings()
    st.kernel_radius = 0.08
    world = nv.FluidWorld(mb.build(), [blk], nv.SolverSettings(), st, 1.0)
    world.set_gravity([0.0, 0.0, -9.81])
    n = world.num_particles
    assert n > 500
    dt = 1.0 / 240.0
    world.step(dt)
    host = world.fluid_arrays()
    assert host["positions"].shape == (n, 3) and host["densities"].shape == (n,)
    assert not host["positions"].flags.writeable
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # torch warns that the array is read-only
        assert torch.from_numpy(host["velocities"]).is_pinned()
    for _ in range(2):
        fs = world.fluid_state
        want = {"positions": fs.positions_array, "velocities": fs.velocities_array,
                "densities": fs.densities_array, "lambdas": fs.lambdas_array}
        again = world.fluid_arrays()
        dev = world.fluid_device_arrays()
        for k in want:
            assert np.shares_memory(again[k], host[k]), k  # the same pinned buffer
            assert np.array_equal(host[k], want[k]), k
            t = torch.as_tensor(dev[k], device="cuda")
            assert t.shape == want[k].shape
            assert np.array_equal(t.cpu().numpy(), want[k]), k
        world.step(dt)
