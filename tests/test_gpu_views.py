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
