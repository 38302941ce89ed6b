"""The premise of the GPU step's runs (k_segments in the CUDA kernels): in the
reference's step, restated by the oracle, particles with bit-identical state
(position, velocity, density and lambda) in the same cell come out
bit-identical, step after step, because every sum they take sees the same
terms in the same order.  A small dam break with a clump of identical
particles inside the block and another clamped into the box corner."""
import numpy as np

from novaphy_gb300 import workloads


def test_identical_particles_stay_identical(port):
    from oracle.oracle import Settings

    w = workloads.dam_break((16, 16, 16), 0.025, (1.0, 1.0, 1.0), dt=1.0 / 120.0, seed=4,
                           vorticity=1e-4)
    inside = np.full((300, 3), 0.2125, np.float32)
    corner = np.full((200, 3), 0.0125, np.float32)
    x = np.concatenate([w.x[:2000], inside[:150], w.x[2000:], inside[150:], corner])
    x = x.astype(np.float32)
    v = np.zeros_like(x)
    z = np.zeros(len(x), np.float32)
    n0 = len(w.x)
    groups = [np.r_[2000:2150, n0 + 150:n0 + 300], np.arange(n0 + 300, n0 + 500)]
    st = Settings.make(**w.settings)
    state = (x, v, z, z)
    for _ in range(2):
        state = port.steps(st, *state, w.dt, w.gravity, w.mass, 1)
        for g in groups:
            for a in state:
                a = np.asarray(a).reshape(len(x), -1)[g]
                assert (a.view(np.uint32) == a[:1].view(np.uint32)).all()
