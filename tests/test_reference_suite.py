"""The reference's own Python tests (tests/python in the NovaPhy tree), run
unmodified against this package under the name ``novaphy``, on CPU where the
reference tree is present.

Selected: every test of the fluid, coupling, PBF, performance-monitor,
collision, free-body, math and performance-demo files that needs no CUDA device (this package
steps fluid only on the GPU; those tests run in the GPU suite instead), less
the math file's three tests of the articulated solver's spatial algebra.  The run
writes nothing into the reference tree: no byte-code, no cache, and its
temporary files go to pytest's own tmp directory.
"""
import os
import subprocess
import sys

import pytest

from oracle import build_oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Tests that need a CUDA device (they build or step a PBFSolver/FluidWorld).
NEEDS_DEVICE = [
    "test_fluid_world_boundary_particles", "test_coupled_simulation_runs",
    "test_coupling_sphere_in_fluid", "test_fluid_world_no_coupling_backward_compat",
    "test_pbf_solver_step_runs", "test_pbf_particles_fall", "test_pbf_zero_gravity",
    "test_pbf_density_reasonable", "test_pbf_velocities_updated", "test_fluid_world_creation",
    "test_fluid_world_step", "test_fluid_world_inherits_world",
    "test_fluid_world_monitor_reports_rigid_and_fluid_phases",
    "test_performance_demo_fluid_outputs",
]
# Spatial (6D) algebra of the articulated-body solver, which is not part of
# this package.
SPATIAL = ["test_spatial_transform_identity", "test_spatial_cross_motion",
           "test_spatial_inertia_matrix"]
FILES = ["test_fluid.py", "test_coupling.py", "test_pbf.py", "test_performance_monitor.py",
         "test_collision.py", "test_free_body_sim.py", "test_math.py",
         "test_demo_performance_monitor.py"]

RUNNER = r"""
import sys
sys.path.insert(0, sys.argv[1])
import novaphy_gb300
sys.modules["novaphy"] = novaphy_gb300
import pytest
sys.exit(pytest.main(sys.argv[2:]))
"""


def test_reference_python_suite_passes(tmp_path):
    tests_dir = os.path.join(build_oracle.REFERENCE_ROOT, "tests", "python")
    if not os.path.isdir(tests_dir):
        pytest.skip("reference tests not present on this host")
    deselect = " or ".join(NEEDS_DEVICE + SPATIAL)
    args = [os.path.join(tests_dir, f) for f in FILES] + [
        "-q", "-p", "no:cacheprovider", "--rootdir", str(tmp_path), "--basetemp",
        str(tmp_path / "base"), "-k", f"not ({deselect})", "-rf"]
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", RUNNER, ROOT, *args], cwd=str(tmp_path), env=env,
                       capture_output=True, text=True, timeout=600)
    tail = "\n".join(r.stdout.splitlines()[-15:])
    assert r.returncode == 0, tail
    assert " passed" in tail and "failed" not in tail, tail
