"""The C-ABI library loads and exports what include/novaphy_pbf.h declares
(CPU: no compute calls)."""
import ctypes
import os

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(capi):
    lib = capi.load()
    declared = capi.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_defaults(capi):
    assert b"sm_103a" in capi.load().pbf_version()
    s = capi.default_settings()
    # PBFSettings defaults (include/novaphy/fluid/pbf_solver.h:14-27)
    assert s.rest_density == 1000.0 and s.solver_iterations == 4
    assert np.float32(s.kernel_radius) == np.float32(0.1)
    assert s.corr_n == 4 and s.use_domain_bounds == 0
    assert list(s.domain_lower) == [-10.0, 0.0, -10.0]
    assert s.hash_compat == 1 and s.exact_arithmetic == 1
    # extensions without a counterpart in the reference: off
    assert s.boundary_two_way == 0 and s.boundary_friction == 0.0


def test_settings_layout_matches_oracle():
    from novaphy_gb300.capi import Settings as S
    from oracle.oracle import Settings as O

    for (a, ta), (b, tb) in zip(O._fields_, S._fields_):
        assert a == b and ctypes.sizeof(ta) == ctypes.sizeof(tb)
        assert getattr(O, a).offset == getattr(S, a).offset


def test_invalid_arguments_are_rejected(capi):
    lib = capi.load()
    assert lib.pbf_default_settings(None) == capi.PBF_ERR_INVALID_ARG
    assert b"NULL" in lib.pbf_last_error()
    assert lib.pbf_scene_step(None, ctypes.c_float(0.01), 1) == capi.PBF_ERR_INVALID_ARG
    assert lib.pbf_scene_set_bodies(None, 0, None, None, None) == capi.PBF_ERR_INVALID_ARG
    assert lib.pbf_scene_set_body_velocities(None, 0, None, None) == capi.PBF_ERR_INVALID_ARG
    bad = capi.default_settings(kernel_radius=0.0)
    out = ctypes.c_void_p()
    rc = lib.pbf_scene_create(0, ctypes.byref(bad), 0, None, None, 1.0, ctypes.byref(out))
    assert rc == capi.PBF_ERR_INVALID_ARG


def test_no_device_is_reported_not_faked(capi):
    if capi.device_count() > 0:
        pytest.skip("a GPU is visible")
    s = capi.default_settings()
    x = np.zeros((4, 3), np.float32)
    with pytest.raises(capi.PbfError) as e:
        capi.Scene(s, x, mass=1.0)
    assert e.value.code == capi.PBF_ERR_NO_DEVICE


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof/offsetof of the C ABI structs, from gcc on include/novaphy_pbf.h."""
    import shutil
    import subprocess

    from novaphy_gb300 import capi as c

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"pbf_settings": c.Settings, "pbf_server_config": c.ServerConfig,
               "pbf_server_stats": c.ServerStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "novaphy_pbf.h"',
             "int main(void) {"]
    for name, py in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run(
        [str(exe)], check=True, capture_output=True, text=True).stdout.splitlines())
    for name, py in structs.items():
        assert int(out[name]) == ctypes.sizeof(py), name
        for f, _ in py._fields_:
            assert int(out[f"{name}.{f}"]) == getattr(py, f).offset, (name, f)


def test_server_defaults_and_no_device(capi):
    cfg = capi.server_config()
    assert cfg.hbm_budget_bytes == 120 << 30 and cfg.max_inflight == 2
    assert capi.state_bytes_per_particle() == 52
    if capi.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(capi.PbfError) as e:
        capi.Server(cfg)
    assert e.value.code == capi.PBF_ERR_NO_DEVICE


def test_device_array_interface_layout(capi):
    # No device needed: the exported layout of positions (float4 rows) and
    # of a scalar field.
    v = capi.DeviceArray(object(), capi.FIELD_POSITIONS, 0x1000, 5)
    cai = v.__cuda_array_interface__
    assert cai["shape"] == (5, 3) and cai["strides"] == (16, 4) and cai["typestr"] == "<f4"
    assert cai["data"] == (0x1000, False) and cai["version"] == 3
    d = capi.DeviceArray(object(), capi.FIELD_LAMBDAS, 0x2000, 7).__cuda_array_interface__
    assert d["shape"] == (7,) and d["strides"] == (4,)
    assert capi.DeviceArray(object(), capi.FIELD_DENSITIES, 0x3000, 0).ptr == 0
    with pytest.raises(ValueError):
        capi.DeviceArray(object(), 9, 0x1000, 1)
