"""The C ABI library loads and exports every entry point include/gbl.h declares.

No compute call is made here; on a machine without a GPU the factory must refuse
with the runtime error the reference's CUDA stub raises
(src/fastlattice/CudaLatticeUnavailable.cpp:19-25).
"""
import os
import re

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbl.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gbl_[a-z_0-9]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_backend_api():
    names = declared_functions()
    for required in ("gbl_create", "gbl_upload", "gbl_set_external_forces", "gbl_run", "gbl_download",
                     "gbl_status", "gbl_first_failure_bonds", "gbl_destroy", "gbl_available", "gbl_description",
                     "gbl_multiprocessor_count", "gbl_build_schedule", "gbl_build_state", "gbl_last_error"):
        assert required in names


def test_every_declared_symbol_is_exported(gbl):
    lib = gbl.library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert missing == []


def test_bounds_checked_build_exports_the_same_symbols(gbl):
    import ctypes

    from banjo_gb300 import build

    checked = ctypes.CDLL(build.LIB_CHECKED)
    missing = [n for n in declared_functions() if not hasattr(checked, n)]
    assert missing == []


def test_normal_build_reports_unchecked(gbl):
    # No CUDA call: the normal build has no record to read.
    assert gbl.bounds_report() == {"checked": False, "violations": 0, "site": 0, "index": 0, "length": 0}


def test_struct_layouts_match_binding(gbl):
    lib = gbl.library()
    import ctypes

    for name, cls in [("gbl_step_settings", gbl.StepSettings), ("gbl_run_status", gbl.RunStatus),
                      ("gbl_state_view", gbl.StateView), ("gbl_schedule_view", gbl.ScheduleView),
                      ("gbl_run_control", gbl.RunControlC), ("gbl_sphere", gbl.Sphere),
                      ("gbl_matter_view", gbl.MatterView)]:
        assert lib.gbl_struct_size(name.encode()) == ctypes.sizeof(cls)
    assert lib.gbl_struct_size(b"no_such_struct") == 0


def test_factory_without_device_raises_runtime_error(gbl):
    if gbl.available():
        pytest.skip("a CUDA device is present")
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=4, ny=2, nz=2, steps=1)
    s = gbl.build_lattice_schedule(case["node_count"][0], case["bond_a"], case["bond_b"], case["node_block_begin"])
    with pytest.raises(RuntimeError, match="no CUDA device"):
        gbl.make_gb300_lattice_backend(s)
    assert gbl.multiprocessor_count() == 0
    assert "no CUDA device" in gbl.description()


def test_null_arguments_are_invalid(gbl):
    lib = gbl.library()
    assert lib.gbl_create(None, 0, 0, None) == 1
    assert lib.gbl_upload(None, None, None, None) == 1
    assert lib.gbl_run(None, None, None) == 1
