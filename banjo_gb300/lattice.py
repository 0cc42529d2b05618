"""Python mirror of the reference's lattice step API over the C ABI (include/gbl.h).

Names follow src/fastlattice/FastLattice.hpp: build_lattice_schedule
(buildLatticeSchedule), build_lattice_state (buildLatticeState),
make_gb300_lattice_backend (the makeCudaLatticeBackend factory this library
replaces) returning a backend with upload / set_external_forces / run /
download / status / first_failure_bonds / take_frames. Errors raise the
Python image of the reference's exception types: ValueError for
std::invalid_argument, RuntimeError for std::runtime_error, OverflowError for
std::overflow_error.

The library is the product; there is no fallback. If libgbl.so cannot be
loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
# GBL_LIBRARY=checked loads the bounds-checked build of the same library
# (every data-driven index checked on the device, violations recorded).
LIB_PATH = os.path.join(HERE, "_build",
                        "libgbl_checked.so" if os.environ.get("GBL_LIBRARY") == "checked" else "libgbl.so")

u8p, u32p, f64p, f32p = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.POINTER(C.c_float)
NO_BOND = 0xFFFFFFFF
INF_F = float("inf")


class ScheduleView(C.Structure):
    _fields_ = [("node_count", C.c_uint32), ("bond_count", C.c_uint32), ("block_count", C.c_uint32),
                ("color_count", C.c_uint32), ("boundary_bond_count", C.c_uint32),
                ("node_block_begin", u32p), ("bond_order", u32p), ("bond_schedule_index", u32p),
                ("bond_block_begin", u32p), ("range_begin", u32p), ("range_end", u32p), ("bond_color", u8p)]


_STATE_ARRAYS = [("x0", f64p), ("u", f64p), ("u_prev", f64p), ("v", f64p), ("inv_mass", f64p), ("mass", f64p),
                 ("adj_offsets", u32p), ("adj_bonds", u32p), ("nbr_bond", u32p), ("nbr_other", u32p),
                 ("nbr_rest", f64p), ("nbr_weight", f64p), ("nbr_alive", u8p), ("bond_slot_a", u32p),
                 ("bond_slot_b", u32p), ("bond_a", u32p), ("bond_b", u32p), ("rest_edge", f64p),
                 ("rest_length", f64p), ("rest_length_sq_minus", f64p), ("weight", f64p), ("compliance", f64p),
                 ("threshold", f64p), ("alive", u8p), ("failure_mode", u8p), ("damage", f64p),
                 ("prev_tensile", f64p), ("prev_compressive", f64p), ("prev_shear", f64p),
                 ("plastic_extension", f64p), ("plastic_strain", f64p)]


class StateView(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("node_count", C.c_uint32), ("bond_count", C.c_uint32),
                ("max_degree", C.c_uint32)] + _STATE_ARRAYS


class MatterView(C.Structure):
    _fields_ = [("node_count", C.c_uint32), ("bond_count", C.c_uint32), ("reference_position", f64p),
                ("position", f64p), ("velocity", f64p), ("mass", f64p), ("bond_a", u32p), ("bond_b", u32p),
                ("rest_length", f64p), ("compliance", f64p), ("threshold", f64p), ("alive", u8p),
                ("damage", f64p), ("failure_mode", u8p)]


class Footprint(C.Structure):
    _fields_ = [("center_t", C.c_double), ("center_b", C.c_double), ("half_t", C.c_double), ("half_b", C.c_double)]


class SupportPlane(C.Structure):
    _fields_ = [("point", C.c_double * 3), ("normal", C.c_double * 3), ("tangent", C.c_double * 3),
                ("bitangent", C.c_double * 3), ("restitution", C.c_double), ("static_friction", C.c_double),
                ("dynamic_friction", C.c_double), ("node_radius", C.c_double), ("reach_capped", C.c_uint8),
                ("footprint_count", C.c_uint32), ("footprints", Footprint * 4)]


class ContactSettings(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("static_friction", "dynamic_friction", "restitution",
                                          "restitution_speed_threshold", "node_contact_radius", "contact_margin",
                                          "prefilter_slack")]


class NodeContactSettings(C.Structure):
    _fields_ = [("mode", C.c_uint8)] + [(n, C.c_double) for n in (
        "radius", "skin", "margin", "restitution", "restitution_speed_threshold", "static_friction",
        "dynamic_friction")] + [("bucket_mask", C.c_uint32)]


class StepSettings(C.Structure):
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double * 3), ("constraint_iterations", C.c_uint32),
                ("bond_integrator", C.c_uint8), ("damping_fraction", C.c_double), ("sphere_enabled", C.c_uint8),
                ("direct_arithmetic", C.c_uint8), ("audit_energy", C.c_uint8),
                ("plastic_yield_stretch", C.c_double), ("plastic_hardening", C.c_double),
                ("plate_half_thickness", C.c_double), ("contact", ContactSettings),
                ("node_contact", NodeContactSettings), ("plane_count", C.c_uint32), ("planes", SupportPlane * 2)]


class Sphere(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("velocity", C.c_double * 3), ("angular_velocity", C.c_double * 3),
                ("radius", C.c_double), ("mass", C.c_double), ("inertia", C.c_double)]


class RunControlC(C.Structure):
    _fields_ = [("max_steps", C.c_uint64), ("quiet_steps", C.c_uint64), ("min_steps", C.c_uint64),
                ("no_failure_steps", C.c_uint64), ("energy_flat_steps", C.c_uint64),
                ("energy_flat_fraction", C.c_double), ("calm_steps", C.c_uint64),
                ("calm_damage_margin", C.c_double), ("removable_energy_j", C.c_double),
                ("capture_stride", C.c_uint64), ("max_frames", C.c_uint32), ("steps_per_launch", C.c_uint64),
                ("abandon", C.c_void_p)]


class ContactAccumulators(C.Structure):
    _fields_ = [("impulse_contacts", C.c_ulonglong), ("impulse_to_material_x", C.c_double),
                ("impulse_to_material_y", C.c_double), ("impulse_to_material_z", C.c_double),
                ("dissipated_kinetic_energy_j", C.c_double), ("maximum_penetration_m", C.c_double),
                ("maximum_position_correction_m", C.c_double), ("maximum_center_shift_m", C.c_double),
                ("candidate_overflow", C.c_ulonglong), ("ball_support_events", C.c_ulonglong)]


class LoadLedger(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("elapsed_s", C.c_double), ("requested_impulse_n_s", C.c_double * 3),
                ("impulse_n_s", C.c_double * 3), ("requested_angular_impulse_kg_m2_s", C.c_double * 3),
                ("angular_impulse_kg_m2_s", C.c_double * 3), ("work_j", C.c_double)]


class ExternalWrench(C.Structure):
    _fields_ = [("source", C.c_char_p), ("nodes", C.POINTER(C.c_uint32)), ("node_count", C.c_uint64),
                ("point_world_m", C.c_double * 3), ("force_n", C.c_double * 3), ("torque_n_m", C.c_double * 3)]


def case_wrenches(case: dict) -> list:
    """The wrenches a case carries (scenes.wrenches): (source, nodes, point,
    force, torque) tuples in the caller's order."""
    names = bytes(case["wrench_names"]).split(b"\0")
    counts = case["wrench_node_count"]
    nodes = case["wrench_nodes"]
    vec = case["wrench_vectors"].reshape(-1, 9)
    out, at = [], 0
    for k, n in enumerate(counts):
        out.append((names[k].decode(), nodes[at:at + int(n)], vec[k, 0:3], vec[k, 3:6], vec[k, 6:9]))
        at += int(n)
    return out


def ledger_row(g: LoadLedger) -> list:
    """A load ledger as the case files pack a source's (oracle/case_layout.hpp)."""
    return ([float(g.steps), g.elapsed_s] + list(g.requested_impulse_n_s) + list(g.impulse_n_s) +
            list(g.requested_angular_impulse_kg_m2_s) + list(g.angular_impulse_kg_m2_s) + [g.work_j])


def _wrench_array(wrenches):
    """The C array of (source, nodes, point, force, torque) tuples, and the
    buffers it points into (kept alive by the caller for the call)."""
    keep = []
    arr = (ExternalWrench * max(1, len(wrenches)))()
    for k, (source, nodes, point, force, torque) in enumerate(wrenches):
        idx = np.ascontiguousarray(nodes, dtype=np.uint32)
        name = source.encode() if isinstance(source, str) else source
        keep += [idx, name]
        arr[k].source = name
        arr[k].nodes = idx.ctypes.data_as(C.POINTER(C.c_uint32))
        arr[k].node_count = idx.size
        arr[k].point_world_m[:] = [float(x) for x in point]
        arr[k].force_n[:] = [float(x) for x in force]
        arr[k].torque_n_m[:] = [float(x) for x in torque]
    return arr, keep


def _source(fn, *lead):
    """One (source, LoadLedger) through a gbl_*external_source entry point."""
    length = C.c_size_t()
    _call(fn, *lead, None, 0, C.byref(length), None)
    buf = C.create_string_buffer(length.value + 1)
    g = LoadLedger()
    _call(fn, *lead, buf, len(buf), C.byref(length), C.byref(g))
    return buf.value.decode(), g


def source_arrays(sources: list) -> dict:
    """Source ledgers packed as the case files pack them (empty: no keys)."""
    if not sources:
        return {}
    return {"source_names": np.frombuffer(b"".join(n.encode() + b"\0" for n, _ in sources), dtype=np.uint8).copy(),
            "source_ledgers": np.asarray([ledger_row(g) for _, g in sources], dtype=np.float64).reshape(-1)}


class BoxSpec(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("horizon", C.c_uint32),
                ("max_offset_sq", C.c_uint32), ("slabs", C.c_uint32), ("spacing", C.c_double),
                ("center", C.c_double * 3), ("node_mass", C.c_double), ("compliance", C.c_double),
                ("threshold", C.c_double * 6)]


class Tuning(C.Structure):
    """gbl_tuning: a batch's launch shapes (results never depend on them)."""
    _fields_ = [("sweep_threads", C.c_uint32), ("whole_max_bonds", C.c_uint32), ("group_bytes", C.c_uint64),
                ("sweep_ms", C.c_double), ("default_ms", C.c_double), ("candidates", C.c_uint32),
                ("staged_max_nodes", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ContactPair(C.Structure):
    _fields_ = [("static_friction", C.c_double), ("dynamic_friction", C.c_double), ("restitution", C.c_double)]


class Ledge(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("dimensions", C.c_double * 3)]


class ImpactScene(C.Structure):
    """gbl_impact_scene: what the impact scene's step settings are built from."""
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double * 3), ("constraint_iterations", C.c_uint32),
                ("bond_damping", C.c_double), ("multi_body", C.c_uint8), ("double_precision", C.c_uint8),
                ("audit_energy", C.c_uint8), ("ball_tile", ContactPair), ("tile_tile", ContactPair),
                ("tile_ground", ContactPair), ("cell_size", C.c_double), ("node_contact_radius_factor", C.c_double),
                ("node_contact_skin_factor", C.c_double), ("node_contact_mode", C.c_uint8),
                ("ball_radius", C.c_double), ("yield_stretch", C.c_double), ("plastic_hardening_ratio", C.c_double),
                ("bridge", C.c_uint8), ("ground_y", C.c_double), ("support_y", C.c_double),
                ("ledge_count", C.c_uint32), ("ledges", Ledge * 4), ("origin", C.c_double * 3),
                ("node_count", C.c_uint32)]


class RequestInfo(C.Structure):
    _fields_ = [("phase", C.c_int32), ("slot", C.c_uint32), ("substeps", C.c_uint64), ("substeps_done", C.c_uint64),
                ("device_bytes", C.c_uint64), ("submitted_s", C.c_double), ("admitted_s", C.c_double),
                ("finished_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_uint64), ("running", C.c_uint64), ("done", C.c_uint64), ("bytes_in_use", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("substeps_run", C.c_uint64), ("device_seconds", C.c_double),
                ("clock_s", C.c_double), ("admit_seconds", C.c_double), ("retire_seconds", C.c_double),
                ("run_seconds", C.c_double)]


REQUEST_QUEUED, REQUEST_RUNNING, REQUEST_DONE = 0, 1, 2


class NodeContactAccumulators(C.Structure):
    _fields_ = [(n, C.c_ulonglong) for n in ("contacts", "pair_tests", "rebuilds", "pairs_listed", "pair_overflow")] + \
        [(n, C.c_double) for n in ("dissipated_kinetic_energy_j", "maximum_overlap_m", "maximum_position_correction_m",
                                   "momentum_residual_x", "momentum_residual_y", "momentum_residual_z")]


class RunStatus(C.Structure):
    _fields_ = [("total_steps", C.c_uint64), ("first_failure_step", C.c_uint64), ("last_failure_step", C.c_uint64),
                ("failure_rounds", C.c_uint32), ("broken_bonds", C.c_uint32), ("removed_energy_j", C.c_double),
                ("last_energy_gain_step", C.c_uint64), ("max_damage", C.c_double),
                ("last_damage_gain_step", C.c_uint64), ("contact", ContactAccumulators),
                ("external_load", LoadLedger), ("exit_reason", C.c_uint), ("launches", C.c_uint),
                ("kernel_seconds", C.c_double), ("wall_seconds", C.c_double), ("frames_captured", C.c_uint32),
                ("phase_seconds", C.c_double * 16), ("max_tensile_stretch", C.c_float),
                ("max_compressive_strain", C.c_float), ("max_shear_strain", C.c_float),
                ("rank_deficient_nodes", C.c_uint32), ("plastic_work_j", C.c_double),
                ("max_plastic_stretch", C.c_float), ("node_contact", NodeContactAccumulators),
                ("damping_dissipated_j", C.c_double), ("striker_dissipated_j", C.c_double),
                ("energy_audited", C.c_uint8), ("bond_projections", C.c_uint64)]


PHASE_NAMES = ["capture", "start_sample_nodes", "start_sample_bonds", "kick_classify", "contact_pass_1",
               "sweep_interior", "sweep_boundary", "support_project", "velocity_update", "damping",
               "contact_pass_2", "end_sample_nodes", "end_sample_bonds", "sphere_exit", "node_contact_broad",
               "node_contact_narrow"]

_lib = None


def library() -> C.CDLL:
    """The loaded libgbl.so; raises if it is missing (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"lattice library not built: {LIB_PATH} (run banjo_gb300.build.build())")
    lib = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    sigs = {
        "gbl_available": ([], C.c_int), "gbl_description": ([C.c_char_p, C.c_size_t], C.c_int),
        "gbl_multiprocessor_count": ([], C.c_uint), "gbl_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
        "gbl_struct_size": ([C.c_char_p], C.c_size_t),
        "gbl_create": ([C.POINTER(ScheduleView), C.c_int, C.c_uint, C.POINTER(vp)], C.c_int),
        "gbl_destroy": ([vp], None), "gbl_name": ([vp, C.c_char_p, C.c_size_t], C.c_int),
        "gbl_upload": ([vp, C.POINTER(StateView), C.POINTER(StepSettings), C.POINTER(Sphere)], C.c_int),
        "gbl_set_external_forces": ([vp, f64p, C.c_uint64, C.c_uint64], C.c_int),
        "gbl_set_external_wrenches": ([vp, C.POINTER(ExternalWrench), C.c_uint64, C.c_uint64], C.c_int),
        "gbl_external_source_count": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_external_source": ([vp, C.c_uint64, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t),
                                 C.POINTER(LoadLedger)], C.c_int),
        "gbl_run": ([vp, C.POINTER(RunControlC), C.POINTER(RunStatus)], C.c_int),
        "gbl_status": ([vp, C.POINTER(RunStatus)], C.c_int),
        "gbl_download": ([vp, C.POINTER(StateView), C.POINTER(Sphere)], C.c_int),
        "gbl_first_failure_bonds": ([vp, u32p, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_frame_count": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_take_frame": ([vp, C.c_uint64, C.POINTER(C.c_uint64), f32p, u8p, f32p, C.POINTER(Sphere)], C.c_int),
        "gbl_clear_frames": ([vp], C.c_int), "gbl_set_stream": ([vp, vp], C.c_int),
        "gbl_profile_phases": ([vp, C.c_uint64, f64p], C.c_int),
        "gbl_bounds_report": ([C.POINTER(C.c_uint64), C.POINTER(C.c_int)], C.c_int),
        "gbl_bounds_clear": ([], C.c_int),
        "gbl_serve_set_lane_threshold": ([vp, C.c_uint32], C.c_int),
        "gbl_debug_substep": ([vp, C.c_uint32, C.POINTER(StateView), C.POINTER(Sphere)], C.c_int),
        "gbl_kernels_per_substep": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_build_schedule": ([C.c_uint32, C.c_uint32, u32p, u32p, u32p, C.c_uint32, C.POINTER(vp)], C.c_int),
        "gbl_schedule_view_of": ([vp, C.POINTER(ScheduleView)], C.c_int), "gbl_schedule_free": ([vp], None),
        "gbl_build_state": ([C.POINTER(MatterView), vp, f64p, C.POINTER(vp)], C.c_int),
        "gbl_state_view_of": ([vp, C.POINTER(StateView)], C.c_int), "gbl_state_pin": ([vp, u8p], C.c_int),
        "gbl_state_free": ([vp], None),
        "gbl_batch_create": ([C.c_int, C.POINTER(vp)], C.c_int), "gbl_batch_destroy": ([vp], None),
        "gbl_batch_add": ([vp, C.POINTER(ScheduleView), C.POINTER(StateView), C.POINTER(Sphere),
                           C.POINTER(C.c_uint32)], C.c_int),
        "gbl_batch_settle": ([vp, C.POINTER(StepSettings)], C.c_int),
        "gbl_batch_set_external_forces": ([vp, C.c_uint32, f64p, C.c_uint64, C.c_uint64], C.c_int),
        "gbl_batch_run": ([vp, C.POINTER(RunControlC)], C.c_int),
        "gbl_batch_set_external_wrenches": ([vp, C.c_uint32, C.POINTER(ExternalWrench), C.c_uint64, C.c_uint64],
                                            C.c_int),
        "gbl_batch_external_source_count": ([vp, C.c_uint32, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_batch_external_source": ([vp, C.c_uint32, C.c_uint64, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t),
                                       C.POINTER(LoadLedger)], C.c_int),
        "gbl_batch_size": ([vp, C.POINTER(C.c_uint32)], C.c_int),
        "gbl_batch_status": ([vp, C.c_uint32, C.POINTER(RunStatus)], C.c_int),
        "gbl_batch_download": ([vp, C.c_uint32, C.POINTER(StateView), C.POINTER(Sphere)], C.c_int),
        "gbl_batch_first_failure_bonds": ([vp, C.c_uint32, u32p, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_batch_profile_phases": ([vp, C.c_uint64, f64p], C.c_int),
        "gbl_batch_tune": ([vp, C.POINTER(Tuning)], C.c_int),
        "gbl_impact_settings": ([C.POINTER(ImpactScene), C.POINTER(StepSettings)], C.c_int),
        "gbl_batch_set_tuning": ([vp, C.POINTER(Tuning)], C.c_int),
        "gbl_batch_kernels_per_substep": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "gbl_batch_set_stream": ([vp, vp], C.c_int),
        "gbl_build_box": ([C.POINTER(BoxSpec), C.POINTER(vp)], C.c_int),
        "gbl_box_view_of": ([vp, C.POINTER(MatterView), C.POINTER(u32p), C.POINTER(C.c_uint32)], C.c_int),
        "gbl_box_free": ([vp], None),
        "gbl_serve_create": ([C.c_int, C.POINTER(StepSettings), C.c_uint64, C.POINTER(vp)], C.c_int),
        "gbl_serve_destroy": ([vp], None),
        "gbl_serve_submit": ([vp, C.POINTER(ScheduleView), C.POINTER(StateView), C.POINTER(Sphere), C.c_uint64,
                              C.POINTER(C.c_uint64)], C.c_int),
        "gbl_serve_submit_borrowed": ([vp, C.POINTER(ScheduleView), C.POINTER(StateView), C.POINTER(Sphere), C.c_uint64,
                              C.POINTER(C.c_uint64)], C.c_int),
        "gbl_serve_step": ([vp, C.c_uint64, C.POINTER(ServerStats)], C.c_int),
        "gbl_serve_poll": ([vp, C.c_uint64, C.POINTER(RequestInfo)], C.c_int),
        "gbl_serve_take": ([vp, C.c_uint64, C.POINTER(StateView), C.POINTER(Sphere), C.POINTER(RunStatus)], C.c_int),
        "gbl_serve_cancel": ([vp, C.c_uint64], C.c_int),
        "gbl_serve_stats": ([vp, C.POINTER(ServerStats)], C.c_int),
        "gbl_serve_footprint": ([C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64)],
                                C.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    for name, cls in [("gbl_schedule_view", ScheduleView), ("gbl_state_view", StateView),
                      ("gbl_matter_view", MatterView), ("gbl_support_plane", SupportPlane),
                      ("gbl_step_settings", StepSettings), ("gbl_sphere", Sphere),
                      ("gbl_run_control", RunControlC), ("gbl_run_status", RunStatus),
                      ("gbl_request_info", RequestInfo), ("gbl_server_stats", ServerStats),
                      ("gbl_box_spec", BoxSpec), ("gbl_node_contact_accumulators", NodeContactAccumulators),
                      ("gbl_tuning", Tuning), ("gbl_impact_scene", ImpactScene),
                      ("gbl_external_wrench", ExternalWrench), ("gbl_load_ledger", LoadLedger)]:
        if lib.gbl_struct_size(name.encode()) != C.sizeof(cls):
            raise RuntimeError(f"binding layout of {name} does not match libgbl.so")
    _lib = lib
    return lib


def _error(rc: int):
    buf = C.create_string_buffer(1024)
    library().gbl_last_error(buf, len(buf))
    msg = buf.value.decode()
    if rc == 1:
        return ValueError(msg)
    if rc == 3:
        return OverflowError(msg)
    return RuntimeError(msg)


def _call(fn, *args):
    rc = fn(*args)
    if rc != 0:
        raise _error(rc)


def _ptr(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype)) if arr is not None else None


def available() -> bool:
    return bool(library().gbl_available())


def description() -> str:
    buf = C.create_string_buffer(512)
    _call(library().gbl_description, buf, len(buf))
    return buf.value.decode()


def multiprocessor_count() -> int:
    return int(library().gbl_multiprocessor_count())


def bounds_report() -> dict:
    """The bounds-checked build's record: whether this library checks, the
    violations since the last clear, and the first one's site, index and
    length (all zero in the normal build)."""
    rep = (C.c_uint64 * 4)()
    checked = C.c_int()
    _call(library().gbl_bounds_report, rep, C.byref(checked))
    return {"checked": bool(checked.value), "violations": int(rep[0]), "site": int(rep[1]), "index": int(rep[2]),
            "length": int(rep[3])}


def bounds_clear() -> None:
    _call(library().gbl_bounds_clear)


class Schedule:
    """A LatticeSchedule built by the library (buildLatticeSchedule)."""

    def __init__(self, handle):
        self._h = handle
        self.view = ScheduleView()
        _call(library().gbl_schedule_view_of, handle, C.byref(self.view))

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_schedule_free(self._h)
            self._h = None

    def _arr(self, name, count, dtype):
        p = getattr(self.view, name)
        return np.ctypeslib.as_array(p, shape=(count,)).astype(dtype, copy=True) if count else np.zeros(0, dtype)

    @property
    def block_count(self):
        return self.view.block_count

    @property
    def color_count(self):
        return self.view.color_count

    @property
    def boundary_bond_count(self):
        return self.view.boundary_bond_count

    def arrays(self) -> dict:
        v = self.view
        ranges = v.block_count * 2 * max(v.color_count, 1)
        return {
            "sched_bond_order": self._arr("bond_order", v.bond_count, np.uint32),
            "sched_color": self._arr("bond_color", v.bond_count, np.uint8),
            "sched_range_begin": self._arr("range_begin", ranges, np.uint32),
            "sched_range_end": self._arr("range_end", ranges, np.uint32),
            "sched_bond_block_begin": self._arr("bond_block_begin", v.block_count + 1, np.uint32),
            "sched_color_count": np.array([v.color_count], np.uint32),
            "sched_boundary_bond_count": np.array([v.boundary_bond_count], np.uint32),
        }


def build_lattice_schedule(node_count, bond_a, bond_b, node_block_begin) -> Schedule:
    a = np.ascontiguousarray(bond_a, dtype=np.uint32)
    b = np.ascontiguousarray(bond_b, dtype=np.uint32)
    blocks = np.ascontiguousarray(node_block_begin, dtype=np.uint32)
    h = C.c_void_p()
    _call(library().gbl_build_schedule, int(node_count), a.size, _ptr(a, C.c_uint32), _ptr(b, C.c_uint32),
          _ptr(blocks, C.c_uint32), blocks.size - 1, C.byref(h))
    return Schedule(h)


class State:
    """A LatticeState owned by the library (buildLatticeState); arrays are numpy views."""

    _SIZES = {"x0": 3, "u": 3, "u_prev": 3, "v": 3, "inv_mass": 1, "mass": 1}

    def __init__(self, handle):
        self._h = handle
        self.view = StateView()
        _call(library().gbl_state_view_of, handle, C.byref(self.view))
        v = self.view
        n, b, p = v.node_count, v.bond_count, v.node_count * v.max_degree
        counts = {"x0": 3 * n, "u": 3 * n, "u_prev": 3 * n, "v": 3 * n, "inv_mass": n, "mass": n,
                  "adj_offsets": n + 1, "adj_bonds": 2 * b, "nbr_bond": p, "nbr_other": p, "nbr_rest": 3 * p,
                  "nbr_weight": p, "nbr_alive": p, "bond_slot_a": b, "bond_slot_b": b, "bond_a": b, "bond_b": b,
                  "rest_edge": 3 * b, "rest_length": b, "rest_length_sq_minus": b, "weight": b,
                  "compliance": b, "threshold": 6 * b, "alive": b, "failure_mode": b, "damage": b,
                  "prev_tensile": b, "prev_compressive": b, "prev_shear": b, "plastic_extension": b,
                  "plastic_strain": b}
        self.arrays = {}
        dtypes = {f64p: np.float64, u32p: np.uint32, u8p: np.uint8}
        for name, ptype in _STATE_ARRAYS:
            cnt = counts[name]
            ptr = getattr(v, name)
            self.arrays[name] = np.ctypeslib.as_array(ptr, shape=(cnt,)) if cnt else np.zeros(0, dtype=dtypes[ptype])

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and name in arrays:
            return arrays[name]
        raise AttributeError(name)

    @property
    def node_count(self):
        return self.view.node_count

    @property
    def bond_count(self):
        return self.view.bond_count

    def pin(self, pinned) -> None:
        p = np.ascontiguousarray(pinned, dtype=np.uint8)
        _call(library().gbl_state_pin, self._h, _ptr(p, C.c_uint8))

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_state_free(self._h)
            self._h = None


def build_lattice_state(case: dict, schedule: Schedule) -> State:
    """buildLatticeState from a case's asset and matter arrays (asset bond order)."""
    n = int(case["node_count"][0])
    b = int(case["bond_count"][0])
    keep = {k: np.ascontiguousarray(case[k]) for k in ("ref_pos", "pos", "vel", "mass", "rest_length", "compliance",
                                                        "threshold")}
    keep["bond_a"] = np.ascontiguousarray(case["bond_a"], dtype=np.uint32)
    keep["bond_b"] = np.ascontiguousarray(case["bond_b"], dtype=np.uint32)
    alive = np.ascontiguousarray(case["alive"], dtype=np.uint8) if "alive" in case else None
    m = MatterView(n, b, _ptr(keep["ref_pos"], C.c_double), _ptr(keep["pos"], C.c_double),
                   _ptr(keep["vel"], C.c_double), _ptr(keep["mass"], C.c_double), _ptr(keep["bond_a"], C.c_uint32),
                   _ptr(keep["bond_b"], C.c_uint32), _ptr(keep["rest_length"], C.c_double),
                   _ptr(keep["compliance"], C.c_double), _ptr(keep["threshold"], C.c_double),
                   _ptr(alive, C.c_uint8) if alive is not None else None, None, None)
    origin = np.ascontiguousarray(case.get("origin", np.zeros(3)), dtype=np.float64)
    h = C.c_void_p()
    _call(library().gbl_build_state, C.byref(m), schedule._h, _ptr(origin, C.c_double), C.byref(h))
    st = State(h)
    if "pinned" in case:
        st.pin(case["pinned"])
    return st


class Box:
    """A box lattice built by the library (generateBoxTileLattice's walk,
    src/matter/BoxLattice.cpp:49-195, uniform bonds)."""

    def __init__(self, spec: BoxSpec):
        self._h = None
        h = C.c_void_p()
        _call(library().gbl_build_box, C.byref(spec), C.byref(h))
        self._h = h
        self.matter = MatterView()
        slabs = u32p()
        count = C.c_uint32()
        _call(library().gbl_box_view_of, self._h, C.byref(self.matter), C.byref(slabs), C.byref(count))
        self.node_count = int(self.matter.node_count)
        self.bond_count = int(self.matter.bond_count)
        self.node_block_begin = np.ctypeslib.as_array(slabs, shape=(count.value + 1,)).copy()

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_box_free(self._h)
            self._h = None

    def array(self, name: str) -> np.ndarray:
        """A copy of one matter array: ref_pos, pos, vel, mass, bond_a, bond_b, rest_length, compliance, threshold."""
        m = self.matter
        n, b = self.node_count, self.bond_count
        field, count = {"ref_pos": ("reference_position", 3 * n), "pos": ("position", 3 * n),
                        "vel": ("velocity", 3 * n), "mass": ("mass", n), "bond_a": ("bond_a", b),
                        "bond_b": ("bond_b", b), "rest_length": ("rest_length", b), "compliance": ("compliance", b),
                        "threshold": ("threshold", 6 * b)}[name]
        return np.ctypeslib.as_array(getattr(m, field), shape=(count,)).copy() if count else np.zeros(0)


def build_box(nx, ny, nz, spacing, center=(0.0, 0.0, 0.0), compliance=1e-7, threshold=(INF_F,) * 6,
              node_mass=1e-3, horizon=1, max_offset_sq=2, slabs=1) -> Box:
    spec = BoxSpec(nx, ny, nz, horizon, max_offset_sq, slabs, spacing, (C.c_double * 3)(*center), node_mass,
                   compliance, (C.c_double * 6)(*threshold))
    return Box(spec)


def box_schedule(box: Box) -> Schedule:
    h = C.c_void_p()
    blocks = box.node_block_begin.size - 1
    _call(library().gbl_build_schedule, box.node_count, box.bond_count, box.matter.bond_a, box.matter.bond_b,
          _ptr(box.node_block_begin, C.c_uint32), blocks, C.byref(h))
    return Schedule(h)


def box_state(box: Box, schedule: Schedule, origin=(0.0, 0.0, 0.0)) -> State:
    o = np.asarray(origin, dtype=np.float64)
    h = C.c_void_p()
    _call(library().gbl_build_state, C.byref(box.matter), schedule._h, _ptr(o, C.c_double), C.byref(h))
    return State(h)


def step_settings(packed: np.ndarray) -> StepSettings:
    """StepSettings<double> from the packed settings record (scenes.settings)."""
    s = StepSettings()
    s.dt = packed[scenes.K_DT]
    s.gravity[:] = packed[scenes.K_GRAVITY:scenes.K_GRAVITY + 3]
    s.constraint_iterations = int(packed[scenes.K_ITER])
    s.bond_integrator = 0
    s.damping_fraction = packed[scenes.K_DAMP]
    s.sphere_enabled = int(packed[scenes.K_SPHERE])
    s.direct_arithmetic = int(packed[scenes.K_DIRECT])
    s.audit_energy = int(packed[scenes.K_AUDIT]) if len(packed) > scenes.K_AUDIT else 0
    s.plastic_yield_stretch = packed[scenes.K_YIELD]
    s.plastic_hardening = packed[scenes.K_HARDEN]
    s.plate_half_thickness = packed[scenes.K_PLATE]
    c = packed[scenes.K_CONTACT:scenes.K_CONTACT + 7]
    s.contact = ContactSettings(*c)
    s.plane_count = int(packed[scenes.K_PLANE_COUNT])
    for p in range(2):
        q = packed[scenes.K_PLANES + scenes.PLANE_WIDTH * p: scenes.K_PLANES + scenes.PLANE_WIDTH * (p + 1)]
        pl = s.planes[p]
        pl.point[:], pl.normal[:], pl.tangent[:], pl.bitangent[:] = q[0:3], q[3:6], q[6:9], q[9:12]
        pl.restitution, pl.static_friction, pl.dynamic_friction, pl.node_radius = q[12], q[13], q[14], q[15]
        pl.reach_capped = int(q[16])
        pl.footprint_count = int(q[17])
        for f in range(4):
            pl.footprints[f] = Footprint(*q[18 + 4 * f: 22 + 4 * f])
    if len(packed) > scenes.K_NODE_CONTACT:
        n = packed[scenes.K_NODE_CONTACT:scenes.K_NODE_CONTACT + 9]
        s.node_contact = NodeContactSettings(int(n[0]), *n[1:8], int(n[8]))
    return s


def impact_settings(scene: ImpactScene) -> StepSettings:
    """The impact scene's StepSettings (buildSettings, TileImpactScene.cpp:259-336)."""
    out = StepSettings()
    _call(library().gbl_impact_settings, C.byref(scene), C.byref(out))
    return out


def sphere_state(packed: np.ndarray) -> Sphere:
    s = Sphere()
    s.center[:], s.velocity[:], s.angular_velocity[:] = packed[0:3], packed[3:6], packed[6:9]
    s.radius, s.mass, s.inertia = packed[9], packed[10], packed[11]
    return s


def pack_sphere(s: Sphere) -> np.ndarray:
    return np.array(list(s.center) + list(s.velocity) + list(s.angular_velocity) + [s.radius, s.mass, s.inertia])


@dataclasses.dataclass
class RunControl:
    """RunControl (FastLattice.hpp:79-128); exit rules are off at 0."""
    max_steps: int = 0
    quiet_steps: int = 0
    min_steps: int = 0
    no_failure_steps: int = 0
    energy_flat_steps: int = 0
    energy_flat_fraction: float = 1.0e-3
    calm_steps: int = 0
    calm_damage_margin: float = 0.5
    removable_energy_j: float = 0.0
    capture_stride: int = 0
    max_frames: int = 0
    steps_per_launch: int = 0
    abandon: object = None  # a numpy uint8 array of one element, or None

    def c(self) -> RunControlC:
        ab = self.abandon.ctypes.data if self.abandon is not None else None
        return RunControlC(self.max_steps, self.quiet_steps, self.min_steps, self.no_failure_steps,
                           self.energy_flat_steps, self.energy_flat_fraction, self.calm_steps,
                           self.calm_damage_margin, self.removable_energy_j, self.capture_stride, self.max_frames,
                           self.steps_per_launch, ab)


class Backend:
    """The GB300 LatticeBackend (FastLattice.hpp:255-369)."""

    def __init__(self, schedule: Schedule, precision: str = "float", threads_per_block: int = 0):
        self._h = None
        prec = 1 if precision == "double" else 0
        h = C.c_void_p()
        _call(library().gbl_create, C.byref(schedule.view), prec, threads_per_block, C.byref(h))
        self._h = h
        self.precision = precision
        self._node_count = 0
        self._bond_count = 0

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_destroy(self._h)
            self._h = None

    def name(self) -> str:
        buf = C.create_string_buffer(64)
        _call(library().gbl_name, self._h, buf, len(buf))
        return buf.value.decode()

    def upload(self, state: State, settings: StepSettings, sphere: Sphere) -> None:
        _call(library().gbl_upload, self._h, C.byref(state.view), C.byref(settings), C.byref(sphere))
        self._node_count = state.node_count
        self._bond_count = state.bond_count

    def set_external_forces(self, forces, substeps: int) -> None:
        if forces is None or len(forces) == 0:
            _call(library().gbl_set_external_forces, self._h, None, 0, int(substeps))
            return
        f = np.ascontiguousarray(forces, dtype=np.float64).reshape(-1)
        _call(library().gbl_set_external_forces, self._h, _ptr(f, C.c_double), f.size // 3, int(substeps))

    def set_external_wrenches(self, wrenches, substeps: int) -> None:
        """wrenches: (source, nodes, point, force, torque) tuples."""
        arr, keep = _wrench_array(wrenches)
        _call(library().gbl_set_external_wrenches, self._h, arr if wrenches else None, len(wrenches), int(substeps))
        del keep

    def external_sources(self) -> list:
        """RunStatus::external_sources: (source, LoadLedger) in status order."""
        n = C.c_uint64()
        _call(library().gbl_external_source_count, self._h, C.byref(n))
        return [_source(library().gbl_external_source, self._h, k) for k in range(n.value)]

    def run(self, control: RunControl) -> RunStatus:
        st = RunStatus()
        ctl = control.c()
        _call(library().gbl_run, self._h, C.byref(ctl), C.byref(st))
        return st

    def status(self) -> RunStatus:
        st = RunStatus()
        _call(library().gbl_status, self._h, C.byref(st))
        return st

    def download(self, state: State) -> Sphere:
        sp = Sphere()
        _call(library().gbl_download, self._h, C.byref(state.view), C.byref(sp))
        return sp

    def first_failure_bonds(self) -> np.ndarray:
        n = C.c_uint64()
        _call(library().gbl_first_failure_bonds, self._h, None, 0, C.byref(n))
        out = np.zeros(n.value, dtype=np.uint32)
        _call(library().gbl_first_failure_bonds, self._h, _ptr(out, C.c_uint32), n.value, C.byref(n))
        return out

    def take_frames(self) -> list:
        n = C.c_uint64()
        _call(library().gbl_frame_count, self._h, C.byref(n))
        frames = []
        for k in range(n.value):
            step = C.c_uint64()
            u = np.zeros(3 * self._node_count, dtype=np.float32)
            alive = np.zeros(self._bond_count, dtype=np.uint8)
            damage = np.zeros(self._bond_count, dtype=np.float32)
            sp = Sphere()
            _call(library().gbl_take_frame, self._h, k, C.byref(step), _ptr(u, C.c_float), _ptr(alive, C.c_uint8),
                  _ptr(damage, C.c_float), C.byref(sp))
            frames.append({"step": step.value, "u": u, "alive": alive, "damage": damage, "sphere": pack_sphere(sp)})
        _call(library().gbl_clear_frames, self._h)
        return frames

    def set_stream(self, stream_ptr: int | None) -> None:
        _call(library().gbl_set_stream, self._h, C.c_void_p(stream_ptr) if stream_ptr else None)

    def kernels_per_substep(self) -> int:
        n = C.c_uint64()
        _call(library().gbl_kernels_per_substep, self._h, C.byref(n))
        return int(n.value)

    def profile_phases(self, substeps: int) -> dict:
        out = np.zeros(16, dtype=np.float64)
        _call(library().gbl_profile_phases, self._h, int(substeps), _ptr(out, C.c_double))
        return {PHASE_NAMES[k]: float(out[k]) for k in range(16)}

    def debug_substep(self, phases, states) -> list:
        """The phase-diff mode (gbl_debug_substep): one substep, with the
        lattice's state downloaded into states[i] after phases[i] (ascending
        phase numbers); returns the spheres at those points."""
        phases = list(phases)
        if phases != sorted(set(phases)) or len(states) != len(phases):
            raise ValueError("phases ascending and distinct, one state each")
        mask = 0
        for ph in phases:
            mask |= 1 << int(ph)
        views = (StateView * len(states))(*[st.view for st in states])
        spheres = (Sphere * len(states))()
        _call(library().gbl_debug_substep, self._h, mask, views, spheres)
        return list(spheres)


def make_gb300_lattice_backend(schedule: Schedule, precision: str = "float", threads_per_block: int = 0) -> Backend:
    """The factory that replaces makeCudaLatticeBackend (FastLattice.hpp:401-402)."""
    return Backend(schedule, precision, threads_per_block)


class Batch:
    """Independent lattices stepped together on the device, sharing step
    settings; each lattice's results equal the same lattice run alone. Replaces
    the reference's one-backend-per-trial loop (TileImpactScene.cpp:345-351, 777)."""

    def __init__(self, precision: str = "float"):
        self._h = None
        h = C.c_void_p()
        _call(library().gbl_batch_create, 1 if precision == "double" else 0, C.byref(h))
        self._h = h
        self.precision = precision
        self._keep = []  # schedules stay alive while the batch refers to their lattices

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_batch_destroy(self._h)
            self._h = None

    def add(self, schedule: Schedule, state: State, sphere: Sphere) -> int:
        k = C.c_uint32()
        _call(library().gbl_batch_add, self._h, C.byref(schedule.view), C.byref(state.view), C.byref(sphere),
              C.byref(k))
        self._keep.append(schedule)
        return int(k.value)

    def settle(self, settings: StepSettings) -> None:
        _call(library().gbl_batch_settle, self._h, C.byref(settings))

    def __len__(self) -> int:
        n = C.c_uint32()
        _call(library().gbl_batch_size, self._h, C.byref(n))
        return int(n.value)

    def set_external_wrenches(self, index: int, wrenches, substeps: int) -> None:
        arr, keep = _wrench_array(wrenches)
        _call(library().gbl_batch_set_external_wrenches, self._h, index, arr if wrenches else None, len(wrenches),
              int(substeps))
        del keep

    def external_sources(self, index: int) -> list:
        n = C.c_uint64()
        _call(library().gbl_batch_external_source_count, self._h, index, C.byref(n))
        return [_source(library().gbl_batch_external_source, self._h, index, k) for k in range(n.value)]

    def set_external_forces(self, index: int, forces, substeps: int) -> None:
        if forces is None or len(forces) == 0:
            _call(library().gbl_batch_set_external_forces, self._h, index, None, 0, int(substeps))
            return
        f = np.ascontiguousarray(forces, dtype=np.float64).reshape(-1)
        _call(library().gbl_batch_set_external_forces, self._h, index, _ptr(f, C.c_double), f.size // 3,
              int(substeps))

    def run(self, control: RunControl) -> None:
        ctl = control.c()
        _call(library().gbl_batch_run, self._h, C.byref(ctl))

    def status(self, index: int) -> RunStatus:
        st = RunStatus()
        _call(library().gbl_batch_status, self._h, index, C.byref(st))
        return st

    def download(self, index: int, state: State) -> Sphere:
        sp = Sphere()
        _call(library().gbl_batch_download, self._h, index, C.byref(state.view), C.byref(sp))
        return sp

    def first_failure_bonds(self, index: int) -> np.ndarray:
        n = C.c_uint64()
        _call(library().gbl_batch_first_failure_bonds, self._h, index, None, 0, C.byref(n))
        out = np.zeros(n.value, dtype=np.uint32)
        _call(library().gbl_batch_first_failure_bonds, self._h, index, _ptr(out, C.c_uint32), n.value, C.byref(n))
        return out

    def set_stream(self, stream_ptr: int | None) -> None:
        _call(library().gbl_batch_set_stream, self._h, C.c_void_p(stream_ptr) if stream_ptr else None)

    def kernels_per_substep(self) -> int:
        n = C.c_uint64()
        _call(library().gbl_batch_kernels_per_substep, self._h, C.byref(n))
        return int(n.value)

    def profile_phases(self, substeps: int) -> dict:
        out = np.zeros(16, dtype=np.float64)
        _call(library().gbl_batch_profile_phases, self._h, int(substeps), _ptr(out, C.c_double))
        return {PHASE_NAMES[k]: float(out[k]) for k in range(16)}

    def tune(self) -> dict:
        """Times the sweep under candidate launch shapes, keeps the fastest
        (state unchanged); returns the kept shape and the timings."""
        t = Tuning()
        _call(library().gbl_batch_tune, self._h, C.byref(t))
        return t.as_dict()

    def set_tuning(self, sweep_threads: int = 0, whole_max_bonds: int = 0, group_bytes: int = 0,
                   staged_max_nodes: int = 0) -> None:
        """Launch shapes (0 keeps a value; staged_max_nodes 0xFFFFFFFF turns
        the shared-memory staged sweep off)."""
        t = Tuning(sweep_threads, whole_max_bonds, group_bytes, 0.0, 0.0, 0, staged_max_nodes)
        _call(library().gbl_batch_set_tuning, self._h, C.byref(t))


class Server:
    """Continuous batching of lattice requests under a device memory budget
    (the served form of the step; the reference has no counterpart)."""

    def __init__(self, settings: StepSettings, budget_bytes: int, precision: str = "float"):
        self._h = None
        h = C.c_void_p()
        _call(library().gbl_serve_create, 1 if precision == "double" else 0, C.byref(settings), int(budget_bytes),
              C.byref(h))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            library().gbl_serve_destroy(self._h)
            self._h = None

    def submit(self, schedule: Schedule, state: State, sphere: Sphere, substeps: int, borrow: bool = False) -> int:
        """Queues a request. With `borrow`, the state's arrays are read at
        admission instead of copied now: keep `state` alive and unchanged
        until the request is running (gbl_serve_submit_borrowed)."""
        t = C.c_uint64()
        fn = library().gbl_serve_submit_borrowed if borrow else library().gbl_serve_submit
        _call(fn, self._h, C.byref(schedule.view), C.byref(state.view), C.byref(sphere), int(substeps), C.byref(t))
        return int(t.value)

    def step(self, substeps: int) -> ServerStats:
        st = ServerStats()
        _call(library().gbl_serve_step, self._h, int(substeps), C.byref(st))
        return st

    def poll(self, ticket: int) -> RequestInfo:
        info = RequestInfo()
        _call(library().gbl_serve_poll, self._h, int(ticket), C.byref(info))
        return info

    def take(self, ticket: int, state: State | None) -> tuple:
        """The result into `state` (None: the state is dropped), with the sphere and RunStatus."""
        sp = Sphere()
        st = RunStatus()
        _call(library().gbl_serve_take, self._h, int(ticket), C.byref(state.view) if state is not None else None,
              C.byref(sp), C.byref(st))
        return sp, st

    def cancel(self, ticket: int) -> None:
        _call(library().gbl_serve_cancel, self._h, int(ticket))

    def stats(self) -> ServerStats:
        st = ServerStats()
        _call(library().gbl_serve_stats, self._h, C.byref(st))
        return st

    def set_lane_threshold(self, bonds: int) -> None:
        """Requests submitted from now on with at least `bonds` bonds run in
        the large lane (gbl_serve_set_lane_threshold)."""
        _call(library().gbl_serve_set_lane_threshold, self._h, int(bonds))


def footprint(node_count: int, bond_count: int, max_degree: int, block_count: int, precision: str = "float") -> int:
    n = C.c_uint64()
    _call(library().gbl_serve_footprint, 1 if precision == "double" else 0, node_count, bond_count, max_degree,
          block_count, C.byref(n))
    return int(n.value)


def status_arrays(st: RunStatus) -> dict:
    """RunStatus packed as the case files pack it (oracle/case_layout.hpp)."""
    nc = st.node_contact
    u = np.zeros(19, dtype=np.uint64)
    u[:] = [st.total_steps, st.first_failure_step, st.last_failure_step, st.failure_rounds, st.broken_bonds,
            st.last_energy_gain_step, st.last_damage_gain_step, st.exit_reason, st.rank_deficient_nodes,
            st.contact.impulse_contacts, st.contact.candidate_overflow, st.contact.ball_support_events, st.launches,
            nc.contacts, nc.pair_tests, nc.rebuilds, nc.pairs_listed, nc.pair_overflow, st.energy_audited]
    d = np.zeros(28, dtype=np.float64)
    d[:] = [st.removed_energy_j, st.max_damage, st.plastic_work_j, st.max_tensile_stretch,
            st.max_compressive_strain, st.max_shear_strain, st.max_plastic_stretch,
            st.contact.impulse_to_material_x, st.contact.impulse_to_material_y, st.contact.impulse_to_material_z,
            st.contact.dissipated_kinetic_energy_j, st.contact.maximum_penetration_m,
            st.contact.maximum_position_correction_m, st.contact.maximum_center_shift_m, st.external_load.work_j,
            st.external_load.impulse_n_s[0], st.external_load.impulse_n_s[1], st.external_load.impulse_n_s[2],
            float(st.external_load.steps), st.wall_seconds, nc.dissipated_kinetic_energy_j, nc.maximum_overlap_m,
            nc.maximum_position_correction_m, nc.momentum_residual_x, nc.momentum_residual_y, nc.momentum_residual_z,
            st.damping_dissipated_j, st.striker_dissipated_j]
    return {"status_u64": u, "status_f64": d, "bond_projections": np.array([st.bond_projections], np.uint64)}


def run_case(case: dict, precision: str = "float", per_substep: bool = False, threads_per_block: int = 0) -> dict:
    """Runs a scene case through the GPU backend the way a reference caller
    would (schedule, state, upload, loads, run, download) and returns the same
    output arrays the CPU checkers return."""
    n = int(case["node_count"][0])
    sched = build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = build_lattice_state(case, sched)
    backend = make_gb300_lattice_backend(sched, precision, threads_per_block)
    settings = step_settings(case["settings"])
    settings.direct_arithmetic = 1 if precision == "double" else 0
    backend.upload(state, settings, sphere_state(case["sphere"]))
    steps = int(case["steps"][0])
    per_step = int(case.get("substeps_per_step", [1])[0])
    ramp = "force_ramp_steps" in case
    base = case.get("forces")
    if base is not None and not ramp:
        backend.set_external_forces(base, int(case["force_substeps"][0]))
    if "wrench_names" in case:
        backend.set_external_wrenches(case_wrenches(case), int(case["wrench_substeps"][0]))
    break_step = np.full(int(case["bond_count"][0]), NO_BOND, dtype=np.uint32)
    alive_before = state.alive.copy()
    chunk = 1 if per_substep else (per_step if ramp else steps)
    done = 0
    st = None
    resume_at = int(case["checkpoint_at"][0]) if "checkpoint_at" in case else 0
    while done < steps:
        if ramp and done % per_step == 0:
            scale = float(case["force_ramp_scale"][0]) * (done // per_step) / float(case["force_ramp_steps"][0])
            backend.set_external_forces(scale * base, per_step)
        nsteps = min(chunk, steps - done)
        if resume_at:
            if done < resume_at:
                nsteps = min(nsteps, resume_at - done)
            elif done == resume_at:
                # Checkpoint and resume: the state downloaded, uploaded into a
                # fresh backend, the run carried on (FastLattice.hpp:359-361).
                sp = backend.download(state)
                backend = make_gb300_lattice_backend(sched, precision, threads_per_block)
                backend.upload(state, settings, sp)
        st = backend.run(RunControl(max_steps=nsteps))
        done += nsteps
        if per_substep:
            backend.download(state)
            newly = (alive_before != 0) & (state.alive == 0)
            break_step[newly] = done - 1
            alive_before = state.alive.copy()
    sp = backend.download(state)
    out = state_outputs(state, sp, backend.first_failure_bonds(), st)
    out["state_nbr_other"] = state.nbr_other.copy()
    out["state_max_degree"] = np.array([state.view.max_degree], np.uint32)
    out.update(sched.arrays())
    out.update(source_arrays(backend.external_sources()))
    if per_substep:
        out["break_step"] = break_step
    return out


def state_outputs(state: State, sp: Sphere, ffb: np.ndarray, st: RunStatus) -> dict:
    """A downloaded lattice and its status as the output arrays the CPU
    checkers return (the state and status keys of run_case)."""
    out = {"u": state.u.copy(), "u_prev": state.u_prev.copy(), "v": state.v.copy(), "alive": state.alive.copy(),
           "failure_mode": state.failure_mode.copy(), "damage": state.damage.copy(),
           "plastic_extension": state.plastic_extension.copy(), "plastic_strain": state.plastic_strain.copy(),
           "prev_tensile": state.prev_tensile.copy(), "prev_compressive": state.prev_compressive.copy(),
           "prev_shear": state.prev_shear.copy(), "sphere_out": pack_sphere(sp), "first_failure_bonds": ffb}
    out.update(status_arrays(st))
    return out


def run_batch(cases: list, precision: str = "float", control: RunControl | None = None, tuning=None) -> list:
    """Runs scene cases as one batch (they must share step settings) and
    returns one output dict per case: the state and status keys of run_case.
    Every case runs `control` (default: the longest case's substep count);
    exit rules stop each case on its own. `tuning`: "tune" runs the autotuner
    after settling, a dict sets launch shapes (Batch.set_tuning)."""
    for c in cases[1:]:
        if not np.array_equal(c["settings"], cases[0]["settings"]):
            raise ValueError("the cases of one batch share their step settings")
    batch = Batch(precision)
    settings = step_settings(cases[0]["settings"])
    settings.direct_arithmetic = 1 if precision == "double" else 0
    states = []
    for c in cases:
        n = int(c["node_count"][0])
        sched = build_lattice_schedule(n, c["bond_a"], c["bond_b"], c["node_block_begin"])
        state = build_lattice_state(c, sched)
        batch.add(sched, state, sphere_state(c["sphere"]))
        states.append(state)
    batch.settle(settings)
    if tuning == "tune":
        batch.tune()
    elif tuning:
        batch.set_tuning(**tuning)
    for k, c in enumerate(cases):
        if c.get("forces") is not None and "force_ramp_steps" not in c:
            batch.set_external_forces(k, c["forces"], int(c["force_substeps"][0]))
        if "wrench_names" in c:
            batch.set_external_wrenches(k, case_wrenches(c), int(c["wrench_substeps"][0]))
    steps = max(int(c["steps"][0]) for c in cases)
    batch.run(control if control is not None else RunControl(max_steps=steps))
    outs = []
    for k, state in enumerate(states):
        sp = batch.download(k, state)
        out = state_outputs(state, sp, batch.first_failure_bonds(k), batch.status(k))
        out.update(source_arrays(batch.external_sources(k)))
        outs.append(out)
    return outs
