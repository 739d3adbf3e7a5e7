"""Python binding of libb2g.so (the GB300 Step engine) through its C ABI (include/b2g_capi.h).

The records below mirror the C structs field for field (ctypes applies the same alignment rules
as the C compiler). ``Lib`` loads the shared library built in-tree by ``build.py``; there is no
fallback path: if the library is missing, loading fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libb2g.so"

B2G_OK = 0
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "TIMEOUT", 4: "WORLD_FAULT", 5: "CUDA",
          6: "LOCKED", 7: "CAPACITY", 8: "CANCELLED"}

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
SHAPE_CIRCLE, SHAPE_EDGE, SHAPE_POLYGON = 0, 1, 2
JOINT_REVOLUTE, JOINT_PRISMATIC, JOINT_DISTANCE = 1, 2, 3
POLY_HULL, POLY_BOX, POLY_BOX_ORIENTED, POLY_RAW = 0, 1, 2, 3
SCENE_PYRAMID, SCENE_MIXED_DROP, SCENE_CHAINS, SCENE_BATCH_WORLD, SCENE_JOINTS, SCENE_SLIDERS, SCENE_GEARS = 0, 1, 2, 3, 4, 5, 6
SCENE_BULLETS = 7
JOINT_REVOLUTE, JOINT_PRISMATIC, JOINT_DISTANCE, JOINT_PULLEY, JOINT_MOUSE = 1, 2, 3, 4, 5
JOINT_WHEEL, JOINT_WELD, JOINT_FRICTION, JOINT_MOTOR, JOINT_GEAR = 7, 8, 9, 11, 6
BODY_ENABLED, BODY_FIXED_ROTATION, BODY_BULLET, BODY_AWAKE, BODY_AUTO_SLEEP = 1, 2, 4, 8, 16
HOST_ONLY = -1  # B2G_HOST_ONLY: a batch built and read on the host only (no device)
EVENT_BEGIN, EVENT_END, EVENT_PRESOLVE, EVENT_POSTSOLVE = 1, 2, 3, 4
CONTACT_TOUCHING, CONTACT_ENABLED = 2, 4

F2 = C.c_float * 2


class Shape(C.Structure):
    _fields_ = [("type", C.c_int32), ("count", C.c_int32), ("radius", C.c_float),
                ("one_sided", C.c_int32), ("vertices", F2 * 8), ("normals", F2 * 8),
                ("centroid", F2)]


class ManifoldPoint(C.Structure):
    _fields_ = [("local_point", F2), ("normal_impulse", C.c_float),
                ("tangent_impulse", C.c_float), ("id", C.c_uint32)]


class Manifold(C.Structure):
    _fields_ = [("points", ManifoldPoint * 2), ("local_normal", F2), ("local_point", F2),
                ("type", C.c_int32), ("point_count", C.c_int32)]


class Sweep(C.Structure):
    _fields_ = [("local_center", F2), ("c0", F2), ("c", F2), ("a0", C.c_float), ("a", C.c_float),
                ("alpha0", C.c_float)]


class TOIInput(C.Structure):
    _fields_ = [("shape_a", Shape), ("shape_b", Shape), ("sweep_a", Sweep), ("sweep_b", Sweep),
                ("t_max", C.c_float)]


class TOIOutput(C.Structure):
    _fields_ = [("state", C.c_int32), ("t", C.c_float)]


TOI_UNKNOWN, TOI_FAILED, TOI_OVERLAPPED, TOI_TOUCHING, TOI_SEPARATED = 0, 1, 2, 3, 4


class BodyDef(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", F2), ("angle", C.c_float),
                ("linear_velocity", F2), ("angular_velocity", C.c_float),
                ("linear_damping", C.c_float), ("angular_damping", C.c_float),
                ("gravity_scale", C.c_float), ("allow_sleep", C.c_int32), ("awake", C.c_int32),
                ("fixed_rotation", C.c_int32), ("bullet", C.c_int32), ("enabled", C.c_int32),
                ("user_data", C.c_uint64)]


class FixtureDef(C.Structure):
    _fields_ = [("body", C.c_int32), ("shape_type", C.c_int32), ("poly_mode", C.c_int32),
                ("count", C.c_int32), ("verts", F2 * 8), ("box", C.c_float * 5),
                ("radius", C.c_float), ("center", F2), ("one_sided", C.c_int32),
                ("friction", C.c_float), ("restitution", C.c_float),
                ("restitution_threshold", C.c_float), ("density", C.c_float),
                ("is_sensor", C.c_int32), ("category_bits", C.c_uint16),
                ("mask_bits", C.c_uint16), ("group_index", C.c_int16), ("pad0", C.c_int16),
                ("user_data", C.c_uint64), ("shape", Shape)]


class JointDef(C.Structure):
    _fields_ = [("type", C.c_int32), ("body_a", C.c_int32), ("body_b", C.c_int32),
                ("collide_connected", C.c_int32), ("local_anchor_a", F2),
                ("local_anchor_b", F2), ("reference_angle", C.c_float),
                ("local_axis_a", F2), ("enable_limit", C.c_int32), ("lower", C.c_float),
                ("upper", C.c_float), ("enable_motor", C.c_int32), ("max_motor", C.c_float),
                ("motor_speed", C.c_float), ("length", C.c_float), ("min_length", C.c_float),
                ("max_length", C.c_float), ("stiffness", C.c_float), ("damping", C.c_float),
                ("linear_offset", F2), ("max_force", C.c_float), ("max_torque", C.c_float),
                ("correction_factor", C.c_float), ("target", F2), ("ground_anchor_a", F2),
                ("ground_anchor_b", F2), ("length_a", C.c_float), ("length_b", C.c_float),
                ("ratio", C.c_float), ("user_data", C.c_uint64), ("joint_1", C.c_int32),
                ("joint_2", C.c_int32), ("gear_constant", C.c_float), ("reserved", C.c_int32)]


class Body(C.Structure):
    _fields_ = [("xf", C.c_float * 4), ("c", F2), ("a", C.c_float), ("v", F2),
                ("w", C.c_float), ("local_center", F2), ("mass", C.c_float),
                ("inv_mass", C.c_float), ("inertia", C.c_float), ("inv_inertia", C.c_float),
                ("linear_damping", C.c_float), ("angular_damping", C.c_float),
                ("gravity_scale", C.c_float), ("force", F2), ("torque", C.c_float),
                ("type", C.c_int32), ("flags", C.c_uint32)]


class Fixture(C.Structure):
    _fields_ = [("shape", Shape), ("body", C.c_int32), ("density", C.c_float),
                ("friction", C.c_float), ("restitution", C.c_float),
                ("restitution_threshold", C.c_float), ("category_bits", C.c_uint16),
                ("mask_bits", C.c_uint16), ("group_index", C.c_int16), ("is_sensor", C.c_uint8),
                ("pad0", C.c_uint8)]


class Joint(C.Structure):
    _fields_ = [("def_", JointDef), ("impulse", C.c_float * 3), ("motor_impulse", C.c_float),
                ("lower_impulse", C.c_float), ("upper_impulse", C.c_float),
                ("reaction_impulse", F2), ("reaction_angular_impulse", C.c_float)]


class Contact(C.Structure):
    _fields_ = [("fixture_a", C.c_int32), ("fixture_b", C.c_int32), ("flags", C.c_uint32),
                ("friction", C.c_float), ("restitution", C.c_float),
                ("restitution_threshold", C.c_float), ("tangent_speed", C.c_float),
                ("manifold", Manifold)]


class Event(C.Structure):
    _fields_ = [("kind", C.c_int32), ("world", C.c_int32), ("fixture_a", C.c_int32),
                ("fixture_b", C.c_int32), ("point_count", C.c_int32),
                ("normal_impulses", F2), ("tangent_impulses", F2), ("old_manifold", Manifold)]


class Profile(C.Structure):
    _fields_ = [("step", C.c_float), ("collide", C.c_float), ("solve", C.c_float),
                ("broadphase", C.c_float), ("solve_toi", C.c_float), ("bodies", C.c_int64),
                ("fixtures", C.c_int64), ("contacts", C.c_int64), ("touching", C.c_int64),
                ("joints", C.c_int64), ("colors_max", C.c_int64), ("touching_total", C.c_int64),
                ("host_step", C.c_float), ("host_admit_upload", C.c_float),
                ("host_admit_broadphase", C.c_float), ("host_grow", C.c_float)]


class RayHit(C.Structure):
    _fields_ = [("fixture", C.c_int32), ("point", C.c_float * 2), ("normal", C.c_float * 2),
                ("fraction", C.c_float)]


class RequestResult(C.Structure):
    _fields_ = [("request_id", C.c_int64), ("status", C.c_int32), ("bodies", C.c_int32),
                ("steps", C.c_int32), ("submit_time_s", C.c_double),
                ("admit_time_s", C.c_double), ("finish_time_s", C.c_double),
                ("checksum", C.c_float * 4)]


RECORD_SIZES = {"b2g_shape": 152, "b2g_manifold_point": 20, "b2g_manifold": 64, "b2g_body": 96}


def body_array_to_numpy(arr) -> dict:
    """Body records -> dict of numpy arrays (xf[n,4], c[n,2], a[n], v[n,2], w[n], type[n])."""
    n = len(arr)
    raw = np.frombuffer(arr, dtype=np.uint8).reshape(n, C.sizeof(Body))
    f = raw[:, :88].copy().view(np.float32).reshape(n, 22)
    t = raw[:, 88:92].copy().view(np.int32).reshape(n)
    return {"xf": f[:, 0:4], "c": f[:, 4:6], "a": f[:, 6], "v": f[:, 7:9], "w": f[:, 9],
            "local_center": f[:, 10:12], "mass": f[:, 12], "inv_mass": f[:, 13],
            "inertia": f[:, 14], "inv_inertia": f[:, 15], "type": t}


class Server:
    """Continuous-batching rollout server (b2g_server)."""

    def __init__(self, lib, device=0, budget_bytes=120 << 30, max_worlds=4096, dt=1 / 60, vi=8, pi=3,
                 builders=None):
        self.lib = lib
        h = C.c_void_p()
        lib.check(lib.b2g_server_create(device, budget_bytes, max_worlds, dt, vi, pi, C.byref(h)),
                  "b2g_server_create")
        self.h = h
        if builders is not None:
            lib.check(lib.b2g_server_set_builders(h, builders), "b2g_server_set_builders")

    def close(self):
        if self.h:
            self.lib.b2g_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def submit(self, seed, bodies, steps) -> int:
        rid = C.c_int64()
        self.lib.check(self.lib.b2g_server_submit(self.h, seed, bodies, steps, C.byref(rid)), "submit")
        return rid.value

    def tick(self):
        active = C.c_int32()
        ms = C.c_double()
        self.lib.check(self.lib.b2g_server_tick(self.h, C.byref(active), C.byref(ms)), "tick")
        return active.value, ms.value

    def poll(self, cap=4096):
        arr = (RequestResult * cap)()
        n = C.c_int32()
        self.lib.check(self.lib.b2g_server_poll(self.h, arr, cap, C.byref(n)), "poll")
        return arr[:n.value]

    def cancel(self, request_id):
        """Cancels a queued or running request (it finishes with status B2G_E_CANCELLED)."""
        return self.lib.b2g_server_cancel(self.h, request_id)

    def stats(self):
        v = [C.c_int64() for _ in range(5)]
        self.lib.check(self.lib.b2g_server_stats(self.h, *[C.byref(x) for x in v]), "stats")
        return dict(zip(("queued", "active", "completed", "rejected", "hbm_bytes"), (x.value for x in v)))


class B2GError(RuntimeError):
    pass


def _check(status: int, what: str, lib=None):
    if status != B2G_OK:
        detail = ""
        if lib is not None:
            try:
                detail = lib.b2g_last_error().decode()
            except Exception:  # noqa: BLE001 - the message is best effort
                detail = ""
        raise B2GError(f"{what} failed: {STATUS.get(status, status)} {detail}")


class Lib:
    """The loaded libb2g.so with argument types declared for every C-ABI entry point."""

    SYMBOLS = [
        "b2g_batch_create", "b2g_batch_destroy", "b2g_world_add", "b2g_world_count",
        "b2g_world_set_gravity", "b2g_world_set_flags", "b2g_bodies_add", "b2g_fixtures_add",
        "b2g_joints_add", "b2g_world_sizes", "b2g_step", "b2g_step_n", "b2g_step_timed",
        "b2g_batch_set_forces", "b2g_batch_set_graphs", "b2g_batch_set_debug_checks",
        "b2g_batch_set_solver_threads",
        "b2g_batch_get_solver_threads", "b2g_batch_autotune", "b2g_world_retire", "b2g_compact", "b2g_debug_set_contact_capacity",
        "b2g_pairs_static", "b2g_reserve",
        "b2g_bodies_read", "b2g_bodies_write", "b2g_batch_read_states", "b2g_fixtures_read",
        "b2g_joints_read", "b2g_contacts_read", "b2g_events_enable", "b2g_events_drain",
        "b2g_profile_get", "b2g_solver_order", "b2g_collide", "b2g_time_of_impact", "b2g_pairs", "b2g_scene_build",
        "b2g_batch_world_params", "b2g_server_create", "b2g_server_destroy", "b2g_server_submit",
        "b2g_server_tick", "b2g_server_poll", "b2g_server_stats", "b2g_status_string",
        "b2g_last_error", "b2g_device_count", "b2g_query_aabb", "b2g_raycast_closest", "b2g_world_status",
        "b2g_world_snapshot", "b2g_world_restore", "b2g_server_cancel", "b2g_body_set_awake", "b2g_body_set_bullet",
        "b2g_bodies_sleep_time_read", "b2g_world_get_flags", "b2g_server_batch", "b2g_step_begin",
        "b2g_step_poll", "b2g_step_end", "b2g_batch_stage", "b2g_server_set_builders", "b2g_batch_set_solver_waves", "b2g_batch_set_tree_rebuild_period",
        "b2g_batch_set_cluster_solve", "b2g_batch_get_cluster_solve", "b2g_events_drain_world",
        "b2g_bodies_remove", "b2g_fixtures_remove", "b2g_joints_remove", "b2g_world_dump", "b2g_step_io",
    ]

    def __init__(self, path: os.PathLike | str | None = None):
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise B2GError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; "
                           f"g.build()'` (the engine has no CPU fallback)")
        self.path = p
        self.lib = C.CDLL(str(p))
        L = self.lib
        vp, i32, u32, f32, i64 = C.c_void_p, C.c_int32, C.c_uint32, C.c_float, C.c_int64
        P = C.POINTER
        sig = {
            "b2g_batch_create": ([C.c_int, C.c_uint64, P(vp)], C.c_int),
            "b2g_batch_destroy": ([vp], C.c_int),
            "b2g_world_add": ([vp, f32, f32, P(i32)], C.c_int),
            "b2g_world_count": ([vp, P(i32)], C.c_int),
            "b2g_world_set_gravity": ([vp, i32, f32, f32], C.c_int),
            "b2g_world_set_flags": ([vp, i32, i32, i32, i32, i32], C.c_int),
            "b2g_bodies_add": ([vp, i32, P(BodyDef), i32, P(i32)], C.c_int),
            "b2g_fixtures_add": ([vp, i32, P(FixtureDef), i32, P(i32)], C.c_int),
            "b2g_joints_add": ([vp, i32, P(JointDef), i32, P(i32)], C.c_int),
            "b2g_world_sizes": ([vp, i32, P(i32), P(i32), P(i32), P(i32)], C.c_int),
            "b2g_step": ([vp, f32, i32, i32, P(C.c_uint8)], C.c_int),
            "b2g_step_n": ([vp, f32, i32, i32, i32, i32], C.c_int),
            "b2g_step_timed": ([vp, f32, i32, i32, i32, P(f32)], C.c_int),
            "b2g_batch_set_forces": ([vp, vp, i64], C.c_int),
            "b2g_step_io": ([vp, f32, i32, i32, vp, i64, vp, i64, P(i64)], C.c_int),
            "b2g_batch_set_graphs": ([vp, i32], C.c_int),
            "b2g_world_retire": ([vp, i32], C.c_int),
            "b2g_compact": ([vp, P(i32), i32], C.c_int),
            "b2g_debug_set_contact_capacity": ([vp, i64], C.c_int),
            "b2g_pairs_static": ([vp, i32, vp, i64, P(i64), vp], C.c_int),
            "b2g_reserve": ([vp, i64], C.c_int),
            "b2g_bodies_read": ([vp, i32, i32, i32, P(Body)], C.c_int),
            "b2g_bodies_write": ([vp, i32, i32, i32, P(Body)], C.c_int),
            "b2g_batch_read_states": ([vp, P(f32), P(f32), i64, P(i64)], C.c_int),
            "b2g_fixtures_read": ([vp, i32, i32, i32, P(Fixture)], C.c_int),
            "b2g_joints_read": ([vp, i32, i32, i32, P(Joint)], C.c_int),
            "b2g_contacts_read": ([vp, i32, P(Contact), i32, P(i32)], C.c_int),
            "b2g_events_enable": ([vp, i32], C.c_int),
            "b2g_events_drain": ([vp, P(Event), i32, P(i32)], C.c_int),
            "b2g_events_drain_world": ([vp, i32, P(Event), i32, P(i32)], C.c_int),
            "b2g_bodies_remove": ([vp, i32, P(i32), i32, P(Event), i32, P(i32)], C.c_int),
            "b2g_fixtures_remove": ([vp, i32, P(i32), i32, P(Event), i32, P(i32)], C.c_int),
            "b2g_joints_remove": ([vp, i32, P(i32), i32], C.c_int),
            "b2g_world_dump": ([vp, i32, C.c_char_p, C.c_uint64, P(C.c_uint64)], C.c_int),
            "b2g_profile_get": ([vp, P(Profile)], C.c_int),
            "b2g_batch_set_solver_threads": ([vp, P(i32)], C.c_int),
            "b2g_batch_get_solver_threads": ([vp, P(i32)], C.c_int),
            "b2g_batch_autotune": ([vp, i32, f32, i32, i32, P(i32), P(i32)], C.c_int),
            "b2g_world_status": ([vp, i32, P(i32)], C.c_int),
            "b2g_server_cancel": ([vp, i64], C.c_int),
            "b2g_server_batch": ([vp, P(vp)], C.c_int),
            "b2g_step_begin": ([vp, f32, i32, i32, P(C.c_uint8)], C.c_int),
            "b2g_step_poll": ([vp, P(i32)], C.c_int),
            "b2g_step_end": ([vp], C.c_int),
            "b2g_batch_stage": ([vp], C.c_int),
            "b2g_server_set_builders": ([vp, i32], C.c_int),
            "b2g_batch_set_solver_waves": ([vp, f32], C.c_int),
            "b2g_batch_set_cluster_solve": ([vp, i32], C.c_int),
            "b2g_batch_get_cluster_solve": ([vp, P(i32)], C.c_int),
            "b2g_batch_set_tree_rebuild_period": ([vp, i32], C.c_int),
            "b2g_batch_set_debug_checks": ([vp, i32], C.c_int),
            "b2g_body_set_awake": ([vp, i32, i32, i32], C.c_int),
            "b2g_body_set_bullet": ([vp, i32, i32, i32], C.c_int),
            "b2g_world_get_flags": ([vp, i32, P(i32), P(i32), P(i32), P(i32)], C.c_int),
            "b2g_bodies_sleep_time_read": ([vp, i32, i32, i32, P(f32)], C.c_int),
            "b2g_world_snapshot": ([vp, i32, vp, C.c_uint64, P(C.c_uint64)], C.c_int),
            "b2g_world_restore": ([vp, vp, C.c_uint64, P(i32)], C.c_int),
            "b2g_query_aabb": ([vp, P(i32), P(f32), i32, P(i32), P(i32), i64, P(i64)], C.c_int),
            "b2g_raycast_closest": ([vp, P(i32), P(f32), i32, P(RayHit)], C.c_int),
            "b2g_solver_order": ([vp, i32, P(i32), P(u32), i32, P(i32), P(u32), i32], C.c_int),
            "b2g_collide": ([vp, vp, vp, vp, i32, vp, vp], C.c_int),
            "b2g_time_of_impact": ([vp, i32, vp, vp], C.c_int),
            "b2g_pairs": ([vp, i32, vp, i64, P(i64), vp], C.c_int),
            "b2g_scene_build": ([vp, i32, i32, u32, i32, f32, f32, P(i32)], C.c_int),
            "b2g_batch_world_params": ([u32, P(i32), P(f32), P(f32)], C.c_int),
            "b2g_server_create": ([C.c_int, C.c_uint64, i32, f32, i32, i32, P(vp)], C.c_int),
            "b2g_server_destroy": ([vp], C.c_int),
            "b2g_server_submit": ([vp, u32, i32, i32, P(i64)], C.c_int),
            "b2g_server_tick": ([vp, P(i32), P(C.c_double)], C.c_int),
            "b2g_server_poll": ([vp, P(RequestResult), i32, P(i32)], C.c_int),
            "b2g_server_stats": ([vp, P(i64), P(i64), P(i64), P(i64), P(i64)], C.c_int),
            "b2g_status_string": ([C.c_int], C.c_char_p),
            "b2g_last_error": ([], C.c_char_p),
            "b2g_device_count": ([P(i32)], C.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res

    def __getattr__(self, name):
        return getattr(self.lib, name)

    def check(self, status: int, what: str):
        _check(status, what, self.lib)


class Batch:
    """A batch of worlds on one GPU (b2g_batch)."""

    def __init__(self, lib: Lib, device: int = 0, budget_bytes: int = 0):
        self.lib = lib
        h = C.c_void_p()
        lib.check(lib.b2g_batch_create(device, budget_bytes, C.byref(h)), "b2g_batch_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.b2g_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def add_world(self, gx=0.0, gy=-10.0) -> int:
        w = C.c_int32()
        self.lib.check(self.lib.b2g_world_add(self.h, gx, gy, C.byref(w)), "b2g_world_add")
        return w.value

    def set_flags(self, world, allow_sleep=False, warm_starting=True, continuous=False,
                  auto_clear_forces=True):
        self.lib.check(self.lib.b2g_world_set_flags(self.h, world, int(allow_sleep),
                                                    int(warm_starting), int(continuous),
                                                    int(auto_clear_forces)),
                       "b2g_world_set_flags")

    def scene(self, world, kind, seed=1, n=20, p0=1.0, p1=0.6):
        counts = (C.c_int32 * 3)()
        self.lib.check(self.lib.b2g_scene_build(self.h, world, kind, seed, n, p0, p1, counts),
                       "b2g_scene_build")
        return tuple(counts)

    def sizes(self, world):
        v = [C.c_int32() for _ in range(4)]
        self.lib.check(self.lib.b2g_world_sizes(self.h, world, *[C.byref(x) for x in v]),
                       "b2g_world_sizes")
        return tuple(x.value for x in v)

    def step(self, dt=1 / 60, vi=8, pi=3, mask=None):
        m = None
        if mask is not None:
            arr = (C.c_uint8 * len(mask))(*[1 if x else 0 for x in mask])
            m = C.cast(arr, C.POINTER(C.c_uint8))
        self.lib.check(self.lib.b2g_step(self.h, dt, vi, pi, m), "b2g_step")

    def step_begin(self, dt=1 / 60, vi=8, pi=3, mask=None):
        """Launches one step and returns at once (b2g_step_begin); finish it with step_end."""
        self._mask = None
        if mask is not None:
            self._mask = (C.c_uint8 * len(mask))(*[1 if x else 0 for x in mask])
        m = C.cast(self._mask, C.POINTER(C.c_uint8)) if self._mask is not None else None
        self.lib.check(self.lib.b2g_step_begin(self.h, dt, vi, pi, m), "b2g_step_begin")

    def step_done(self) -> bool:
        d = C.c_int32()
        self.lib.check(self.lib.b2g_step_poll(self.h, C.byref(d)), "b2g_step_poll")
        return bool(d.value)

    def step_end(self):
        self.lib.check(self.lib.b2g_step_end(self.h), "b2g_step_end")

    def stage(self):
        """Packs the worlds not on the device yet for the next step's upload (b2g_batch_stage)."""
        self.lib.check(self.lib.b2g_batch_stage(self.h), "b2g_batch_stage")

    def step_n(self, n, dt=1 / 60, vi=8, pi=3, use_graph=False):
        self.lib.check(self.lib.b2g_step_n(self.h, dt, vi, pi, n, int(use_graph)), "b2g_step_n")

    def step_timed(self, n, dt=1 / 60, vi=8, pi=3) -> float:
        ms = C.c_float()
        self.lib.check(self.lib.b2g_step_timed(self.h, dt, vi, pi, n, C.byref(ms)), "b2g_step_timed")
        return ms.value

    def bodies(self, world):
        nb = self.sizes(world)[0]
        arr = (Body * max(nb, 1))()
        self.lib.check(self.lib.b2g_bodies_read(self.h, world, 0, nb, arr), "b2g_bodies_read")
        return arr[:nb] if nb else []

    def bodies_np(self, world):
        nb = self.sizes(world)[0]
        arr = (Body * max(nb, 1))()
        self.lib.check(self.lib.b2g_bodies_read(self.h, world, 0, nb, arr), "b2g_bodies_read")
        return body_array_to_numpy((Body * nb).from_buffer(arr)) if nb else None

    def write_bodies(self, world, recs):
        arr = (Body * len(recs))(*recs)
        self.lib.check(self.lib.b2g_bodies_write(self.h, world, 0, len(recs), arr),
                       "b2g_bodies_write")

    def fixtures(self, world):
        nf = self.sizes(world)[1]
        arr = (Fixture * max(nf, 1))()
        self.lib.check(self.lib.b2g_fixtures_read(self.h, world, 0, nf, arr), "b2g_fixtures_read")
        return arr[:nf] if nf else []

    def joints(self, world):
        nj = self.sizes(world)[2]
        arr = (Joint * max(nj, 1))()
        self.lib.check(self.lib.b2g_joints_read(self.h, world, 0, nj, arr), "b2g_joints_read")
        return arr[:nj] if nj else []

    def contacts(self, world):
        n = C.c_int32()
        self.lib.check(self.lib.b2g_contacts_read(self.h, world, None, 0, C.byref(n)),
                       "b2g_contacts_read")
        arr = (Contact * max(n.value, 1))()
        self.lib.check(self.lib.b2g_contacts_read(self.h, world, arr, n.value, C.byref(n)),
                       "b2g_contacts_read")
        return arr[:n.value]

    def set_awake(self, world, body, awake=True):
        """b2Body::SetAwake."""
        self.lib.check(self.lib.b2g_body_set_awake(self.h, world, body, int(awake)), "b2g_body_set_awake")

    def set_bullet(self, world, body, bullet=True):
        """b2Body::SetBullet: continuous collision with other dynamic bodies."""
        self.lib.check(self.lib.b2g_body_set_bullet(self.h, world, body, int(bullet)), "b2g_body_set_bullet")

    def sleep_times(self, world):
        """The bodies' sleep timers (b2Body::m_sleepTime) in creation order."""
        nb = self.sizes(world)[0]
        arr = (C.c_float * max(nb, 1))()
        self.lib.check(self.lib.b2g_bodies_sleep_time_read(self.h, world, 0, nb, arr), "b2g_bodies_sleep_time_read")
        return list(arr[:nb])

    def step_io(self, forces_ptr, n_bodies, xf_ptr, cap_bodies, dt=1 / 60, vi=8, pi=3) -> int:
        """One step with its host I/O (b2g_step_io): the forces of every body from host address
        `forces_ptr` (0: the forces already set), the transforms to host address `xf_ptr` (0:
        none). Returns the number of bodies."""
        n = C.c_int64()
        self.lib.check(self.lib.b2g_step_io(self.h, dt, vi, pi, C.c_void_p(forces_ptr or None), n_bodies,
                                            C.c_void_p(xf_ptr or None), cap_bodies, C.byref(n)), "b2g_step_io")
        return n.value

    def set_graphs(self, enable=True):
        """Whether unmasked steps replay a captured CUDA graph (default on)."""
        self.lib.check(self.lib.b2g_batch_set_graphs(self.h, int(enable)), "b2g_batch_set_graphs")

    def cluster_solve(self, ctas=-1):
        """CTAs per world of the thread-block cluster that solves worlds above 8192 bodies (-1:
        the device's largest; 0 or 1: one CTA per world). Results do not depend on it."""
        self.lib.check(self.lib.b2g_batch_set_cluster_solve(self.h, int(ctas)), "b2g_batch_set_cluster_solve")

    def cluster_ctas(self) -> int:
        """CTAs per world the worlds above 8192 bodies are solved with (1: one CTA)."""
        v = C.c_int32()
        self.lib.check(self.lib.b2g_batch_get_cluster_solve(self.h, C.byref(v)), "b2g_batch_get_cluster_solve")
        return v.value

    def set_debug_checks(self, enable=True):
        """Verify every step's constraint colouring on the device (a violation fails the step)."""
        self.lib.check(self.lib.b2g_batch_set_debug_checks(self.h, int(enable)), "b2g_batch_set_debug_checks")

    def solver_threads(self, threads=None):
        """Threads per world CTA of the solver for the five size classes (sets when given)."""
        arr = (C.c_int32 * 5)()
        if threads is not None:
            arr = (C.c_int32 * 5)(*threads)
            self.lib.check(self.lib.b2g_batch_set_solver_threads(self.h, arr), "b2g_batch_set_solver_threads")
        self.lib.check(self.lib.b2g_batch_get_solver_threads(self.h, arr), "b2g_batch_get_solver_threads")
        return list(arr)

    def autotune(self, steps=3, dt=1 / 60, vi=8, pi=3):
        """Picks the solver's threads per world for each size class by timing real steps;
        returns (threads per class, steps taken)."""
        arr = (C.c_int32 * 5)()
        taken = C.c_int32()
        self.lib.check(self.lib.b2g_batch_autotune(self.h, steps, dt, vi, pi, arr, C.byref(taken)),
                       "b2g_batch_autotune")
        return list(arr), taken.value

    def snapshot(self, world) -> bytes:
        """The world's complete state (checkpoint) as bytes."""
        size = C.c_uint64()
        st = self.lib.lib.b2g_world_snapshot(self.h, world, None, 0, C.byref(size))
        if st not in (0, 7):  # B2G_OK for an empty world, B2G_E_CAPACITY otherwise
            self.lib.check(st, "b2g_world_snapshot")
        buf = C.create_string_buffer(size.value)
        self.lib.check(self.lib.b2g_world_snapshot(self.h, world, buf, size.value, C.byref(size)), "b2g_world_snapshot")
        return buf.raw[:size.value]

    def restore(self, blob: bytes) -> int:
        """Appends a world from a snapshot; returns its index."""
        w = C.c_int32()
        buf = C.create_string_buffer(blob, len(blob))
        self.lib.check(self.lib.b2g_world_restore(self.h, buf, len(blob), C.byref(w)), "b2g_world_restore")
        return w.value

    def world_status(self, world):
        """B2G_OK, or B2G_E_WORLD_FAULT once the world was frozen after a non-finite state."""
        st = C.c_int32()
        self.lib.check(self.lib.b2g_world_status(self.h, world, C.byref(st)), "b2g_world_status")
        return st.value

    def raycast(self, worlds, rays):
        """Closest hit of each ray (x1, y1, x2, y2) in its world: list of
        (fixture, point, normal, fraction), fixture -1 for no hit."""
        n = len(worlds)
        w = (C.c_int32 * max(n, 1))(*worlds)
        r = (C.c_float * max(4 * n, 1))(*[v for ray in rays for v in ray])
        out = (RayHit * max(n, 1))()
        self.lib.check(self.lib.b2g_raycast_closest(self.h, w, r, n, out), "b2g_raycast_closest")
        return [(h.fixture, tuple(h.point), tuple(h.normal), h.fraction) if h.fixture >= 0 else (-1, None, None, None)
                for h in out[:n]]

    def query_aabb(self, worlds, boxes, cap=1 << 20):
        """Fixtures overlapping each box (lower x, y, upper x, y) in its world, ascending."""
        n = len(worlds)
        w = (C.c_int32 * max(n, 1))(*worlds)
        bx = (C.c_float * max(4 * n, 1))(*[v for box in boxes for v in box])
        counts = (C.c_int32 * max(n, 1))()
        out = (C.c_int32 * max(cap, 1))()
        total = C.c_int64()
        self.lib.check(self.lib.b2g_query_aabb(self.h, w, bx, n, counts, out, cap, C.byref(total)), "b2g_query_aabb")
        res, k = [], 0
        for q in range(n):
            res.append(list(out[k:k + counts[q]]))
            k += counts[q]
        return res

    def solver_order(self, world, nc, nj):
        cc = (C.c_int32 * max(nc, 1))()
        cp = (C.c_uint32 * max(nc, 1))()
        jc = (C.c_int32 * max(nj, 1))()
        jp = (C.c_uint32 * max(nj, 1))()
        self.lib.check(self.lib.b2g_solver_order(self.h, world, cc, cp, nc, jc, jp, nj),
                       "b2g_solver_order")
        return list(cc[:nc]), list(cp[:nc]), list(jc[:nj]), list(jp[:nj])

    def events(self, enable=None, cap=1 << 20):
        if enable is not None:
            self.lib.check(self.lib.b2g_events_enable(self.h, int(enable)), "b2g_events_enable")
            return None
        n = C.c_int32()
        arr = (Event * cap)()
        self.lib.check(self.lib.b2g_events_drain(self.h, arr, cap, C.byref(n)), "b2g_events_drain")
        return arr[:n.value]

    def remove(self, world, bodies=(), fixtures=(), joints=(), cap=1 << 16):
        """Removes bodies, then fixtures, then joints of `world` (indices as they are before each
        call); returns the End events of the touching contacts destroyed."""
        ended = []
        for fn, ids in ((self.lib.b2g_bodies_remove, bodies), (self.lib.b2g_fixtures_remove, fixtures)):
            if ids:
                arr = (C.c_int32 * len(ids))(*ids)
                ev = (Event * cap)()
                n = C.c_int32()
                self.lib.check(fn(self.h, world, arr, len(ids), ev, cap, C.byref(n)), "remove")
                ended += ev[:min(n.value, cap)]
        if joints:
            arr = (C.c_int32 * len(joints))(*joints)
            self.lib.check(self.lib.b2g_joints_remove(self.h, world, arr, len(joints)), "b2g_joints_remove")
        return ended

    def dump(self, world) -> str:
        """b2World::Dump of `world` as text (b2g_world_dump)."""
        n = C.c_uint64()
        self.lib.b2g_world_dump(self.h, world, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        self.lib.check(self.lib.b2g_world_dump(self.h, world, buf, n.value + 1, C.byref(n)), "b2g_world_dump")
        return buf.value.decode()

    def world_events(self, world, cap=1 << 20):
        """World `world`'s listener events of the last step (b2g_events_drain_world)."""
        n = C.c_int32()
        arr = (Event * cap)()
        self.lib.check(self.lib.b2g_events_drain_world(self.h, world, arr, cap, C.byref(n)), "b2g_events_drain_world")
        return arr[:n.value]

    def profile(self) -> Profile:
        p = Profile()
        self.lib.check(self.lib.b2g_profile_get(self.h, C.byref(p)), "b2g_profile_get")
        return p
