"""jsb: GB300-native soft-body solver step for Jolt Physics.

The product is ``libjsb.so`` (CUDA kernels for sm_103a + C++ host runtime) behind the C ABI declared
in ``include/jsb.h``. This module is a thin ctypes binding over that ABI, used by the tests and the
benchmark; it mirrors the reference's objects (shared settings bytes, creation settings, colliders,
bodies) and raises ``JsbError`` with the library's message on any non-zero status. There is no CPU
fallback: importing without a built ``libjsb.so`` raises.
"""
from __future__ import annotations

import ctypes
import os
import struct

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libjsb.so")

JSB_OK = 0
STATUS_NAMES = {
    1: "JSB_ERR_INVALID_ARGUMENT", 2: "JSB_ERR_BLOB", 3: "JSB_ERR_UNSUPPORTED", 4: "JSB_ERR_CUDA",
    5: "JSB_ERR_OUT_OF_MEMORY", 6: "JSB_ERR_TIMEOUT", 7: "JSB_ERR_NONFINITE", 8: "JSB_ERR_CAPACITY",
}
globals().update({name: code for code, name in STATUS_NAMES.items()})

# Every entry point of include/jsb.h with its ctypes signature.
_c = ctypes
_P = _c.c_void_p
SIGNATURES = {
    "jsb_context_create": [_c.c_int, _c.POINTER(_P)],
    "jsb_context_destroy": [_P],
    "jsb_last_error_string": [],
    "jsb_version": [],
    "jsb_set_gravity": [_P, _c.POINTER(_c.c_float)],
    "jsb_settings_upload": [_P, _c.c_char_p, _c.c_size_t, _c.POINTER(_c.c_uint32)],
    "jsb_body_add": [_P, _c.c_uint32, _c.c_char_p, _c.POINTER(_c.c_float), _c.POINTER(_c.c_uint32)],
    "jsb_body_restore_state": [_P, _c.c_uint32, _c.c_char_p, _c.c_size_t, _c.POINTER(_c.c_float)],
    "jsb_body_add_force": [_P, _c.c_uint32, _c.POINTER(_c.c_float)],
    "jsb_body_set_step_force": [_P, _c.c_uint32, _c.POINTER(_c.c_float)],
    "jsb_collider_add": [_P, _c.c_char_p, _c.POINTER(_c.c_uint32)],
    "jsb_set_sleep_settings": [_P, _c.c_float, _c.c_float],
    "jsb_body_is_active": [_P, _c.c_uint32, _c.POINTER(_c.c_int)],
    "jsb_body_set_active": [_P, _c.c_uint32, _c.c_int],
    "jsb_body_num_vertices": [_P, _c.c_uint32, _c.POINTER(_c.c_uint32)],
    "jsb_body_set_colliding_shapes": [_P, _c.c_uint32, _c.c_char_p, _c.c_uint32],
    "jsb_adjoint_bend_gradients": [_P, _c.c_uint32, _P],
    "jsb_body_bounds": [_P, _c.c_uint32, _P, _P],
    "jsb_hull_add": [_P, _P, _c.POINTER(_c.c_uint32)],
    "jsb_adjoint_timings": [_P, _P],
    "jsb_set_contact_readback": [_P, _c.c_int],
    "jsb_body_contacts": [_P, _c.c_uint32, _P, _P, _P, _P, _P],
    "jsb_body_clear_colliding_shapes": [_P, _c.c_uint32],
    "jsb_body_shape_velocities": [_P, _c.c_uint32, _P, _c.POINTER(_c.c_uint32)],
    "jsb_body_sensor_contacts": [_P, _c.c_uint32, _c.POINTER(_c.c_uint32)],
    "jsb_settings_regroup": [_c.c_char_p, _c.c_size_t, _P, _c.c_size_t, _c.POINTER(_c.c_size_t), _P],
    "jsb_body_skin_vertices": [_P, _c.c_uint32, _P, _c.c_uint32, _c.c_int],
    "jsb_body_set_skin_settings": [_P, _c.c_uint32, _c.c_int, _c.c_float],
    "jsb_step": [_P, _c.c_float, _c.c_int, _P],
    "jsb_step_plain": [_P, _c.c_float, _c.c_int, _P],
    "jsb_step_graph": [_P, _c.c_float, _c.c_int, _c.c_int, _c.c_int, _P],
    "jsb_synchronize": [_P],
    "jsb_body_read": [_P, _c.c_uint32, _P, _P, _P],
    "jsb_body_save_state": [_P, _c.c_uint32, _P, _c.c_size_t, _c.POINTER(_c.c_size_t)],
    "jsb_state_upload_all": [_P, _P, _P, _P],
    "jsb_state_download_all": [_P, _P, _P, _P],
    "jsb_total_vertices": [_P, _c.POINTER(_c.c_uint64)],
    "jsb_body_schedule_info": [_P, _c.c_uint32, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32)],
    "jsb_settings_schedule": [_c.c_char_p, _c.c_size_t, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32), _P, _P, _P],
    "jsb_set_bucket_config": [_P, _c.c_uint32, _c.c_uint32, _c.c_uint32],
    "jsb_set_bucket_threads": [_P, _c.c_uint32, _c.c_uint32],
    "jsb_get_bucket_config": [_P, _c.c_uint32, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32)],
    "jsb_set_cluster_config": [_P, _c.c_uint32, _c.c_uint32],
    "jsb_set_step_walk": [_P, _c.c_int],
    "jsb_settings_step_schedule": [_c.c_char_p, _c.c_size_t, _c.c_uint32, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32), _P,
                                   _P, _P],
    "jsb_get_cluster_config": [_P, _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32)],
    "jsb_autotune": [_P, _c.c_float, _c.c_int],
    "jsb_last_launch_count": [_P, _c.POINTER(_c.c_uint32)],
    "jsb_last_kernel_ms": [_P, _c.POINTER(_c.c_float)],
    "jsb_body_set_compliance": [_P, _c.c_uint32, _P, _c.c_uint32, _P, _c.c_uint32],
    "jsb_adjoint_begin": [_P, _c.c_float, _c.c_int, _c.c_int],
    "jsb_adjoint_forward": [_P, _c.c_int],
    "jsb_adjoint_seed": [_P, _c.c_int, _c.c_uint32, _P],
    "jsb_adjoint_seed_all": [_P, _c.c_int, _c.c_void_p],
    "jsb_adjoint_gradients_all": [_P, _c.c_void_p, _c.c_void_p, _c.c_void_p],
    "jsb_body_positions_all": [_P, _c.c_void_p],
    "jsb_adjoint_backward": [_P],
    "jsb_adjoint_gradients": [_P, _c.c_uint32, _P, _P, _P, _P, _P],
    "jsb_adjoint_end": [_P],
    "jsb_step_body_noalloc": [_c.c_char_p, _c.c_size_t, _c.c_char_p, _c.c_char_p, _c.c_uint32, _c.POINTER(_c.c_float),
                              _c.POINTER(_c.c_float), _c.c_float, _P, _P, _P, _P, _P],
}


class JsbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib() -> ctypes.CDLL:
    """Loads libjsb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m joltphysics_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_char_p if name in ("jsb_last_error_string", "jsb_version") else ctypes.c_int
        _lib = L
    return _lib


def check(status: int):
    if status != JSB_OK:
        raise JsbError(status, lib().jsb_last_error_string().decode(errors="replace"))


def _f3(v) -> ctypes.Array:
    return (ctypes.c_float * 3)(*[float(x) for x in v])


CREATION_FMT = "<I7f4B"
COLLIDER_FMT = "<i3f3f3f"


def blob_counts(blob: bytes) -> dict:
    """Element counts of a SaveBinaryState blob (vertices, faces, edges, bends, volumes, ..., lra)."""
    names = [("vertices", 28), ("faces", 16), ("edges", 16), ("bends", 24), ("volumes", 24), ("skinned", 52),
             ("skinned_normals", 4), ("lra", 12)]
    out, off = {}, 0
    for name, size in names:
        (n,) = struct.unpack_from("<I", blob, off)
        out[name] = n
        off += 4 + n * size
    return out


def settings_schedule(blob: bytes):
    """Dependency-level schedule for settings bytes (host only): (levels (L+2, 4), records (R, 4), source (R,))."""
    nl, nr = ctypes.c_uint32(), ctypes.c_uint32()
    check(lib().jsb_settings_schedule(blob, len(blob), ctypes.byref(nl), ctypes.byref(nr), None, None, None))
    levels = np.zeros((nl.value + 2, 4), np.uint32)
    records = np.zeros((nr.value, 4), np.uint32)
    source = np.zeros(nr.value, np.uint32)
    check(lib().jsb_settings_schedule(blob, len(blob), ctypes.byref(nl), ctypes.byref(nr), levels.ctypes.data,
                                      records.ctypes.data, source.ctypes.data))
    return levels, records, source


def settings_regroup(blob: bytes):
    """Opt-in regrouped settings bytes (not the reference's constraint order; jsb_settings_regroup) and
    the remap: for the edges, bends, volumes and LRA constraints in their new order, the original index."""
    n = ctypes.c_size_t(0)
    check(lib().jsb_settings_regroup(blob, len(blob), None, 0, ctypes.byref(n), None))
    out = ctypes.create_string_buffer(n.value)
    remap = np.zeros(len(blob) // 12 + 1, np.uint32)  # more than the constraints of any blob of this size
    check(lib().jsb_settings_regroup(blob, len(blob), out, n.value, ctypes.byref(n), remap.ctypes.data))
    counts = blob_constraint_counts(out.raw[: n.value])
    return out.raw[: n.value], remap[:counts]


def blob_constraint_counts(blob: bytes) -> int:
    """Edges + bends + volumes + LRA constraints of settings bytes."""
    import struct

    off, total = 0, 0
    for name, size in (("v", 28), ("f", 16), ("e", 16), ("b", 24), ("vol", 24), ("sk", 52), ("skn", 4), ("lra", 12)):
        (n,) = struct.unpack_from("<I", blob, off)
        if name in ("e", "b", "vol", "lra"):
            total += n
        off += 4 + n * size
    return total


def settings_step_schedule(blob: bytes, num_iterations: int):
    """Whole-step schedule for settings bytes (host only): (levels (L, 4), records (S, 4), source (S, 2)),
    or None when the settings have none."""
    nl, ns = ctypes.c_uint32(), ctypes.c_uint32()
    check(lib().jsb_settings_step_schedule(blob, len(blob), num_iterations, ctypes.byref(nl), ctypes.byref(ns), None, None, None))
    if nl.value == 0:
        return None
    levels = np.zeros((nl.value, 4), np.uint32)
    records = np.zeros((ns.value, 4), np.uint32)
    source = np.zeros((ns.value, 2), np.uint32)
    check(lib().jsb_settings_step_schedule(blob, len(blob), num_iterations, ctypes.byref(nl), ctypes.byref(ns),
                                           levels.ctypes.data, records.ctypes.data, source.ctypes.data))
    return levels, records, source


class Context:
    """One GPU solver context (jsb_context)."""

    def __init__(self, device: int = 0):
        self.h = ctypes.c_void_p()
        check(lib().jsb_context_create(device, ctypes.byref(self.h)))
        self.num_vertices: list[int] = []
        self.bodies: list[dict] = []

    def close(self):
        if self.h:
            check(lib().jsb_context_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup -----------------------------------------------------------------------------------
    def set_gravity(self, g):
        check(lib().jsb_set_gravity(self.h, _f3(g)))

    def upload_settings(self, blob: bytes) -> int:
        sid = ctypes.c_uint32()
        check(lib().jsb_settings_upload(self.h, blob, len(blob), ctypes.byref(sid)))
        return sid.value

    def add_body(self, settings_id: int, creation: tuple, position) -> int:
        bid = ctypes.c_uint32()
        check(lib().jsb_body_add(self.h, settings_id, struct.pack(CREATION_FMT, *creation), _f3(position),
                                 ctypes.byref(bid)))
        n = ctypes.c_uint32()
        check(lib().jsb_body_num_vertices(self.h, bid.value, ctypes.byref(n)))
        self.num_vertices.append(n.value)
        return bid.value

    def add_collider(self, type_: int, position, half_extent=(0, 0, 0), radius=0.0, friction=0.2,
                     restitution=0.0) -> int:
        cid = ctypes.c_uint32()
        raw = struct.pack(COLLIDER_FMT, type_, *position, *half_extent, radius, friction, restitution)
        check(lib().jsb_collider_add(self.h, raw, ctypes.byref(cid)))
        return cid.value

    def load_scene(self, scene_bytes: bytes) -> list[dict]:
        """Adds the colliders and bodies of a serialised scene; returns per-body info of the added bodies
        (`self.bodies` lists every body of the context)."""
        b = scene_bytes
        assert b[:4] == b"JSBS"
        _, nb, nc = struct.unpack_from("<III", b, 4)
        g = struct.unpack_from("<3f", b, 16)
        dt, cs, ns = struct.unpack_from("<fii", b, 28)
        self.set_gravity(g)
        self.dt, self.collision_steps, self.scene_steps = dt, cs, ns
        off = 40
        for _ in range(nc):
            v = struct.unpack_from(COLLIDER_FMT, b, off)
            off += 40
            self.add_collider(v[0], v[1:4], v[4:7], v[7], v[8], v[9])
        bodies = []
        for _ in range(nb):
            pos = struct.unpack_from("<3f", b, off)
            cr = struct.unpack_from(CREATION_FMT, b, off + 12)
            force = struct.unpack_from("<3f", b, off + 48)
            (bl,) = struct.unpack_from("<I", b, off + 60)
            blob = b[off + 64: off + 64 + bl]
            off += 64 + bl
            sid = self.upload_settings(blob)
            bid = self.add_body(sid, cr, pos)
            counts = blob_counts(blob)
            bodies.append({"id": bid, "force": force, "iterations": cr[0], "vertices": self.num_vertices[bid],
                           "position": pos, "num_edges": counts["edges"], "num_volumes": counts["volumes"],
                           "num_bends": counts["bends"]})
        self.bodies = self.bodies + bodies
        return bodies

    def set_sleep_settings(self, time_before_sleep: float = 0.5, point_velocity_sleep_threshold: float = 0.03):
        check(lib().jsb_set_sleep_settings(self.h, time_before_sleep, point_velocity_sleep_threshold))

    def is_active(self, body: int) -> bool:
        a = ctypes.c_int()
        check(lib().jsb_body_is_active(self.h, body, ctypes.byref(a)))
        return bool(a.value)

    def set_active(self, body: int, active: bool):
        check(lib().jsb_body_set_active(self.h, body, 1 if active else 0))

    def set_colliding_shapes(self, body: int, shapes: list[bytes] | None):
        """Host-determined colliding shapes of a body (jsb_colliding_shape records, 172 bytes each), or None
        to return it to the context's colliders."""
        if shapes is None:
            check(lib().jsb_body_clear_colliding_shapes(self.h, body))
        else:
            check(lib().jsb_body_set_colliding_shapes(self.h, body, b"".join(shapes), len(shapes)))

    def add_hull(self, points, planes, faces) -> int:
        """Registers a convex hull (ConvexHullShape's points, per-face planes and vertex lists); returns its id."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        pls = np.ascontiguousarray(planes, np.float32).reshape(-1, 4)
        counts = np.array([len(f) for f in faces], np.uint32)
        idx = np.ascontiguousarray(np.concatenate([np.asarray(f, np.uint32) for f in faces]), np.uint32)

        class Hull(ctypes.Structure):
            _fields_ = [("num_points", ctypes.c_uint32), ("points", ctypes.c_void_p), ("num_faces", ctypes.c_uint32),
                        ("planes", ctypes.c_void_p), ("face_vertex_counts", ctypes.c_void_p), ("face_vertices", ctypes.c_void_p)]

        h = Hull(len(pts), pts.ctypes.data, len(pls), pls.ctypes.data, counts.ctypes.data, idx.ctypes.data)
        out = ctypes.c_uint32()
        check(lib().jsb_hull_add(self.h, ctypes.byref(h), ctypes.byref(out)))
        return out.value

    def set_contact_readback(self, enable: bool = True):
        check(lib().jsb_set_contact_readback(self.h, 1 if enable else 0))

    def contacts(self, body: int) -> dict:
        """The body's SoftBodyManifold after the last step: has_contact (N,), contact points (N, 3, local,
        before the recentring), normals (N, 3), shape index (N,), recentring offset (3,)."""
        n = self.num_vertices[body]
        has = np.zeros(n, np.uint8)
        cp = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        shape = np.zeros(n, np.int32)
        delta = np.zeros(3, np.float32)
        check(lib().jsb_body_contacts(self.h, body, has.ctypes.data, cp.ctypes.data, nrm.ctypes.data, shape.ctypes.data,
                                      delta.ctypes.data))
        return {"has_contact": has, "points": cp, "normals": nrm, "shape": shape, "delta": delta}

    def skin_vertices(self, body: int, joint_matrices, hard_skin_all: bool = False):
        """SkinVertices: joint_matrices (J, 4, 4) column-major (Mat44 columns) as float32."""
        m = np.ascontiguousarray(joint_matrices, np.float32)
        check(lib().jsb_body_skin_vertices(self.h, body, m.ctypes.data, m.shape[0], 1 if hard_skin_all else 0))

    def set_skin_settings(self, body: int, enable: bool = True, max_distance_multiplier: float = 1.0):
        check(lib().jsb_body_set_skin_settings(self.h, body, 1 if enable else 0, max_distance_multiplier))

    def sensor_contacts(self, body: int) -> int:
        """Bit k: host-determined shape k is a sensor shape a vertex penetrated in the last step."""
        m = ctypes.c_uint32()
        check(lib().jsb_body_sensor_contacts(self.h, body, ctypes.byref(m)))
        return int(m.value)

    def shape_velocities(self, body: int) -> np.ndarray:
        """Per host-determined shape after the last step: (updated, linear velocity[3], angular velocity[3])."""
        out = np.zeros((16, 7), np.float32)
        n = ctypes.c_uint32()
        check(lib().jsb_body_shape_velocities(self.h, body, out.ctypes.data, ctypes.byref(n)))
        return out[:n.value]

    # -- stepping --------------------------------------------------------------------------------
    def add_force(self, body: int, f):
        check(lib().jsb_body_add_force(self.h, body, _f3(f)))

    def set_step_force(self, body: int, f):
        check(lib().jsb_body_set_step_force(self.h, body, _f3(f)))

    def apply_scene_forces(self):
        """One-shot AddForce of every body's scene force (consumed by the next step)."""
        for b in self.bodies:
            if any(x != 0.0 for x in b["force"]):
                self.add_force(b["id"], b["force"])

    def set_scene_step_forces(self):
        """Scene forces applied before every step (graph-capturable)."""
        for b in self.bodies:
            if any(x != 0.0 for x in b["force"]):
                self.set_step_force(b["id"], b["force"])

    def step(self, dt: float | None = None, collision_steps: int | None = None, stream: int = 0):
        check(lib().jsb_step(self.h, dt or self.dt, collision_steps or self.collision_steps, ctypes.c_void_p(stream)))

    def step_plain(self, dt: float | None = None, collision_steps: int | None = None, stream: int = 0):
        check(lib().jsb_step_plain(self.h, dt or self.dt, collision_steps or self.collision_steps,
                                   ctypes.c_void_p(stream)))

    def step_graph(self, num_steps: int, repeats: int = 1, dt: float | None = None, collision_steps: int | None = None,
                   stream: int = 0):
        check(lib().jsb_step_graph(self.h, dt or self.dt, collision_steps or self.collision_steps, num_steps, repeats,
                                   ctypes.c_void_p(stream)))

    def synchronize(self):
        check(lib().jsb_synchronize(self.h))

    def autotune(self, dt: float | None = None, trials: int = 2):
        check(lib().jsb_autotune(self.h, dt or self.dt, trials))

    def set_bucket_threads(self, max_vertices: int, threads: int):
        check(lib().jsb_set_bucket_threads(self.h, max_vertices, threads))

    def set_bucket_config(self, max_vertices: int, threads: int, state_mode: int):
        check(lib().jsb_set_bucket_config(self.h, max_vertices, threads, state_mode))

    def set_cluster_config(self, cluster_size: int = 0, threads: int = 256):
        """Shape of the thread-block-cluster path (cluster_size 0 = largest that fits)."""
        check(lib().jsb_set_cluster_config(self.h, cluster_size, threads))

    def set_step_walk(self, enable: bool):
        """Whole-step walk for bodies without pressure (default on); off walks every substep separately."""
        check(lib().jsb_set_step_walk(self.h, 1 if enable else 0))

    def cluster_config(self) -> dict:
        c, t, n = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().jsb_get_cluster_config(self.h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(n)))
        return {"cluster_size": c.value, "threads": t.value, "bodies": n.value}

    def bucket_table(self) -> list[tuple[int, int, int]]:
        out, i = [], 0
        while True:
            mv, t, m = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
            if lib().jsb_get_bucket_config(self.h, i, ctypes.byref(mv), ctypes.byref(t), ctypes.byref(m)) != JSB_OK:
                return out
            out.append((mv.value, t.value, m.value))
            i += 1

    # -- readback --------------------------------------------------------------------------------
    def read_body(self, body: int):
        n = self.num_vertices[body]
        pos = np.zeros(3, np.float32)
        loc = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        check(lib().jsb_body_read(self.h, body, pos.ctypes.data, loc.ctypes.data, vel.ctypes.data))
        return pos, loc, vel

    def save_state(self, body: int) -> bytes:
        n = ctypes.c_size_t()
        check(lib().jsb_body_save_state(self.h, body, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        check(lib().jsb_body_save_state(self.h, body, buf, n.value, ctypes.byref(n)))
        return buf.raw

    def restore_state(self, body: int, state: bytes, position):
        check(lib().jsb_body_restore_state(self.h, body, state, len(state), _f3(position)))

    def save_all(self) -> list[tuple[bytes, np.ndarray]]:
        """SaveState bytes and world position of every body."""
        return [(self.save_state(b), self.read_body(b)[0]) for b in range(len(self.num_vertices))]

    def restore_all(self, saved: list[tuple[bytes, np.ndarray]]):
        for b, (state, position) in enumerate(saved):
            self.restore_state(b, state, position)

    def total_vertices(self) -> int:
        t = ctypes.c_uint64()
        check(lib().jsb_total_vertices(self.h, ctypes.byref(t)))
        return t.value

    def schedule_info(self, body: int):
        lv, nc = ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().jsb_body_schedule_info(self.h, body, ctypes.byref(lv), ctypes.byref(nc)))
        return lv.value, nc.value

    def last_launch_count(self) -> int:
        n = ctypes.c_uint32()
        check(lib().jsb_last_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def last_kernel_ms(self) -> float:
        v = ctypes.c_float()
        check(lib().jsb_last_kernel_ms(self.h, ctypes.byref(v)))
        return v.value

    # -- differentiable runs ---------------------------------------------------------------------
    def set_compliance(self, body: int, edge=None, volume=None):
        e = None if edge is None else np.ascontiguousarray(edge, np.float32)
        v = None if volume is None else np.ascontiguousarray(volume, np.float32)
        check(lib().jsb_body_set_compliance(self.h, body, None if e is None else e.ctypes.data, 0 if e is None else len(e),
                                            None if v is None else v.ctypes.data, 0 if v is None else len(v)))

    def adjoint_begin(self, num_steps: int, checkpoint_every: int, dt: float | None = None):
        check(lib().jsb_adjoint_begin(self.h, dt or self.dt, num_steps, checkpoint_every))

    def adjoint_forward(self, until_step: int = -1):
        check(lib().jsb_adjoint_forward(self.h, until_step))

    def adjoint_seed(self, step: int, body: int, dl_dx: np.ndarray):
        a = np.ascontiguousarray(dl_dx, np.float32)
        check(lib().jsb_adjoint_seed(self.h, step, body, a.ctypes.data))

    def body_positions(self) -> np.ndarray:
        """World positions of every body (num_bodies x 3)."""
        out = np.zeros((len(self.num_vertices), 3), np.float32)
        check(lib().jsb_body_positions_all(self.h, out.ctypes.data))
        return out

    def adjoint_seed_all(self, step: int, dl_dx: np.ndarray):
        """d loss / d world positions of every vertex of the context after `step` (total_vertices x 3)."""
        a = np.ascontiguousarray(dl_dx, np.float32)
        check(lib().jsb_adjoint_seed_all(self.h, step, a.ctypes.data))

    def adjoint_gradients_all(self) -> dict:
        n, nb = sum(self.num_vertices), len(self.num_vertices)
        dx = np.zeros((n, 3), np.float32)
        dv = np.zeros((n, 3), np.float32)
        df = np.zeros((nb, 3), np.float32)
        check(lib().jsb_adjoint_gradients_all(self.h, dx.ctypes.data, dv.ctypes.data, df.ctypes.data))
        return {"x0": dx, "v0": dv, "force": df}

    def adjoint_backward(self):
        check(lib().jsb_adjoint_backward(self.h))

    def adjoint_gradients(self, body: int, num_edges: int = 0, num_volumes: int = 0):
        n = self.num_vertices[body]
        dx = np.zeros((n, 3), np.float32)
        dv = np.zeros((n, 3), np.float32)
        df = np.zeros(3, np.float32)
        de = np.zeros(num_edges, np.float32)
        dvol = np.zeros(num_volumes, np.float32)
        check(lib().jsb_adjoint_gradients(self.h, body, dx.ctypes.data, dv.ctypes.data, df.ctypes.data,
                                          de.ctypes.data if num_edges else None, dvol.ctypes.data if num_volumes else None))
        return {"x0": dx, "v0": dv, "force": df, "edge_compliance": de, "volume_compliance": dvol}

    def adjoint_timings(self) -> dict:
        """Device milliseconds of the last differentiable run's forward, taped recomputation and reverse."""
        out = np.zeros(3, np.float32)
        check(lib().jsb_adjoint_timings(self.h, out.ctypes.data))
        return {"forward_ms": float(out[0]), "recompute_ms": float(out[1]), "reverse_ms": float(out[2])}

    def adjoint_bend_gradients(self, body: int, num_bends: int) -> np.ndarray:
        """d loss / d each dihedral bend's compliance (settings order) after adjoint_backward."""
        out = np.zeros(num_bends, np.float32)
        if num_bends:
            check(lib().jsb_adjoint_bend_gradients(self.h, body, out.ctypes.data))
        return out

    def adjoint_end(self):
        check(lib().jsb_adjoint_end(self.h))

    def upload_all(self, positions: np.ndarray, velocities: np.ndarray, stream: int = 0):
        check(lib().jsb_state_upload_all(self.h, ctypes.c_void_p(positions.ctypes.data),
                                         ctypes.c_void_p(velocities.ctypes.data), ctypes.c_void_p(stream)))

    def download_all(self, positions: np.ndarray, velocities: np.ndarray, stream: int = 0):
        check(lib().jsb_state_download_all(self.h, ctypes.c_void_p(positions.ctypes.data),
                                           ctypes.c_void_p(velocities.ctypes.data), ctypes.c_void_p(stream)))
