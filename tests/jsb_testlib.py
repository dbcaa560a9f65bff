"""Test helpers: scene/dump parsing and the CPU oracle binding.

The oracle (oracle/liboracle.so) is test infrastructure: these helpers are the only code that loads it,
and they are imported only by tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
from dataclasses import dataclass, field

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_DRIVER = {v: os.path.join(ORACLE_DIR, "_ref", v, "ref_driver") for v in ("det", "fast")}

CREATION_FMT = "<I7f4B"  # jsb_creation_settings, 36 bytes
COLLIDER_FMT = "<i3f3f3f"  # type, position, half_extent, radius, friction, restitution (40 bytes)


@dataclass
class Collider:
    type: int
    position: tuple
    half_extent: tuple
    radius: float
    friction: float
    restitution: float

    def pack(self) -> bytes:
        return struct.pack(COLLIDER_FMT, self.type, *self.position, *self.half_extent, self.radius, self.friction,
                           self.restitution)


@dataclass
class Body:
    position: tuple
    creation: tuple  # (num_iterations, damping, max_v, restitution, friction, pressure, gravity_factor, radius, 4 flags)
    force: tuple
    blob: bytes
    num_vertices: int = 0

    @property
    def num_iterations(self) -> int:
        return int(self.creation[0])

    def creation_bytes(self) -> bytes:
        return struct.pack(CREATION_FMT, *self.creation)


@dataclass
class Scene:
    gravity: tuple
    dt: float
    collision_steps: int
    num_steps: int
    colliders: list = field(default_factory=list)
    bodies: list = field(default_factory=list)
    raw: bytes = b""


def blob_num_vertices(blob: bytes) -> int:
    return struct.unpack_from("<I", blob, 0)[0]


def parse_scene(buf: bytes, off: int = 0) -> tuple[Scene, int]:
    assert buf[off:off + 4] == b"JSBS", "not a scene"
    start = off
    _, nb, nc = struct.unpack_from("<III", buf, off + 4)
    off += 16
    g = struct.unpack_from("<3f", buf, off)
    dt, cs, ns = struct.unpack_from("<fii", buf, off + 12)
    off += 24
    sc = Scene(gravity=g, dt=dt, collision_steps=cs, num_steps=ns)
    for _ in range(nc):
        v = struct.unpack_from(COLLIDER_FMT, buf, off)
        off += 40
        sc.colliders.append(Collider(v[0], v[1:4], v[4:7], v[7], v[8], v[9]))
    for _ in range(nb):
        pos = struct.unpack_from("<3f", buf, off)
        off += 12
        cr = struct.unpack_from(CREATION_FMT, buf, off)
        off += 36
        force = struct.unpack_from("<3f", buf, off)
        off += 12
        (bl,) = struct.unpack_from("<I", buf, off)
        off += 4
        blob = bytes(buf[off:off + bl])
        off += bl
        sc.bodies.append(Body(pos, cr, force, blob, blob_num_vertices(blob)))
    sc.raw = bytes(buf[start:off])
    return sc, off


def rewrite_scene_blobs(buf: bytes, rewrite) -> bytes:
    """The scene bytes with every body's settings blob replaced by rewrite(blob)."""
    assert buf[:4] == b"JSBS", "not a scene"
    _, nb, nc = struct.unpack_from("<III", buf, 4)
    off = 40 + 40 * nc
    out = bytearray(buf[:off])
    for _ in range(nb):
        (bl,) = struct.unpack_from("<I", buf, off + 60)
        blob = rewrite(bytes(buf[off + 64:off + 64 + bl]))
        out += buf[off:off + 60] + struct.pack("<I", len(blob)) + blob
        off += 64 + bl
    return bytes(out)


@dataclass
class Dump:
    step: int
    positions: list  # per body: body position (3,)
    local: list  # per body: (N, 3)
    velocities: list  # per body: (N, 3)
    states: list  # per body: SaveState bytes

    def world(self, b: int) -> np.ndarray:
        return self.local[b].astype(np.float64) + np.asarray(self.positions[b], np.float64)


def parse_dump(path: str) -> tuple[Scene, list]:
    buf = open(path, "rb").read()
    assert buf[:4] == b"JSBD"
    ver, nd, sl = struct.unpack_from("<III", buf, 4)
    assert ver == 2
    scene, off = parse_scene(buf, 16)
    dumps = []
    for _ in range(nd):
        (step,) = struct.unpack_from("<i", buf, off)
        off += 4
        d = Dump(step, [], [], [], [])
        for b in scene.bodies:
            n = b.num_vertices
            d.positions.append(np.frombuffer(buf, np.float32, 3, off).copy())
            off += 12
            d.local.append(np.frombuffer(buf, np.float32, 3 * n, off).reshape(n, 3).copy())
            off += 12 * n
            d.velocities.append(np.frombuffer(buf, np.float32, 3 * n, off).reshape(n, 3).copy())
            off += 12 * n
            (stl,) = struct.unpack_from("<I", buf, off)
            off += 4
            d.states.append(bytes(buf[off:off + stl]))
            off += stl
        dumps.append(d)
    return scene, dumps


def state_digest(position, local, velocity) -> bytes:
    """16-byte digest of one body's state (float32 body position, local positions and velocities) in which
    every NaN is replaced by the same quiet NaN, so that states agreeing bit for bit except in the payload
    and sign of their NaNs (the CPU's default NaN differs from the GPU's) give the same digest."""
    import hashlib

    h = hashlib.sha256()
    for a in (position, local, velocity):
        a = np.array(a, np.float32, copy=True).reshape(-1)
        a[np.isnan(a)] = np.float32(np.nan)
        h.update(a.tobytes())
    return h.digest()[:16]


def run_reference(variant: str, scene: str, out: str, **kv) -> dict:
    """Runs the reference driver (only where oracle/_ref was built)."""
    args = [REF_DRIVER[variant], scene, out] + [f"{k}={v}" for k, v in kv.items()]
    res = subprocess.run(args, check=True, capture_output=True, text=True)
    import json
    return json.loads(res.stdout.strip().splitlines()[-1])


# jsb_colliding_shape (include/jsb.h): type, motion type, transform[12], half_extent[3], radius, friction,
# restitution, soft-body inverse-mass scale, inverse mass, inverse inertia[12], centre of mass[3], linear
# velocity[3], angular velocity[3], hull id
SHAPE_FMT = "<2i41fI"  # (+ hull id)
SHAPE_BYTES = struct.calcsize(SHAPE_FMT)
_TABLE_ENTRY = "<2I2i16f3f3f2f16f16f3f3f3f3f"  # oracle/ref_driver.cpp TableEntry


def parse_tables(path: str, num_soft: int = 0) -> dict:
    """The reference driver's tables file: {"steps": {step: [(soft body, rigid index, shape bytes
    (SHAPE_FMT; a hull's id field holds its rigid index), rigid linear and angular velocity (world) when
    collected)]}, "rigid_after": (steps, num_rigid, 6) velocities after each step, "hulls": {rigid index:
    (points (N, 3), planes (F, 4), [face vertex lists])}, "manifolds": {(step, soft body): per vertex
    (has, point, normal, rigid)} (version 3; num_soft: the scene's soft bodies), "sensors": {(step, soft
    body): rigid indices of the manifold's sensor contacts} (version 4)}."""
    buf = open(path, "rb").read()
    assert buf[:4] == b"JSBT"
    version, steps, nr = struct.unpack_from("<III", buf, 4)
    off, esz = 16, struct.calcsize(_TABLE_ENTRY)
    hulls = {}
    if version >= 2:
        for r in range(nr):
            (npts,) = struct.unpack_from("<I", buf, off)
            off += 4
            pts = np.frombuffer(buf, np.float32, 3 * npts, off).reshape(npts, 3).copy()
            off += 12 * npts
            (nf,) = struct.unpack_from("<I", buf, off)
            off += 4
            planes, faces = [], []
            for _ in range(nf):
                planes.append(np.frombuffer(buf, np.float32, 4, off).copy())
                (cnt,) = struct.unpack_from("<I", buf, off + 16)
                faces.append(list(struct.unpack_from(f"<{cnt}I", buf, off + 20)))
                off += 20 + 4 * cnt
            if npts:
                hulls[r] = (pts, np.array(planes, np.float32).reshape(nf, 4), faces)
    out, after, manifolds, sensors = {}, np.zeros((steps, nr, 6), np.float32), {}, {}
    for k in range(steps):
        st, n = struct.unpack_from("<iI", buf, off)
        off += 8
        rows = []
        for _ in range(n):
            v = struct.unpack_from(_TABLE_ENTRY, buf, off)
            off += esz
            sb, rg, ty, mo = v[0:4]
            leaf = np.array(v[4:20], np.float32).reshape(4, 4)  # columns
            he, rad, fr, rs = v[20:23], v[23], v[24], v[25]
            isc, im = v[26], v[27]
            inert = np.array(v[28:44], np.float32).reshape(4, 4)
            com = np.array(v[44:60], np.float32).reshape(4, 4)
            lin, ang, lw, aw = v[60:63], v[63:66], v[66:69], v[69:72]
            shape = struct.pack(SHAPE_FMT, ty, mo, *leaf[:, :3].ravel(), *he, rad, fr, rs, isc, im, *inert[:, :3].ravel(),
                                *com[3, :3], *lin, *ang, rg if ty == 4 else 0)
            rows.append((sb, rg, shape, np.array(lw + aw, np.float32)))
        out[st] = rows
        after[k] = np.frombuffer(buf, np.float32, 6 * nr, off).reshape(nr, 6)
        off += 24 * nr
        if version >= 3:  # per soft body: the SoftBodyManifold of OnSoftBodyContactAdded, if it was called
            for b in range(num_soft):
                (n,) = struct.unpack_from("<I", buf, off)
                off += 4
                if n:
                    rec = np.frombuffer(buf, np.dtype([("has", "<u4"), ("point", "<f4", 3), ("normal", "<f4", 3), ("rigid", "<i4")]),
                                        n, off)
                    manifolds[(st, b)] = rec.copy()
                    off += 32 * n
                if version >= 4:  # the manifold's sensor contacts (rigid indices)
                    (ns,) = struct.unpack_from("<I", buf, off)
                    off += 4
                    if ns:
                        sensors[(st, b)] = list(struct.unpack_from(f"<{ns}i", buf, off))
                        off += 4 * ns
    return {"steps": out, "rigid_after": after, "hulls": hulls, "manifolds": manifolds, "sensors": sensors}


def build_oracle() -> str:
    """oracle/build.py's build_oracle (compiles liboracle.so when it is missing or stale)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(ORACLE_DIR, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_oracle()


class Oracle:
    """ctypes wrapper of the CPU oracle (float = bitwise restatement of the reference; double = FP64)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            build_oracle()
            L = ctypes.CDLL(ORACLE_LIB)
            L.oracle_world_create.restype = ctypes.c_void_p
            L.oracle_world_create.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int]
            L.oracle_world_destroy.argtypes = [ctypes.c_void_p]
            L.oracle_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_add_collider.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_float,
                                              ctypes.c_float]
            L.oracle_add_body.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
            L.oracle_set_force.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
            L.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_int]
            L.oracle_num_vertices.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_get_body.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]
            L.oracle_get_world_positions_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_set_state_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_set_state.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_set_compliance_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                    ctypes.c_void_p, ctypes.c_int]
            L.oracle_set_force_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_get_world_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_body_active.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_body_sleep_timer.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_body_sleep_timer.restype = ctypes.c_float
            L.oracle_set_sleep_settings.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float]
            L.oracle_set_freeze.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_copy_decisions.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_set_noise.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64]
            L.oracle_set_colliding_shapes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
            L.oracle_get_shape_velocities.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_add_hull.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_set_contact_readback.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.oracle_get_contacts.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_get_sensor_contacts.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
            L.oracle_skin_vertices.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
            L.oracle_set_skin_settings.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float]
            L.oracle_get_skin_state.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.oracle_last_error.restype = ctypes.c_char_p
            L.oracle_last_error.argtypes = [ctypes.c_void_p]
            cls._lib = L
        return cls._lib

    def __init__(self, scene: Scene, use_double: bool = False, threads: int = 1):
        L = self.lib()
        self.scene = scene
        g = (ctypes.c_float * 3)(*scene.gravity)
        self.h = L.oracle_world_create(g, int(use_double))
        L.oracle_set_threads(self.h, int(threads))
        for c in scene.colliders:
            L.oracle_add_collider(self.h, c.type, (ctypes.c_float * 3)(*c.position),
                                  (ctypes.c_float * 3)(*c.half_extent), c.radius, c.friction, c.restitution)
        self.nv = []
        for b in scene.bodies:
            cr = b.creation
            creation = (ctypes.c_float * 10)(cr[0], cr[1], cr[2], cr[3], cr[4], cr[5], cr[6], cr[7], cr[8], cr[10])
            idx = L.oracle_add_body(self.h, b.blob, len(b.blob), (ctypes.c_float * 3)(*b.position), creation)
            if idx < 0:
                raise RuntimeError(L.oracle_last_error(self.h).decode())
            self.nv.append(L.oracle_num_vertices(self.h, idx))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().oracle_world_destroy(self.h)
            self.h = None

    def step(self, n: int = 1):
        L = self.lib()
        for _ in range(n):
            for i, b in enumerate(self.scene.bodies):
                if any(f != 0.0 for f in b.force):
                    L.oracle_set_force(self.h, i, (ctypes.c_float * 3)(*b.force))
            L.oracle_step(self.h, self.scene.dt, self.scene.collision_steps)

    def set_colliding_shapes(self, i: int, shapes: list[bytes] | None):
        """Host-determined colliding shapes of body i for the following steps (SHAPE_FMT records); None
        returns the body to the scene's colliders."""
        data = b"".join(shapes or [])
        self.lib().oracle_set_colliding_shapes(self.h, i, data, -1 if shapes is None else len(shapes))

    def add_hull(self, points, planes, faces) -> int:
        """Registers a convex hull (points (N, 3), planes (F, 4), face vertex lists); returns its index."""
        pts = np.ascontiguousarray(points, np.float32)
        pls = np.ascontiguousarray(planes, np.float32)
        counts = np.array([len(f) for f in faces], np.uint32)
        idx = np.ascontiguousarray(np.concatenate([np.asarray(f, np.uint32) for f in faces]), np.uint32)
        return self.lib().oracle_add_hull(self.h, pts.ctypes.data, len(pts), pls.ctypes.data, len(pls), counts.ctypes.data,
                                          idx.ctypes.data)

    def set_contact_readback(self, on: bool = True):
        self.lib().oracle_set_contact_readback(self.h, 1 if on else 0)

    def contacts(self, i: int) -> np.ndarray:
        """The last step's manifold of body i: (N, 8) {has contact, point xyz, normal xyz, shape index}."""
        out = np.zeros((self.nv[i], 8), np.float32)
        n = self.lib().oracle_get_contacts(self.h, i, out.ctypes.data)
        return out[:n]

    def skin_vertices(self, i: int, joints, hard: bool = False):
        """SkinVertices of body i; joints (J, 16) float32, Mat44 columns."""
        j = np.ascontiguousarray(joints, np.float32)
        assert self.lib().oracle_skin_vertices(self.h, i, j.ctypes.data, j.shape[0], 1 if hard else 0) == 0

    def set_skin_settings(self, i: int, enable: bool, multiplier: float):
        self.lib().oracle_set_skin_settings(self.h, i, 1 if enable else 0, multiplier)

    def skin_state(self, i: int) -> np.ndarray:
        """(N, 3, 3): per vertex previous skinned position, skinned position, normal."""
        out = np.zeros((self.nv[i], 9), np.float32)
        n = self.lib().oracle_get_skin_state(self.h, i, out.ctypes.data)
        return out[:n].reshape(n, 3, 3)

    def sensor_contacts(self, i: int) -> int:
        """After a step with host-determined shapes: bit k = shape k is a sensor shape a vertex penetrated."""
        m = ctypes.c_uint32()
        self.lib().oracle_get_sensor_contacts(self.h, i, ctypes.byref(m))
        return int(m.value)

    def shape_velocities(self, i: int) -> np.ndarray:
        """After a step with host-determined shapes: per shape (updated, linear velocity, angular velocity)."""
        out = np.zeros((16, 7), np.float32)
        n = self.lib().oracle_get_shape_velocities(self.h, i, out.ctypes.data)
        return out[:n]

    def active(self, i: int) -> bool:
        return bool(self.lib().oracle_body_active(self.h, i))

    def sleep_timer(self, i: int) -> float:
        return float(self.lib().oracle_body_sleep_timer(self.h, i))

    def set_state(self, i: int, local_positions, velocities):
        """Local positions and velocities (N, 3) of body i (float world)."""
        p = np.ascontiguousarray(local_positions, np.float32)
        v = np.ascontiguousarray(velocities, np.float32)
        self.lib().oracle_set_state(self.h, i, p.ctypes.data, v.ctypes.data)

    def body(self, i: int):
        n = self.nv[i]
        pos = np.zeros(3, np.float32)
        loc = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        self.lib().oracle_get_body(self.h, i, pos.ctypes.data, loc.ctypes.data, vel.ctypes.data)
        return pos, loc, vel

    def world_f64(self, i: int) -> np.ndarray:
        out = np.zeros((self.nv[i], 3), np.float64)
        self.lib().oracle_get_world_positions_f64(self.h, i, out.ctypes.data)
        return out


def blob_arrays(blob: bytes):
    """Initial local positions, velocities (N, 3) and inverse masses (N,) of a settings blob."""
    n = struct.unpack_from("<I", blob, 0)[0]
    v = np.frombuffer(blob, np.float32, 7 * n, 4).reshape(n, 7)
    return v[:, 0:3].astype(np.float64), v[:, 3:6].astype(np.float64), v[:, 6].copy()


def blob_compliance(blob: bytes):
    """Edge and volume compliance arrays (settings order) of a settings blob."""
    off, out = 0, {}
    for name, size in [("v", 28), ("f", 16), ("e", 16), ("b", 24), ("vol", 24)]:
        (n,) = struct.unpack_from("<I", blob, off)
        out[name] = (off + 4, n)
        off += 4 + n * size
    eo, en = out["e"]
    vo, vn = out["vol"]
    edges = np.frombuffer(blob, np.float32, 4 * en, eo).reshape(en, 4)[:, 3].astype(np.float64) if en else np.zeros(0)
    vols = np.frombuffer(blob, np.float32, 6 * vn, vo).reshape(vn, 6)[:, 5].astype(np.float64) if vn else np.zeros(0)
    return edges, vols


def blob_bend_compliance(blob: bytes) -> np.ndarray:
    """Dihedral bend compliance array (settings order) of a settings blob."""
    off = 0
    for size in (28, 16, 16):  # vertices, faces, edges
        (n,) = struct.unpack_from("<I", blob, off)
        off += 4 + n * size
    (nb,) = struct.unpack_from("<I", blob, off)
    return np.frombuffer(blob, np.float32, 6 * nb, off + 4).reshape(nb, 6)[:, 4].astype(np.float64) if nb else np.zeros(0)


class FD64:
    """Linear functionals of the FP64 oracle trajectory, for central finite differences.

    loss(params) = sum over (step, body) seeds of seed . world positions after that step, with optional
    per-body overrides of initial local positions "x0", velocities "v0", edge / volume compliance and a
    step force "force" (added before every step, like the scene forces)."""

    def __init__(self, scene: Scene, seeds: dict, steps: int):
        self.scene, self.seeds, self.steps = scene, seeds, steps

    def loss(self, overrides: dict | None = None, record: list | None = None, replay=None) -> float:
        """record: a list receiving the run's oracle with its collision decisions recorded; replay: such an
        oracle, whose decisions this run replays (the collision active set frozen, as the adjoint has it)."""
        overrides = overrides or {}
        L = Oracle.lib()
        o = Oracle(self.scene, use_double=True)
        if record is not None:
            L.oracle_set_freeze(o.h, 1)
            record.append(o)
        elif replay is not None:
            L.oracle_copy_decisions(o.h, replay.h)
            L.oracle_set_freeze(o.h, 2)
        forces = {}
        for b, body in enumerate(self.scene.bodies):
            ov = overrides.get(b, {})
            x0, v0, _ = blob_arrays(body.blob)
            x0 = np.ascontiguousarray(ov.get("x0", x0), np.float64)
            v0 = np.ascontiguousarray(ov.get("v0", v0), np.float64)
            L.oracle_set_state_f64(o.h, b, x0.ctypes.data, v0.ctypes.data)
            ec, vc = blob_compliance(body.blob)
            ec = np.ascontiguousarray(ov.get("edge", ec), np.float64)
            vc = np.ascontiguousarray(ov.get("volume", vc), np.float64)
            L.oracle_set_compliance_f64(o.h, b, ec.ctypes.data, len(ec), vc.ctypes.data, len(vc))
            forces[b] = np.ascontiguousarray(ov.get("force", np.asarray(body.force, np.float64)), np.float64)
        total = 0.0
        for step in range(1, self.steps + 1):
            for b, f in forces.items():
                if np.any(f != 0.0):
                    L.oracle_set_force_f64(o.h, b, f.ctypes.data)
            L.oracle_step(o.h, self.scene.dt, self.scene.collision_steps)
            for b, r in self.seeds.get(step, {}).items():
                w = np.zeros((self.scene.bodies[b].num_vertices, 3), np.float64)
                L.oracle_get_world_f64(o.h, b, w.ctypes.data)
                total += float((np.asarray(r, np.float64) * w).sum())
        return total

    def record_f32(self):
        """Float run of the base parameters with every collision decision recorded: the GPU's own decisions
        (the float oracle is bitwise equal to the GPU)."""
        o = Oracle(self.scene)
        Oracle.lib().oracle_set_freeze(o.h, 1)
        o.step(self.steps)
        return o

    def central(self, body: int, kind: str, index: tuple, eps: float, frozen: bool = False) -> float:
        """Central difference of the loss in one parameter component; frozen: the perturbed runs replay the
        collision decisions (planes, contacts, friction clamps, restitution, velocity clamp) of the base
        parameters' float run, i.e. of the GPU's run."""
        base = self.base_params(body)[kind]
        rec = self.record_f32() if frozen else None
        vals = []
        for sgn in (1.0, -1.0):
            p = base.copy()
            p[index] += sgn * eps
            vals.append(self.loss({body: {kind: p}}, replay=rec))
        return (vals[0] - vals[1]) / (2.0 * eps)

    def base_params(self, body: int) -> dict:
        b = self.scene.bodies[body]
        x0, v0, _ = blob_arrays(b.blob)
        ec, vc = blob_compliance(b.blob)
        return {"x0": x0, "v0": v0, "edge": ec, "volume": vc, "force": np.asarray(b.force, np.float64)}


def single_body_scene(scene: Scene, b: int) -> Scene:
    """The scene reduced to body b (every collider kept): bodies do not interact within a step."""
    return Scene(gravity=scene.gravity, dt=scene.dt, collision_steps=scene.collision_steps, num_steps=scene.num_steps,
                 colliders=list(scene.colliders), bodies=[scene.bodies[b]])


def run64(scene: Scene, b: int, steps: int, observe, x0=None, v0=None, edge=None, volume=None, force=None,
          record=None, replay=None, noise=0.0) -> dict:
    """FP64 oracle run of body b alone (optionally with its initial local positions / velocities, edge /
    volume compliance or step force replaced); world positions (N, 3) after each step in `observe`.
    record: a list that receives the run's oracle with every collision decision recorded; replay: such an
    oracle, whose decisions this run takes instead of deciding again (the collision active set frozen,
    as the adjoint differentiates it). noise: relative size of a fixed perturbation of the state after every
    step (the same in every run), a probe of how much the gradient depends on the trajectory."""
    sc = single_body_scene(scene, b)
    body = sc.bodies[0]
    L = Oracle.lib()
    o = Oracle(sc, use_double=True)
    if noise:
        L.oracle_set_noise(o.h, float(noise), 12345)
    if record is not None:
        L.oracle_set_freeze(o.h, 1)
        record.append(o)
    elif replay is not None:
        L.oracle_copy_decisions(o.h, replay.h)
        L.oracle_set_freeze(o.h, 2)
    bx0, bv0, _ = blob_arrays(body.blob)
    ec, vc = blob_compliance(body.blob)
    xx = np.ascontiguousarray(bx0 if x0 is None else x0, np.float64)
    vv = np.ascontiguousarray(bv0 if v0 is None else v0, np.float64)
    L.oracle_set_state_f64(o.h, 0, xx.ctypes.data, vv.ctypes.data)
    ee = np.ascontiguousarray(ec if edge is None else edge, np.float64)
    vo = np.ascontiguousarray(vc if volume is None else volume, np.float64)
    L.oracle_set_compliance_f64(o.h, 0, ee.ctypes.data, len(ee), vo.ctypes.data, len(vo))
    f = np.ascontiguousarray(np.asarray(body.force, np.float64) if force is None else force, np.float64)
    out = {}
    n = body.num_vertices
    for s in range(1, steps + 1):
        if np.any(f != 0.0):
            L.oracle_set_force_f64(o.h, 0, f.ctypes.data)
        L.oracle_step(o.h, sc.dt, sc.collision_steps)
        if s in observe:
            w = np.zeros((n, 3), np.float64)
            L.oracle_get_world_f64(o.h, 0, w.ctypes.data)
            out[s] = w
    return out


def record32(scene: Scene, b: int, steps: int):
    """Float oracle run of body b alone over `steps` steps with its scene force, recording every collision
    decision: the decisions of the GPU's own (bitwise equal) run, for FP64 runs to replay."""
    sc = single_body_scene(scene, b)
    L = Oracle.lib()
    o = Oracle(sc)
    L.oracle_set_freeze(o.h, 1)
    o.step(steps)
    return o


def blob_counts_py(blob: bytes) -> dict:
    """Element counts of a SaveBinaryState blob (vertices, faces, edges, bends, volumes, skinned, ..., lra)."""
    out, off = {}, 0
    for name, size in [("vertices", 28), ("faces", 16), ("edges", 16), ("bends", 24), ("volumes", 24), ("skinned", 52),
                       ("skinned_normals", 4), ("lra", 12)]:
        (n,) = struct.unpack_from("<I", blob, off)
        out[name] = n
        off += 4 + n * size
    return out
