"""Body shards for multi-GPU runs: one process per GPU, each stepping its own subset of the bodies.

Soft bodies do not interact within a step (the reference has no soft-soft collision,
SoftBodyMotionProperties.cpp:147), so a batch splits across GPUs with no exchange on the data path.
Bodies are assigned longest-processing-time first onto the least-loaded rank, by an estimated cost:
iterations x (dependency levels per substep + vertices / 32), the critical path of one body's step
on one CTA. `shard_scene` cuts a serialised scene ("JSBS", see tests/scenes/scene_io.h) down to one
rank's bodies (every rank keeps every collider).
"""
from __future__ import annotations

import heapq
import struct

from . import settings_schedule

_HEADER = 40   # 'JSBS', version, num_bodies, num_colliders, gravity[3], dt, collision_steps, num_steps
_COLLIDER = 40
_BODY_FIXED = 64  # position[3], creation (36 bytes), force[3], blob length


def _bodies(scene: bytes):
    if scene[:4] != b"JSBS":
        raise ValueError("not a serialised scene")
    _, nb, nc = struct.unpack_from("<III", scene, 4)
    off = _HEADER + nc * _COLLIDER
    out = []
    for _ in range(nb):
        (blob_len,) = struct.unpack_from("<I", scene, off + 60)
        (iterations,) = struct.unpack_from("<I", scene, off + 12)
        out.append((off, _BODY_FIXED + blob_len, iterations, scene[off + _BODY_FIXED: off + _BODY_FIXED + blob_len]))
        off += _BODY_FIXED + blob_len
    return nb, nc, out


def body_costs(scene: bytes) -> list[float]:
    """Estimated step cost of every body of a serialised scene (arbitrary units)."""
    _, _, bodies = _bodies(scene)
    costs = []
    for _, _, iterations, blob in bodies:
        levels, _, _ = settings_schedule(blob)
        (num_vertices,) = struct.unpack_from("<I", blob, 0)
        costs.append(float(iterations) * (len(levels) - 2 + num_vertices / 32.0))
    return costs


def assign_shards(costs: list[float], world: int) -> list[list[int]]:
    """Longest-processing-time-first assignment: body indices per rank, each list ascending."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in shards]


def shard_scene(scene: bytes, rank: int, world: int) -> tuple[bytes, list[int]]:
    """The scene restricted to `rank`'s bodies, and their indices in the full scene."""
    nb, nc, bodies = _bodies(scene)
    mine = assign_shards(body_costs(scene), world)[rank]
    head = bytearray(scene[:_HEADER + nc * _COLLIDER])
    struct.pack_into("<I", head, 8, len(mine))
    parts = [bytes(head)] + [scene[bodies[i][0]: bodies[i][0] + bodies[i][1]] for i in mine]
    return b"".join(parts), mine
