"""Small scenes that reach the less common branches of World.step: materials
and contact materials, collision filters, kinematic / trigger / response-less
bodies, sleeping and waking, hinge motors, collideConnected = false, quaternion
normalisation modes, AABB broadphase tests, friction gravity, shape offsets,
generic convex hulls, empty and single-body worlds."""
import math

import numpy as np

from cannon_physics_gb300 import _abi as A
from cannon_physics_gb300 import scenes

EDGE_NAMES = ["materials", "filters", "kinematic_trigger", "sleep_wake", "motor", "nocollide", "quat_modes",
              "bbox_naive", "friction_gravity", "shape_offsets", "convex_hulls", "empty", "single", "all_static",
              "sap_y_axis", "grid_spheres", "friction_reduction"]


def _mix(n, seed, spacing=1.1, side=4, kinds=(A.SHAPE_SPHERE, A.SHAPE_BOX, A.SHAPE_CYLINDER)):
    rng = scenes.SplitMix64(seed)
    shapes = A.default_shapes(n + 1)
    bodies = A.default_bodies(n + 1)
    scenes._plane_body(bodies, shapes, 0, 0)
    u = rng.uniform(8 * n).reshape(n, 8)
    for i in range(n):
        k = kinds[i % len(kinds)]
        s = shapes[i + 1]
        s["type"] = k
        if k == A.SHAPE_SPHERE:
            s["radius"] = 0.3 + 0.2 * u[i, 0]
        elif k == A.SHAPE_BOX:
            s["half_extents"] = 0.25 + 0.2 * u[i, :3]
        elif k == A.SHAPE_CYLINDER:
            s["radius_top"] = s["radius_bottom"] = 0.25 + 0.2 * u[i, 0]
            s["height"] = 0.5 + 0.4 * u[i, 1]
            s["num_segments"] = 6 + (i % 3) * 2
        b = bodies[i + 1]
        b["mass"] = 0.5 + u[i, 2]
        b["position"] = ((i % side - side / 2) * spacing + 0.1 * u[i, 3], 0.6 + spacing * (i // (side * side)) + 0.05 * u[i, 4],
                         ((i // side) % side - side / 2) * spacing)
        q = scenes.shoemake(u[i, 5], u[i, 6], u[i, 7])
        b["quaternion"] = q
        b["shape"] = i + 1
    return shapes, bodies


def _tetra_shapes(shapes, idx, with_axes):
    """A ConvexPolyhedron tetrahedron and a square pyramid (faces CCW seen from outside)."""
    verts = []
    for j, i in enumerate(idx):
        if j % 2 == 0:
            v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32) * 0.8 - 0.2
            f = [[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]]
        else:
            v = np.array([[-0.4, -0.3, -0.4], [0.4, -0.3, -0.4], [0.4, -0.3, 0.4], [-0.4, -0.3, 0.4], [0, 0.5, 0]], np.float32)
            f = [[0, 1, 2, 3], [0, 4, 1], [1, 4, 2], [2, 4, 3], [3, 4, 0]]
        sizes = np.array([len(x) for x in f], np.int32)
        flat = np.array([k for x in f for k in x], np.int32)
        verts.append((v, sizes, flat))
        s = shapes[i]
        s["type"] = A.SHAPE_CONVEX
        s["num_vertices"] = len(v)
        s["num_faces"] = len(f)
        s["vertices"] = v.ctypes.data
        s["face_sizes"] = sizes.ctypes.data
        s["face_indices"] = flat.ctypes.data
        s["has_axes"] = 1 if with_axes else 0
        s["num_axes"] = 0
    return verts


def edge_scene(name):
    keep = []
    if name == "materials":
        shapes, bodies = _mix(24, 5)
        mats = np.zeros(3, dtype=A.MATERIAL_DTYPE)
        mats[0] = (0.1, 0.7)
        mats[1] = (-1.0, 0.2)
        mats[2] = (0.6, -1.0)
        bodies["material"][1:] = np.arange(24) % 3
        bodies["material"][0] = 0
        shapes["material"][5] = 2
        shapes["material"][0] = 1
        cms = np.zeros(2, dtype=A.CONTACT_MATERIAL_DTYPE)
        cms[0] = (0, 1, 0.05, 0.9, 1e6, 2.0, 1e7, 3.0)
        cms[1] = (2, 2, 0.8, 0.0, 1e8, 4.0, 1e6, 5.0)
        sc = scenes.Scene(name, shapes, bodies, materials=mats, contact_materials=cms, restitution=0.3)
    elif name == "filters":
        shapes, bodies = _mix(30, 6)
        bodies["collision_filter_group"][1:] = 1 << (np.arange(30) % 3)
        bodies["collision_filter_mask"][1:] = np.where(np.arange(30) % 2 == 0, -1, 1 | 4)
        shapes["collision_filter_group"][7] = 2
        shapes["collision_filter_mask"][9] = 1
        sc = scenes.Scene(name, shapes, bodies)
    elif name == "kinematic_trigger":
        shapes, bodies = _mix(20, 7)
        bodies["type"][3] = A.BODY_KINEMATIC
        bodies["velocity"][3] = (0.5, 0.0, 0.2)
        bodies["angular_velocity"][3] = (0.0, 1.0, 0.0)
        bodies["is_trigger"][5] = 1
        bodies["collision_response"][8] = 0
        shapes["collision_response"][11] = 0
        bodies["type"][12] = A.BODY_KINEMATIC
        sc = scenes.Scene(name, shapes, bodies)
    elif name == "sleep_wake":
        shapes, bodies = _mix(12, 8, side=3)
        bodies["sleep_time_limit"][1:] = 0.2
        bodies["sleep_speed_limit"][1:] = 0.5
        bodies["position"][12] = (0.0, 6.0, 0.0)  # falls later and wakes the pile
        bodies["allow_sleep"][4] = 0
        sc = scenes.Scene(name, shapes, bodies, allow_sleep=True)
    elif name == "motor":
        shapes, bodies = _mix(6, 9, spacing=1.5)
        cons = np.zeros(3, dtype=A.CONSTRAINT_DTYPE)
        for k in range(3):
            c = cons[k]
            c["type"] = A.CON_HINGE
            c["body_a"], c["body_b"] = 1 + 2 * k, 2 + 2 * k
            c["collide_connected"] = 1
            c["motor_enabled"] = 1 if k < 2 else 0
            c["pivot_a"] = (0.75, 0.0, 0.0)
            c["pivot_b"] = (-0.75, 0.0, 0.0)
            c["axis_a"] = (0.0, 0.3, 1.0)
            c["axis_b"] = (0.0, 0.0, 2.0)
            c["max_force"] = 1e6
            c["motor_target_velocity"] = 2.0 - k
            c["motor_max_force"] = 50.0 if k == 0 else 0.0
            c["spook_stiffness"], c["spook_relaxation"], c["spook_time_step"] = 1e7, 4.0, 1 / 60
        sc = scenes.Scene(name, shapes, bodies, constraints=cons)
    elif name == "nocollide":
        shapes, bodies = _mix(8, 10, spacing=0.9)
        cons = np.zeros(4, dtype=A.CONSTRAINT_DTYPE)
        for k in range(4):
            c = cons[k]
            c["type"] = (A.CON_P2P, A.CON_DISTANCE, A.CON_HINGE, A.CON_P2P)[k]
            c["body_a"], c["body_b"] = 1 + k, 2 + k
            c["collide_connected"] = 0 if k != 1 else 1
            c["pivot_a"] = (0.45, 0.0, 0.0)
            c["pivot_b"] = (-0.45, 0.0, 0.0)
            c["axis_a"] = c["axis_b"] = (0.0, 0.0, 1.0)
            c["distance"] = 0.8 if k == 1 else -1.0
            c["max_force"] = 1e6 if k != 3 else 5.0
            c["spook_stiffness"], c["spook_relaxation"], c["spook_time_step"] = 1e7, 4.0, 1 / 60
        sc = scenes.Scene(name, shapes, bodies, constraints=cons)
    elif name == "quat_modes":
        shapes, bodies = _mix(16, 11)
        bodies["angular_velocity"][1:] = (1.0, 2.0, -0.5)
        sc = scenes.Scene(name, shapes, bodies, quat_normalize_fast=True, quat_normalize_skip=2)
    elif name == "bbox_naive":
        shapes, bodies = _mix(20, 12)
        sc = scenes.Scene(name, shapes, bodies, use_bounding_boxes=True)
    elif name == "friction_gravity":
        shapes, bodies = _mix(16, 13)
        sc = scenes.Scene(name, shapes, bodies, friction_gravity=(0.0, -3.0, 0.0))
    elif name == "shape_offsets":
        shapes, bodies = _mix(16, 14)
        bodies["shape_offset"][1:] = (0.1, -0.05, 0.2)
        bodies["shape_orientation"][1:] = scenes.shoemake(np.array([0.3]), np.array([0.6]), np.array([0.1]))[0]
        bodies["fixed_rotation"][6] = 1
        bodies["linear_factor"][7] = (1.0, 0.0, 1.0)
        bodies["angular_factor"][9] = (0.0, 1.0, 0.0)
        sc = scenes.Scene(name, shapes, bodies)
    elif name == "convex_hulls":
        shapes, bodies = _mix(16, 15)
        keep = _tetra_shapes(shapes, list(range(2, 17, 3)), with_axes=True)
        keep += _tetra_shapes(shapes, [3, 7], with_axes=False)
        sc = scenes.Scene(name, shapes, bodies)
    elif name == "empty":
        sc = scenes.Scene(name, A.default_shapes(0), A.default_bodies(0))
    elif name == "single":
        shapes, bodies = _mix(1, 16)
        sc = scenes.Scene(name, shapes[1:], bodies[1:2].copy())
        sc.bodies["shape"] = 0
    elif name == "all_static":
        shapes, bodies = _mix(6, 17)
        bodies["mass"][:] = 0.0
        sc = scenes.Scene(name, shapes, bodies)
    elif name == "sap_y_axis":
        shapes, bodies = _mix(40, 18, side=6)
        sc = scenes.Scene(name, shapes, bodies, broadphase=A.BROAD_SAP, sap_axis=1)
    elif name == "grid_spheres":
        shapes, bodies = _mix(40, 19, side=5, kinds=(A.SHAPE_SPHERE,))
        sc = scenes.Scene(name, shapes, bodies, broadphase=A.BROAD_GRID, grid_n=(7, 9, 6), grid_min=(-4.0, -1.0, -4.0),
                          grid_max=(4.0, 6.0, 4.0))
    elif name == "friction_reduction":
        # Narrowphase.enableFrictionReduction: plane-hull and hull-hull pairs
        # take one averaged friction pair per shape pair; materials put the
        # friction of some pairs at zero
        shapes, bodies = _mix(30, 20, spacing=0.95, side=4)
        keep = _tetra_shapes(shapes, [4, 13], with_axes=True)
        mats = np.zeros(2, dtype=A.MATERIAL_DTYPE)
        mats[0] = (0.0, -1.0)
        mats[1] = (0.5, -1.0)
        bodies["material"][1:] = np.where(np.arange(30) % 7 == 0, 0, 1)
        bodies["material"][0] = 1
        sc = scenes.Scene(name, shapes, bodies, materials=mats, enable_friction_reduction=True)
    else:
        raise KeyError(name)
    sc._keep = keep
    return sc
