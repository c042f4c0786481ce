"""ctypes / numpy mirrors of the structs in include/cannon_gpu.h.

The same layouts are used for the GPU library (libcannon_gpu.so) and for the
test harness; keep them in step with the header.
"""
import ctypes as C

import numpy as np

CP_OK = 0
CP_ERR_ARG = 1
CP_ERR_CAPACITY = 2
CP_ERR_NONFINITE = 3
CP_ERR_TIMEOUT = 4
CP_ERR_OOM = 5
CP_ERR_CUDA = 6
CP_ERR_UNSUPPORTED = 7

SHAPE_SPHERE, SHAPE_PLANE, SHAPE_BOX, SHAPE_CONVEX, SHAPE_CYLINDER = 0, 1, 2, 3, 4
SHAPE_CAPSULE, SHAPE_CONE, SHAPE_SIZED_PLANE = 5, 6, 7
BODY_DYNAMIC, BODY_STATIC, BODY_KINEMATIC = 0, 1, 2
AWAKE, SLEEPY, SLEEPING = 0, 1, 2
BROAD_NAIVE, BROAD_SAP, BROAD_GRID = 0, 1, 2
CON_P2P, CON_HINGE, CON_DISTANCE, CON_LOCK, CON_CONE_TWIST, CON_SPRING = 0, 1, 2, 3, 4, 5
SOLVER_GS, SOLVER_SPLIT = 0, 1
ROW_CONTACT, ROW_FRICTION, ROW_ROTATIONAL, ROW_MOTOR = 0, 1, 2, 3

f3 = C.c_float * 3
f4 = C.c_float * 4
f9 = C.c_float * 9
i3 = C.c_int32 * 3


class ShapeDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("collision_filter_group", C.c_int32),
        ("collision_filter_mask", C.c_int32),
        ("collision_response", C.c_int32),
        ("material", C.c_int32),
        ("num_segments", C.c_int32),
        ("radius", C.c_double),
        ("radius_top", C.c_double),
        ("radius_bottom", C.c_double),
        ("height", C.c_double),
        ("half_extents", f3),
        ("num_vertices", C.c_int32),
        ("num_faces", C.c_int32),
        ("num_axes", C.c_int32),
        ("has_axes", C.c_int32),
        ("vertices", C.c_void_p),
        ("face_sizes", C.c_void_p),
        ("face_indices", C.c_void_p),
        ("axes", C.c_void_p),
        ("bounding_sphere_radius", C.c_double),
    ]


class BodyDesc(C.Structure):
    _fields_ = [
        ("position", f3),
        ("quaternion", f4),
        ("velocity", f3),
        ("angular_velocity", f3),
        ("force", f3),
        ("torque", f3),
        ("linear_factor", f3),
        ("angular_factor", f3),
        ("inv_inertia", f3),
        ("inv_inertia_world", f9),
        ("aabb_lower", f3),
        ("aabb_upper", f3),
        ("shape_offset", f3),
        ("shape_orientation", f4),
        ("previous_position", f3),
        ("previous_quaternion", f4),
        ("mass", C.c_double),
        ("inv_mass", C.c_double),
        ("linear_damping", C.c_double),
        ("angular_damping", C.c_double),
        ("sleep_speed_limit", C.c_double),
        ("sleep_time_limit", C.c_double),
        ("time_last_sleepy", C.c_double),
        ("bounding_radius", C.c_double),
        ("type", C.c_int32),
        ("sleep_state", C.c_int32),
        ("allow_sleep", C.c_int32),
        ("wake_up_after_narrowphase", C.c_int32),
        ("collision_filter_group", C.c_int32),
        ("collision_filter_mask", C.c_int32),
        ("collision_response", C.c_int32),
        ("is_trigger", C.c_int32),
        ("material", C.c_int32),
        ("shape", C.c_int32),
        ("fixed_rotation", C.c_int32),
        ("aabb_needs_update", C.c_int32),
        ("interpolated_position", f3),
        ("interpolated_quaternion", f4),
        ("extra_shapes_first", C.c_int32),
        ("extra_shapes_count", C.c_int32),
    ]


class BodyShape(C.Structure):
    _fields_ = [("shape", C.c_int32), ("offset", f3), ("orientation", f4)]


class BodyState(C.Structure):
    _fields_ = [
        ("position", f3),
        ("quaternion", f4),
        ("velocity", f3),
        ("angular_velocity", f3),
        ("force", f3),
        ("torque", f3),
        ("previous_position", f3),
        ("previous_quaternion", f4),
        ("interpolated_position", f3),
        ("interpolated_quaternion", f4),
        ("sleep_state", C.c_int32),
        ("wake_up_after_narrowphase", C.c_int32),
        ("aabb_needs_update", C.c_int32),
        ("pad0", C.c_int32),
        ("time_last_sleepy", C.c_double),
    ]


class Material(C.Structure):
    _fields_ = [("friction", C.c_double), ("restitution", C.c_double)]


class ContactMaterial(C.Structure):
    _fields_ = [
        ("material_a", C.c_int32),
        ("material_b", C.c_int32),
        ("friction", C.c_double),
        ("restitution", C.c_double),
        ("contact_stiffness", C.c_double),
        ("contact_relaxation", C.c_double),
        ("friction_stiffness", C.c_double),
        ("friction_relaxation", C.c_double),
    ]


class ConstraintDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("body_a", C.c_int32),
        ("body_b", C.c_int32),
        ("collide_connected", C.c_int32),
        ("motor_enabled", C.c_int32),
        ("pad0", C.c_int32),
        ("pivot_a", f3),
        ("pivot_b", f3),
        ("axis_a", f3),
        ("axis_b", f3),
        ("distance", C.c_double),
        ("max_force", C.c_double),
        ("motor_target_velocity", C.c_double),
        ("motor_max_force", C.c_double),
        ("spook_stiffness", C.c_double),
        ("spook_relaxation", C.c_double),
        ("spook_time_step", C.c_double),
        ("lock_axes", (C.c_float * 3) * 6),
        ("angle", C.c_double),
        ("twist_angle", C.c_double),
        ("first_equation_id", C.c_int64),
    ]


class WorldDesc(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_int32),
        ("num_shapes", C.c_int32),
        ("num_materials", C.c_int32),
        ("num_contact_materials", C.c_int32),
        ("num_constraints", C.c_int32),
        ("allow_sleep", C.c_int32),
        ("quat_normalize_skip", C.c_int32),
        ("quat_normalize_fast", C.c_int32),
        ("solver_iterations", C.c_int32),
        ("broadphase", C.c_int32),
        ("use_bounding_boxes", C.c_int32),
        ("sap_axis", C.c_int32),
        ("grid_n", i3),
        ("enable_friction_reduction", C.c_int32),
        ("has_friction_gravity", C.c_int32),
        ("stepnumber", C.c_int32),
        ("solver_tolerance", C.c_double),
        ("time", C.c_double),
        ("gravity", f3),
        ("friction_gravity", f3),
        ("grid_aabb_min", f3),
        ("grid_aabb_max", f3),
        ("bodies", C.c_void_p),
        ("shapes", C.c_void_p),
        ("materials", C.c_void_p),
        ("contact_materials", C.c_void_p),
        ("constraints", C.c_void_p),
        ("sap_axis_list", C.c_void_p),
        ("default_contact_material", ContactMaterial),
        ("body_shapes", C.c_void_p),
        ("num_body_shapes", C.c_int32),
        ("solver", C.c_int32),
        ("equation_id_counter", C.c_int64),
    ]


class Contact(C.Structure):
    _fields_ = [
        ("bi", C.c_int32),
        ("bj", C.c_int32),
        ("si", C.c_int32),
        ("sj", C.c_int32),
        ("ni", f3),
        ("ri", f3),
        ("rj", f3),
        ("enabled", C.c_int32),
        ("pair", C.c_int32),
        ("restitution", C.c_double),
    ]


class Row(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("bi", C.c_int32),
        ("bj", C.c_int32),
        ("pad", C.c_int32),
        ("B", C.c_double),
        ("inv_c", C.c_double),
        ("lambda_", C.c_double),
        ("multiplier", C.c_double),
        ("min_force", C.c_double),
        ("max_force", C.c_double),
        ("eps", C.c_double),
        ("id", C.c_int64),
    ]


class StepInfo(C.Structure):
    _fields_ = [
        ("stepnumber", C.c_int64),
        ("time", C.c_double),
        ("num_pairs", C.c_int32),
        ("num_contacts", C.c_int32),
        ("num_rows", C.c_int32),
        ("iterations", C.c_int32),
        ("status", C.c_int32),
        ("num_bodies", C.c_int32),
        ("num_levels", C.c_int32),
        ("substeps", C.c_int32),
        ("accumulator", C.c_double),
    ]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("block_threads", C.c_int32), ("arena_bytes", C.c_int64)]


_SCALARS = {
    C.c_float: "<f4",
    C.c_double: "<f8",
    C.c_int32: "<i4",
    C.c_int64: "<i8",
    C.c_void_p: "<u8",
}


def np_dtype(struct_cls):
    """numpy structured dtype with the exact ctypes layout of `struct_cls`."""
    names, formats, offsets = [], [], []
    for name, ctype in struct_cls._fields_:
        field = getattr(struct_cls, name)
        names.append(name)
        offsets.append(field.offset)
        if ctype in _SCALARS:
            formats.append(_SCALARS[ctype])
        elif issubclass(ctype, C.Array) and issubclass(ctype._type_, C.Array):  # two-dimensional
            formats.append((_SCALARS[ctype._type_._type_], (ctype._length_, ctype._type_._length_)))
        elif issubclass(ctype, C.Array):
            formats.append((_SCALARS[ctype._type_], (ctype._length_,)))
        elif issubclass(ctype, C.Structure):
            formats.append(np_dtype(ctype))
        else:
            raise TypeError(f"unmapped field {name}: {ctype}")
    return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": C.sizeof(struct_cls)})


class Event(C.Structure):
    _fields_ = [("type", C.c_int32), ("a", C.c_int32), ("b", C.c_int32), ("contact", C.c_int32), ("stepnumber", C.c_int64)]


EV_COLLIDE, EV_BEGIN_CONTACT, EV_END_CONTACT, EV_BEGIN_SHAPE_CONTACT, EV_END_SHAPE_CONTACT = 0, 1, 2, 3, 4


class Ray(C.Structure):
    _fields_ = [("from_", f3), ("to", f3), ("collision_filter_group", C.c_int32), ("collision_filter_mask", C.c_int32),
                ("skip_backfaces", C.c_int32), ("check_collision_response", C.c_int32)]


class RayHit(C.Structure):
    _fields_ = [("has_hit", C.c_int32), ("body", C.c_int32), ("shape", C.c_int32), ("hit_face_index", C.c_int32),
                ("hit_point", f3), ("hit_normal", f3), ("distance", C.c_double)]


RAY_CLOSEST, RAY_ANY, RAY_ALL = 0, 1, 2

SHAPE_DTYPE = np_dtype(ShapeDesc)
EVENT_DTYPE = np_dtype(Event)
RAY_DTYPE = np_dtype(Ray)
RAY_HIT_DTYPE = np_dtype(RayHit)
BODY_DTYPE = np_dtype(BodyDesc)
BODY_STATE_DTYPE = np_dtype(BodyState)
BODY_SHAPE_DTYPE = np_dtype(BodyShape)
MATERIAL_DTYPE = np_dtype(Material)
CONTACT_MATERIAL_DTYPE = np_dtype(ContactMaterial)
CONSTRAINT_DTYPE = np_dtype(ConstraintDesc)
CONTACT_DTYPE = np_dtype(Contact)
ROW_DTYPE = np_dtype(Row)


def ptr(arr):
    """Address of a contiguous numpy array (0 for None / empty)."""
    if arr is None or len(arr) == 0:
        return 0
    assert arr.flags["C_CONTIGUOUS"]
    return arr.ctypes.data


def default_bodies(n):
    """Body descriptors holding the reference Body constructor defaults
    (lib/objects/rigid_body.dart:27-48,118-236)."""
    b = np.zeros(n, dtype=BODY_DTYPE)
    b["quaternion"][:, 3] = 1.0
    b["previous_quaternion"][:, 3] = 1.0
    b["interpolated_quaternion"][:, 3] = 1.0
    b["shape_orientation"][:, 3] = 1.0
    b["linear_factor"] = 1.0
    b["angular_factor"] = 1.0
    b["linear_damping"] = 0.01
    b["angular_damping"] = 0.01
    b["sleep_speed_limit"] = 0.1
    b["sleep_time_limit"] = 1.0
    b["type"] = -1
    b["allow_sleep"] = 1
    b["collision_filter_group"] = 1
    b["collision_filter_mask"] = -1
    b["collision_response"] = 1
    b["material"] = -1
    b["shape"] = -1
    b["aabb_needs_update"] = 1
    return b


def rays(from_, to, group=-1, mask=-1, skip_backfaces=True, check_collision_response=True):
    """Ray records (RayOptions defaults of Ray.intersectWorld) from (n, 3)
    start and end points."""
    from_ = np.asarray(from_, np.float32).reshape(-1, 3)
    r = np.zeros(len(from_), dtype=RAY_DTYPE)
    r["from_"] = from_
    r["to"] = np.asarray(to, np.float32).reshape(-1, 3)
    r["collision_filter_group"] = group
    r["collision_filter_mask"] = mask
    r["skip_backfaces"] = int(skip_backfaces)
    r["check_collision_response"] = int(check_collision_response)
    return r


def body_shapes(n):
    """Extra-shape entries (Body.addShape beyond the first) with identity
    orientations."""
    t = np.zeros(n, dtype=BODY_SHAPE_DTYPE)
    t["orientation"][:, 3] = 1.0
    return t


def default_shapes(n):
    s = np.zeros(n, dtype=SHAPE_DTYPE)
    s["collision_filter_group"] = -1
    s["collision_filter_mask"] = -1
    s["collision_response"] = 1
    s["material"] = -1
    s["radius"] = 1.0
    return s


def default_contact_material(friction=0.3, restitution=0.3):
    """ContactMaterial constructor defaults (contact_material.dart:63-101)."""
    cm = ContactMaterial()
    cm.material_a = -1
    cm.material_b = -1
    cm.friction = friction
    cm.restitution = restitution
    cm.contact_stiffness = 1e7
    cm.contact_relaxation = 3.0
    cm.friction_stiffness = 1e7
    cm.friction_relaxation = 3.0
    return cm
