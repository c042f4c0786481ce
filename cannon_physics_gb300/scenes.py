"""Seeded synthetic scenes for the World.step workloads.

The reference publishes no benchmark scenes, so these stand in for them with
the shapes, sizes and value distributions of the five workloads:

  spheres_on_plane   64 Sphere(0.5) dropped on a Plane, NaiveBroadphase, 10 iterations
  box_pile           4096 random boxes piled on a Plane, SAPBroadphase(x), 20 iterations
  mixed_chains       8192 spheres/boxes/cylinders, 128 chains of 16 joined by
                     PointToPoint/Hinge/Distance, GridBroadphase(cell 1.0), sleeping
  batch_worlds       4096 worlds of log-uniform 8..512 spheres/boxes, Naive, 10 iterations
  serve_requests     Poisson arrivals of worlds with 16..4096 bodies and horizons 1..240

Random numbers come from SplitMix64 (53-bit uniform doubles) and random unit
quaternions from Shoemake's method, so every scene is reproducible from its
seed.  Bodies are built the way the reference builds them:
Body(mass, position, quaternion) then addShape, so inertia comes from the
rotated AABB (lib/objects/rigid_body.dart:587-609).
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """SplitMix64 stream; `uniform(n)` returns n doubles in [0, 1)."""

    def __init__(self, seed):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def next_u64(self, n):
        with np.errstate(over="ignore"):
            k = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + k * _GAMMA
            self.state = self.state + np.uint64(n) * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n):
        return (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def shoemake(u1, u2, u3):
    """Uniform random unit quaternions (x, y, z, w) from three uniforms."""
    a = np.sqrt(1.0 - u1)
    b = np.sqrt(u1)
    t2 = 2.0 * math.pi * u2
    t3 = 2.0 * math.pi * u3
    return np.stack([a * np.sin(t2), a * np.cos(t2), b * np.sin(t3), b * np.cos(t3)], axis=-1)


def euler_xyz(x, y, z):
    """Quaternion.setFromEuler(x, y, z, Order.xyz) (lib/math/quaternion.dart:358-370)."""
    c1, c2, c3 = math.cos(x / 2), math.cos(y / 2), math.cos(z / 2)
    s1, s2, s3 = math.sin(x / 2), math.sin(y / 2), math.sin(z / 2)
    return (s1 * c2 * c3 + c1 * s2 * s3, c1 * s2 * c3 - s1 * c2 * s3, c1 * c2 * s3 + s1 * s2 * c3, c1 * c2 * c3 - s1 * s2 * s3)


@dataclass
class Scene:
    """A World descriptor held as numpy arrays (layouts of include/cannon_gpu.h)."""

    name: str
    shapes: np.ndarray
    bodies: np.ndarray
    gravity: tuple = (0.0, -9.82, 0.0)
    materials: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=A.MATERIAL_DTYPE))
    contact_materials: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=A.CONTACT_MATERIAL_DTYPE))
    constraints: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=A.CONSTRAINT_DTYPE))
    friction: float = 0.3
    restitution: float = 0.0
    iterations: int = 10
    tolerance: float = 1e-7
    broadphase: int = A.BROAD_NAIVE
    sap_axis: int = 0
    grid_n: tuple = (10, 10, 10)
    grid_min: tuple = (0.0, 0.0, 0.0)
    grid_max: tuple = (1.0, 1.0, 1.0)
    allow_sleep: bool = False
    dt: float = 1.0 / 60.0
    steps: int = 1
    quat_normalize_skip: int = 0
    quat_normalize_fast: bool = False
    use_bounding_boxes: bool = False
    enable_friction_reduction: bool = False
    time: float = 0.0
    stepnumber: int = 0
    friction_gravity: tuple = None
    solver: int = A.SOLVER_GS
    equation_id_counter: int = 0  # SPLIT: Equation.idCounter when the world is handed over
    # the extra shapes of compound bodies (bodies' extra_shapes_first / _count index it)
    body_shapes: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=A.BODY_SHAPE_DTYPE))
    _keep: list = field(default_factory=list)

    @property
    def num_bodies(self):
        return len(self.bodies)

    def world_desc(self):
        """cp_world_desc pointing at this scene's arrays (kept alive by the scene)."""
        d = A.WorldDesc()
        d.num_bodies = len(self.bodies)
        d.num_shapes = len(self.shapes)
        d.num_materials = len(self.materials)
        d.num_contact_materials = len(self.contact_materials)
        d.num_constraints = len(self.constraints)
        d.allow_sleep = int(self.allow_sleep)
        d.quat_normalize_skip = self.quat_normalize_skip
        d.quat_normalize_fast = int(self.quat_normalize_fast)
        d.solver_iterations = self.iterations
        d.broadphase = self.broadphase
        d.use_bounding_boxes = int(self.use_bounding_boxes)
        d.sap_axis = self.sap_axis
        d.grid_n[:] = list(self.grid_n)
        d.enable_friction_reduction = int(self.enable_friction_reduction)
        d.has_friction_gravity = 0 if self.friction_gravity is None else 1
        if self.friction_gravity is not None:
            d.friction_gravity[:] = list(self.friction_gravity)
        d.stepnumber = self.stepnumber
        d.solver_tolerance = self.tolerance
        d.time = self.time
        d.gravity[:] = list(self.gravity)
        d.grid_aabb_min[:] = list(self.grid_min)
        d.grid_aabb_max[:] = list(self.grid_max)
        for arr in (self.bodies, self.shapes, self.materials, self.contact_materials, self.constraints, self.body_shapes):
            assert arr.flags["C_CONTIGUOUS"]
        d.body_shapes = A.ptr(self.body_shapes)
        d.num_body_shapes = len(self.body_shapes)
        d.bodies = A.ptr(self.bodies)
        d.shapes = A.ptr(self.shapes)
        d.materials = A.ptr(self.materials)
        d.contact_materials = A.ptr(self.contact_materials)
        d.constraints = A.ptr(self.constraints)
        d.sap_axis_list = 0
        d.solver = self.solver
        d.equation_id_counter = self.equation_id_counter
        d.default_contact_material = A.default_contact_material(self.friction, self.restitution)
        return d


# equations each constraint type's constructor creates (cp_constraint_desc)
CONSTRAINT_EQUATIONS = {A.CON_P2P: 3, A.CON_HINGE: 6, A.CON_DISTANCE: 1, A.CON_LOCK: 6, A.CON_CONE_TWIST: 5,
                        A.CON_SPRING: 1}


def use_split_solver(scene, first_id=0):
    """Switch a scene to the SplitSolver with the equation ids a fresh Dart
    process gives it: the constraints' equations first (constructors run in
    constraint order, ids from first_id), the contact and friction equations
    of the steps after them."""
    scene.solver = A.SOLVER_SPLIT
    nxt = first_id
    for c in scene.constraints:
        c["first_equation_id"] = nxt
        nxt += CONSTRAINT_EQUATIONS[int(c["type"])]
    scene.equation_id_counter = nxt
    return scene


def _plane_body(bodies, shapes, i, shape_index, y=0.0):
    q = euler_xyz(-math.pi / 2, 0.0, 0.0)  # groundBody.quaternion.setFromEuler(-pi/2, 0, 0)
    shapes[shape_index]["type"] = A.SHAPE_PLANE
    bodies[i]["mass"] = 0.0
    bodies[i]["position"] = (0.0, y, 0.0)
    bodies[i]["quaternion"] = q
    bodies[i]["shape"] = shape_index


def spheres_on_plane(n=64, seed=1, radius=0.5):
    """64 Sphere(0.5), mass 1, positions U[-5,5]xU[1,20]xU[-5,5], on a Plane at y=0."""
    rng = SplitMix64(seed)
    shapes = A.default_shapes(2)
    bodies = A.default_bodies(n + 1)
    _plane_body(bodies, shapes, 0, 0)
    shapes[1]["type"] = A.SHAPE_SPHERE
    shapes[1]["radius"] = radius
    u = rng.uniform(3 * n).reshape(n, 3)
    pos = np.stack([-5 + 10 * u[:, 0], 1 + 19 * u[:, 1], -5 + 10 * u[:, 2]], axis=1)
    bodies["mass"][1:] = 1.0
    bodies["position"][1:] = pos
    bodies["shape"][1:] = 1
    return Scene("spheres_on_plane", shapes, bodies, friction=0.3, restitution=0.0, iterations=10,
                 broadphase=A.BROAD_NAIVE, dt=1 / 60, steps=600)


def _box_shapes(shapes, first, he):
    k = len(he)
    shapes["type"][first:first + k] = A.SHAPE_BOX
    shapes["half_extents"][first:first + k] = he


def box_pile(nx=16, nz=16, layers=16, seed=2, pitch=1.1):
    """4096 boxes (half-extents U[0.2,0.5], density 1, random orientation) in a
    16x16 footprint of 16 layers above a Plane; SAP on x, 20 iterations."""
    rng = SplitMix64(seed)
    n = nx * nz * layers
    shapes = A.default_shapes(n + 1)
    bodies = A.default_bodies(n + 1)
    _plane_body(bodies, shapes, 0, 0)
    u = rng.uniform(6 * n).reshape(n, 6)
    he = (0.2 + 0.3 * u[:, :3]).astype(np.float32)
    _box_shapes(shapes, 1, he)
    q = shoemake(u[:, 3], u[:, 4], u[:, 5])
    idx = np.arange(n)
    ix, iz, k = idx % nx, (idx // nx) % nz, idx // (nx * nz)
    pos = np.stack([(ix - (nx - 1) / 2) * pitch, 0.6 + pitch * k, (iz - (nz - 1) / 2) * pitch], axis=1)
    hed = he.astype(np.float64)
    bodies["mass"][1:] = 8.0 * hed[:, 0] * hed[:, 1] * hed[:, 2] * 1.0
    bodies["position"][1:] = pos
    bodies["quaternion"][1:] = q
    bodies["shape"][1:] = np.arange(1, n + 1)
    return Scene("box_pile", shapes, bodies, friction=0.4, restitution=0.0, iterations=20,
                 broadphase=A.BROAD_SAP, sap_axis=0, dt=1 / 60, steps=300)


def mixed_chains(nx=32, nz=16, layers=16, seed=3, pitch=1.3, chains=128, chain_len=16, segments=10):
    """8192 bodies (40% Sphere r U[0.2,0.6], 40% Box as box_pile, 20% Cylinder
    with 10 segments r U[0.2,0.5] h U[0.4,1.0]) on a lattice; the first 2048
    form 128 chains of 16 along x joined by PointToPoint / Hinge(axis z) /
    Distance by link index mod 3.  GridBroadphase with unit cells over the
    scene bounds +-1, sleeping on, 15 iterations, dt 1/120."""
    rng = SplitMix64(seed)
    n = nx * nz * layers
    shapes = A.default_shapes(n + 1)
    bodies = A.default_bodies(n + 1)
    _plane_body(bodies, shapes, 0, 0)
    u = rng.uniform(8 * n).reshape(n, 8)
    kind = np.arange(n) % 5  # 0,1 sphere; 2,3 box; 4 cylinder
    idx = np.arange(n)
    ix, iz, k = idx % nx, (idx // nx) % nz, idx // (nx * nz)
    pos = np.stack([(ix - (nx - 1) / 2) * pitch, 1.0 + pitch * k, (iz - (nz - 1) / 2) * pitch], axis=1)
    mass = np.zeros(n)
    sph = kind <= 1
    box = (kind == 2) | (kind == 3)
    cyl = kind == 4
    s = shapes[1:]
    s["type"][sph] = A.SHAPE_SPHERE
    r = 0.2 + 0.4 * u[sph, 0]
    s["radius"][sph] = r
    mass[sph] = 4.0 / 3.0 * math.pi * r ** 3
    he = (0.2 + 0.3 * u[box, :3]).astype(np.float32)
    s["type"][box] = A.SHAPE_BOX
    s["half_extents"][box] = he
    hed = he.astype(np.float64)
    mass[box] = 8.0 * hed[:, 0] * hed[:, 1] * hed[:, 2]
    s["type"][cyl] = A.SHAPE_CYLINDER
    rc = 0.2 + 0.3 * u[cyl, 0]
    hc = 0.4 + 0.6 * u[cyl, 1]
    s["radius_top"][cyl] = rc
    s["radius_bottom"][cyl] = rc
    s["height"][cyl] = hc
    s["num_segments"][cyl] = segments
    mass[cyl] = math.pi * rc ** 2 * hc
    q = shoemake(u[:, 3], u[:, 4], u[:, 5])
    q[sph] = (0.0, 0.0, 0.0, 1.0)
    bodies["mass"][1:] = mass
    bodies["position"][1:] = pos
    bodies["quaternion"][1:] = q
    bodies["shape"][1:] = np.arange(1, n + 1)
    cons = np.zeros(chains * (chain_len - 1), dtype=A.CONSTRAINT_DTYPE)
    c = 0
    for ch in range(chains):
        first = 1 + ch * chain_len
        for j in range(chain_len - 1):
            rec = cons[c]
            rec["type"] = (A.CON_P2P, A.CON_HINGE, A.CON_DISTANCE)[j % 3]
            rec["body_a"] = first + j
            rec["body_b"] = first + j + 1
            rec["collide_connected"] = 1
            rec["pivot_a"] = (pitch / 2, 0.0, 0.0)
            rec["pivot_b"] = (-pitch / 2, 0.0, 0.0)
            rec["axis_a"] = (0.0, 0.0, 1.0)
            rec["axis_b"] = (0.0, 0.0, 1.0)
            rec["distance"] = -1.0
            rec["max_force"] = 1e6
            rec["spook_stiffness"] = 1e7
            rec["spook_relaxation"] = 4.0
            rec["spook_time_step"] = 1.0 / 60.0
            c += 1
    lo = np.minimum(pos.min(axis=0), 0.0) - 1.0
    hi = pos.max(axis=0) + 1.0
    lo32 = lo.astype(np.float32).astype(np.float64)
    hi32 = hi.astype(np.float32).astype(np.float64)
    gn = tuple(int(max(1, math.ceil(e))) for e in (hi32 - lo32))
    return Scene("mixed_chains", shapes, bodies, constraints=cons, friction=0.3, restitution=0.0, iterations=15,
                 broadphase=A.BROAD_GRID, grid_n=gn, grid_min=tuple(lo), grid_max=tuple(hi), allow_sleep=True,
                 dt=1 / 120, steps=240)


def column_world(n, seed, mix="sphere_box", footprint=None, pitch=1.2, name="world"):
    """One world of `n` bodies dropped in a column above a Plane (the plane is
    body 0, so the world holds n+1 bodies).  mix="sphere_box": 50/50 Sphere(0.5)
    mass 1 / Box as box_pile; mix="mixed": the 40/40/20 sphere/box/cylinder mix."""
    rng = SplitMix64(seed)
    side = footprint or max(2, int(math.ceil(math.sqrt(n / 8.0))))
    shapes = A.default_shapes(n + 1)
    bodies = A.default_bodies(n + 1)
    _plane_body(bodies, shapes, 0, 0)
    u = rng.uniform(8 * n).reshape(n, 8)
    idx = np.arange(n)
    cell, layer = idx % (side * side), idx // (side * side)
    jitter = (u[:, 6:8] - 0.5) * 0.1
    pos = np.stack([(cell % side - (side - 1) / 2) * pitch + jitter[:, 0], 1.0 + pitch * layer,
                    (cell // side - (side - 1) / 2) * pitch + jitter[:, 1]], axis=1)
    s = shapes[1:]
    mass = np.zeros(n)
    if mix == "sphere_box":
        sph = u[:, 7] < 0.5
        box = ~sph
        cyl = np.zeros(n, dtype=bool)
        r = np.full(int(sph.sum()), 0.5)
    else:
        kind = (u[:, 7] * 5).astype(np.int64)
        sph = kind <= 1
        box = (kind == 2) | (kind == 3)
        cyl = kind == 4
        r = 0.2 + 0.4 * u[sph, 0]
    s["type"][sph] = A.SHAPE_SPHERE
    s["radius"][sph] = r
    mass[sph] = 1.0 if mix == "sphere_box" else 4.0 / 3.0 * math.pi * r ** 3
    he = (0.2 + 0.3 * u[box, :3]).astype(np.float32)
    s["type"][box] = A.SHAPE_BOX
    s["half_extents"][box] = he
    hed = he.astype(np.float64)
    mass[box] = 8.0 * hed[:, 0] * hed[:, 1] * hed[:, 2]
    if cyl.any():
        rc = 0.2 + 0.3 * u[cyl, 0]
        hc = 0.4 + 0.6 * u[cyl, 1]
        s["type"][cyl] = A.SHAPE_CYLINDER
        s["radius_top"][cyl] = rc
        s["radius_bottom"][cyl] = rc
        s["height"][cyl] = hc
        s["num_segments"][cyl] = 10
        mass[cyl] = math.pi * rc ** 2 * hc
    q = shoemake(u[:, 3], u[:, 4], u[:, 5])
    q[sph] = (0.0, 0.0, 0.0, 1.0)
    bodies["mass"][1:] = mass
    bodies["position"][1:] = pos
    bodies["quaternion"][1:] = q
    bodies["shape"][1:] = np.arange(1, n + 1)
    return Scene(name, shapes, bodies, friction=0.3, restitution=0.0, iterations=10, broadphase=A.BROAD_NAIVE,
                 dt=1 / 60, steps=120)


def compound_pile(n=40, seed=31, broadphase=A.BROAD_NAIVE, kinematic=True, pitch=1.9, per_row=5, kinds=(0, 1, 2, 3, 4)):
    """Compound bodies (Body.addShape with offsets and orientations) dropped
    in a pile on a Plane, with single-shape bodies between them: dumbbells
    (a box bar and two spheres), L pieces (two boxes, the second turned
    90 degrees about z), tables (a box top on four box legs), and a cylinder
    with a sphere cap.  With `kinematic`, a kinematic dumbbell sweeps through
    the pile and a static L piece stands in it, so kinematic / static shape
    pairs take the justTest path.  Body i is of kind kinds[i % len(kinds)]
    (0 dumbbell, 1 L piece, 2 table, 3 capped cylinder, 4 single shape)."""
    rng = SplitMix64(seed)
    shapes, entries, bodies_l = [], [], []  # shape rows, extra-shape rows, (first shape, extras, mass, pos, quat)

    def shape(kind, **f):
        shapes.append((kind, f))
        return len(shapes) - 1

    def body(parts, mass, pos, quat, **extra):
        # parts: (shape index, offset, orientation); the first is the body's shape
        first = len(entries)
        for sh, off, q in parts[1:]:
            entries.append((sh, off, q))
        bodies_l.append(dict(first=parts[0], extra_first=first, extra_count=len(parts) - 1, mass=mass, pos=pos,
                             quat=quat, **extra))

    ident = (0.0, 0.0, 0.0, 1.0)
    zq = euler_xyz(0.0, 0.0, math.pi / 2)
    plane = shape(A.SHAPE_PLANE)
    body([(plane, (0.0, 0.0, 0.0), ident)], 0.0, (0.0, 0.0, 0.0), euler_xyz(-math.pi / 2, 0.0, 0.0))
    u = rng.uniform(8 * n).reshape(n, 8)
    for i in range(n):
        kind = kinds[i % len(kinds)]
        pos = ((i % per_row - (per_row - 1) / 2) * pitch + 0.2 * u[i, 0], 1.0 + 1.2 * (i // per_row),
               ((i // per_row) % 3 - 1) * 0.6 + 0.2 * u[i, 1])
        q = tuple(shoemake(u[i:i + 1, 2], u[i:i + 1, 3], u[i:i + 1, 4])[0])
        if kind == 0:  # dumbbell
            bar = shape(A.SHAPE_BOX, half_extents=(0.4, 0.08, 0.08))
            s1 = shape(A.SHAPE_SPHERE, radius=0.18 + 0.05 * u[i, 5])
            s2 = shape(A.SHAPE_SPHERE, radius=0.18)
            body([(bar, (0.0, 0.0, 0.0), ident), (s1, (-0.45, 0.0, 0.0), ident), (s2, (0.45, 0.0, 0.0), ident)],
                 1.2, pos, q)
        elif kind == 1:  # L piece
            a = shape(A.SHAPE_BOX, half_extents=(0.35, 0.1, 0.15))
            b = shape(A.SHAPE_BOX, half_extents=(0.25, 0.1, 0.15))
            body([(a, (0.1, 0.0, 0.0), ident), (b, (-0.15, 0.3, 0.0), zq)], 0.9, pos, q)
        elif kind == 2:  # table: top and four legs, the top offset from the centre of mass
            top = shape(A.SHAPE_BOX, half_extents=(0.45, 0.05, 0.3))
            legs = [shape(A.SHAPE_BOX, half_extents=(0.04, 0.2, 0.04)) for _ in range(4)]
            parts = [(top, (0.0, 0.2, 0.0), ident)]
            for k, (sx, sz) in enumerate(((1, 1), (1, -1), (-1, 1), (-1, -1))):
                parts.append((legs[k], (0.4 * sx, -0.05, 0.25 * sz), ident))
            body(parts, 1.5, pos, q)
        elif kind == 3:  # cylinder with a sphere cap
            cyl = shape(A.SHAPE_CYLINDER, radius_top=0.2, radius_bottom=0.2, height=0.6, num_segments=8)
            cap = shape(A.SHAPE_SPHERE, radius=0.22)
            body([(cyl, (0.0, 0.0, 0.0), ident), (cap, (0.0, 0.35, 0.0), ident)], 1.0, pos, q)
        else:  # a single box or sphere between the compounds
            if u[i, 6] < 0.5:
                body([(shape(A.SHAPE_BOX, half_extents=(0.25, 0.2, 0.3)), (0.0, 0.0, 0.0), ident)], 0.6, pos, q)
            else:
                body([(shape(A.SHAPE_SPHERE, radius=0.3), (0.05, 0.0, 0.0), ident)], 0.5, pos, ident)
    if kinematic:
        bar = shape(A.SHAPE_BOX, half_extents=(0.6, 0.1, 0.1))
        s1 = shape(A.SHAPE_SPHERE, radius=0.25)
        s2 = shape(A.SHAPE_BOX, half_extents=(0.2, 0.2, 0.2))
        body([(bar, (0.0, 0.0, 0.0), ident), (s1, (-0.7, 0.0, 0.0), ident), (s2, (0.7, 0.0, 0.0), euler_xyz(0.3, 0.2, 0.1))],
             0.0, (-6.0, 0.6, 0.0), ident, type=A.BODY_KINEMATIC, velocity=(2.0, 0.0, 0.0), angular_velocity=(0.0, 1.0, 0.0))
        a = shape(A.SHAPE_BOX, half_extents=(0.5, 0.1, 0.5))
        b = shape(A.SHAPE_BOX, half_extents=(0.1, 0.5, 0.1))
        body([(a, (0.0, 1.0, 0.0), ident), (b, (0.0, 0.4, 0.0), ident)], 0.0, (3.0, 0.0, 1.5), ident)
    S = A.default_shapes(len(shapes))
    for k, (kind, f) in enumerate(shapes):
        S[k]["type"] = kind
        for name, v in f.items():
            S[k][name] = v
    E = A.body_shapes(len(entries))
    for k, (sh, off, q) in enumerate(entries):
        E[k]["shape"] = sh
        E[k]["offset"] = off
        E[k]["orientation"] = q
    B = A.default_bodies(len(bodies_l))
    for k, d in enumerate(bodies_l):
        sh, off, q = d["first"]
        B[k]["shape"] = sh
        B[k]["shape_offset"] = off
        B[k]["shape_orientation"] = q
        B[k]["extra_shapes_first"] = d["extra_first"] if d["extra_count"] else 0
        B[k]["extra_shapes_count"] = d["extra_count"]
        B[k]["mass"] = d["mass"]
        B[k]["position"] = d["pos"]
        B[k]["quaternion"] = d["quat"]
        if "type" in d:
            B[k]["type"] = d["type"]
        for f in ("velocity", "angular_velocity"):
            if f in d:
                B[k][f] = d[f]
    sc = Scene("compound_pile", S, B, friction=0.4, restitution=0.1, iterations=12, broadphase=broadphase, dt=1 / 60,
               steps=150, body_shapes=E)
    if broadphase == A.BROAD_SAP:
        sc.sap_axis = 0
    elif broadphase == A.BROAD_GRID:
        sc.grid_n = (8, 4, 4)
        sc.grid_min = (-6.0, -1.0, -3.0)
        sc.grid_max = (6.0, 8.0, 3.0)
    return sc


# ---------------------------------------------------------------------------
# hulls of the ConvexPolyhedron subclasses with their own ShapeType, built as
# their constructors build them (vertices in binary32, faces, uniqueAxes)


def cone_hull(radius=1.0, height=1.0, num_segments=8):
    """Cone (lib/rigid_body_shapes/cone.dart:15-64): apex, base ring, side
    triangles and the base face; uniqueAxes [(0, 1, 0)]."""
    n = num_segments
    verts = [(0.0, height * 0.5, 0.0), (-radius * math.sin(0), -height * 0.5, radius * math.cos(0))]
    faces, bottom = [], [1]
    for i in range(n):
        theta = ((2 * math.pi) / n) * (i + 1)
        if i < n - 1:
            verts.append((-radius * math.sin(theta), -height * 0.5, radius * math.cos(theta)))
            bottom.append(i + 2)
            faces.append([0, i + 2, i + 1])
        else:
            faces.append([0, 1, i + 1])
    faces.append(bottom)
    return np.array(verts, np.float32), faces, np.array([(0.0, 1.0, 0.0)], np.float32)


def sized_plane_hull(width=1.0, height=1.0):
    """SizedPlane (lib/rigid_body_shapes/sized_plane.dart:19-37): one face at y = 0."""
    sx, sy, sz = width / 2, 0.0, height / 2
    verts = [(-sx, sy, -sz), (sx, sy, -sz), (sx, sy, sz), (-sx, sy, sz)]
    return np.array(verts, np.float32), [[3, 2, 1, 0]], None


def capsule_hull(radius_top=1.0, radius_bottom=1.0, height=1.0, num_segments=8, num_height_segments=4):
    """Capsule (lib/rigid_body_shapes/capsule.dart:27-170): the cylinder's
    side walls, then two hemisphere grids, both drawn with radiusTop as the
    constructor draws them; no uniqueAxes."""
    rt, rb, h = radius_top, radius_bottom, height
    ns, nh = num_segments, num_height_segments
    verts = [(-rb * math.sin(0), -h * 0.5, rb * math.cos(0)), (-rt * math.sin(0), h * 0.5, rt * math.cos(0))]
    faces, top, bottom, grid = [], [], [], []
    index = 0
    phi_start, phi_length, theta_start, theta_length = math.pi, 2 * math.pi, math.pi / 2, math.pi / 2
    for iy in range(nh + 1):
        row = []
        v = iy / nh
        for ix in range(ns + 1):
            ub = ix / ns
            ut = (ns - ix) / ns
            if iy == 0 and ix < ns:
                theta = ((2 * math.pi) / ns) * (ix + 1)
                if ix < ns - 1:
                    verts.append((-rb * math.sin(theta), -h * 0.5, rb * math.cos(theta)))
                    verts.append((-rt * math.sin(theta), h * 0.5, rt * math.cos(theta)))
                    faces.append([2 * ix, 2 * ix + 1, 2 * ix + 3, 2 * ix + 2])
                else:
                    faces.append([2 * ix, 2 * ix + 1, 1, 0])
            st = math.sin(theta_start + v * theta_length)
            ct = math.cos(theta_start + v * theta_length)
            top.append((-rt * math.cos(phi_start + ut * phi_length) * st, h * 0.5 - rt * ct,
                        rt * math.sin(phi_start + ut * phi_length) * st))
            bottom.append((-rt * math.cos(phi_start + ub * phi_length) * st, -h * 0.5 + rt * ct,
                           rt * math.sin(phi_start + ub * phi_length) * st))
            row.append(index)
            index += 1
        grid.append(row)
    s1 = len(verts)
    s2 = s1 + len(top)
    for iy in range(nh):
        for ix in range(ns):
            for s in (s1, s2):
                a, b = grid[iy][ix + 1] + s, grid[iy][ix] + s
                c, d = grid[iy + 1][ix] + s, grid[iy + 1][ix + 1] + s
                faces.append([a, b, d])
                faces.append([b, c, d])
    verts += top + bottom
    return np.array(verts, np.float32), faces, None


def set_hull(shape, kind, hull, keep):
    """Point shape record `shape` at hull (vertices, faces, axes or None) as a
    shape of type `kind`; the arrays are appended to `keep`."""
    v, faces, axes = hull
    sizes = np.array([len(f) for f in faces], np.int32)
    flat = np.array([k for f in faces for k in f], np.int32)
    v = np.ascontiguousarray(v, np.float32)
    keep += [v, sizes, flat]
    shape["type"] = kind
    shape["num_vertices"] = len(v)
    shape["num_faces"] = len(faces)
    shape["vertices"] = v.ctypes.data
    shape["face_sizes"] = sizes.ctypes.data
    shape["face_indices"] = flat.ctypes.data
    if axes is not None:
        axes = np.ascontiguousarray(axes, np.float32)
        keep.append(axes)
        shape["has_axes"] = 1
        shape["num_axes"] = len(axes)
        shape["axes"] = axes.ctypes.data
    else:
        shape["has_axes"] = 0
        shape["num_axes"] = 0


# ---------------------------------------------------------------------------
# constraint records as the reference's constructors leave them


def _f32(x):
    return float(np.float32(x))


def _vmult(q, v):
    """Quaternion.vmult (lib/math/quaternion.dart:21-44): binary64 arithmetic,
    binary32 result."""
    x, y, z = (float(c) for c in v)
    qx, qy, qz, qw = (float(c) for c in q)
    ix = qw * x + qy * z - qz * y
    iy = qw * y + qz * x - qx * z
    iz = qw * z + qx * y - qy * x
    iw = -qx * x - qy * y - qz * z
    return (_f32(ix * qw + iw * -qx + iy * -qz - iz * -qy), _f32(iy * qw + iw * -qy + iz * -qx - ix * -qz),
            _f32(iz * qw + iw * -qz + ix * -qy - iy * -qx))


def _conj(q):
    return (-float(q[0]), -float(q[1]), -float(q[2]), float(q[3]))


def lock_frames(pos_a, quat_a, pos_b, quat_b):
    """LockConstraint's constructor (lib/constraints/lock_constraint.dart:26-76):
    returns pivot_a, pivot_b and (xA, xB, yA, yB, zA, zB).  Body.pointToLocalFrame
    and vectorToLocalFrame (rigid_body.dart:317-329) conjugate the body's own
    quaternion in place before rotating, so successive calls alternate between
    the conjugate and the quaternion itself: the pivots and yA, yB use the
    conjugates, xA, xB, zA, zB the quaternions (each body ends as it began)."""
    half = tuple(_f32(_f32(float(a) + float(b)) * 0.5) for a, b in zip(pos_a, pos_b))
    rel_b = tuple(_f32(h - float(p)) for h, p in zip(half, pos_b))
    rel_a = tuple(_f32(h - float(p)) for h, p in zip(half, pos_a))
    qa, qb = _conj(quat_a), _conj(quat_b)
    pivot_b = _vmult(qb, rel_b)
    pivot_a = _vmult(qa, rel_a)
    ex, ey, ez = (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)
    axes = []
    for e in (ex, ey, ez):
        qa, qb = _conj(qa), _conj(qb)
        axes.append(_vmult(qa, e))
        axes.append(_vmult(qb, e))
    return pivot_a, pivot_b, axes


def _con(rec, kind, a, b, max_force=1e6, collide=1):
    rec["type"] = kind
    rec["body_a"] = a
    rec["body_b"] = b
    rec["collide_connected"] = collide
    rec["distance"] = -1.0
    rec["max_force"] = max_force
    rec["spook_stiffness"] = 1e7
    rec["spook_relaxation"] = 4.0
    rec["spook_time_step"] = 1.0 / 60.0


def joints_and_hulls(n_chains=4, seed=41, broadphase=A.BROAD_NAIVE):
    """Chains of boxes, cones and capsules joined by LockConstraints,
    ConeTwistConstraints and SpringConstraints in turn, hanging from static
    anchors above a Plane and SizedPlane tiles, and loose spheres, boxes,
    cones, capsules and ConvexPolyhedron pyramids dropped onto the tiles (a
    pyramid finds no resolver against a SizedPlane and falls through to the
    plane); the chains swing into each other and onto the tiles."""
    rng = SplitMix64(seed)
    keep = []
    per = 5
    loose = 10
    n = 1 + 4 + n_chains * (per + 1) + loose
    shapes = A.default_shapes(n)
    bodies = A.default_bodies(n)
    _plane_body(bodies, shapes, 0, 0)
    i = 1
    for t in range(4):  # SizedPlane tiles: static, tilted a little
        set_hull(shapes[i], A.SHAPE_SIZED_PLANE, sized_plane_hull(2.4, 1.6), keep)
        bodies[i]["mass"] = 0.0
        bodies[i]["position"] = ((t - 1.5) * 2.6, 0.3 + 0.1 * t, 0.4)
        bodies[i]["quaternion"] = euler_xyz(0.15 * (t - 1.5), 0.0, 0.1)
        bodies[i]["shape"] = i
        i += 1
    cons = np.zeros(n_chains * per, dtype=A.CONSTRAINT_DTYPE)
    c = 0
    u = rng.uniform(4 * n).reshape(n, 4)
    for ch in range(n_chains):
        x0 = (ch - (n_chains - 1) / 2) * 1.7
        anchor = i
        shapes[i]["type"] = A.SHAPE_SPHERE
        shapes[i]["radius"] = 0.1
        bodies[i]["mass"] = 0.0
        bodies[i]["position"] = (x0, 2.2, 0.0)
        bodies[i]["shape"] = i
        i += 1
        for k in range(per):
            kind = (ch + k) % 3
            if kind == 0:
                shapes[i]["type"] = A.SHAPE_BOX
                shapes[i]["half_extents"] = (0.2, 0.25, 0.15)
            elif kind == 1:
                set_hull(shapes[i], A.SHAPE_CONE, cone_hull(0.25, 0.5, 6 + ch % 3), keep)
            else:
                set_hull(shapes[i], A.SHAPE_CAPSULE, capsule_hull(0.15, 0.15, 0.3, 3, 1), keep)
            bodies[i]["mass"] = 0.5 + 0.5 * u[i, 0]
            bodies[i]["position"] = (x0 + 0.3 * (k + 1) + 0.05 * u[i, 1], 2.2 - 0.1 * (k + 1), 0.05 * u[i, 2])
            bodies[i]["quaternion"] = euler_xyz(0.2 * u[i, 3], 0.1 * k, 0.0)
            bodies[i]["shape"] = i
            prev = anchor if k == 0 else i - 1
            rec = cons[c]
            jt = (ch + k) % 3
            if jt == 0:
                _con(rec, A.CON_LOCK, prev, i, max_force=1e6)
                pa, pb, axes = lock_frames(bodies[prev]["position"], bodies[prev]["quaternion"], bodies[i]["position"],
                                           bodies[i]["quaternion"])
                rec["pivot_a"], rec["pivot_b"] = pa, pb
                rec["lock_axes"] = axes
            elif jt == 1:
                _con(rec, A.CON_CONE_TWIST, prev, i, max_force=1e6)
                rec["pivot_a"] = (0.15, -0.05, 0.0)
                rec["pivot_b"] = (-0.15, 0.05, 0.0)
                rec["axis_a"] = (1.0, 0.0, 0.0)
                rec["axis_b"] = (1.0, 0.0, 0.0)
                rec["angle"] = 0.3 + 0.2 * (ch % 2)
                rec["twist_angle"] = 0.2 + 0.1 * k
            else:
                _con(rec, A.CON_SPRING, prev, i, max_force=30.0 + 10.0 * k)
            c += 1
            i += 1
    pyramid = (np.array([(-0.2, 0.0, -0.2), (0.2, 0.0, -0.2), (0.2, 0.0, 0.2), (-0.2, 0.0, 0.2), (0.0, 0.3, 0.0)],
                        np.float32), [[3, 2, 1, 0], [0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4]], None)
    for k in range(loose):
        kind = k % 5
        if kind == 0:
            shapes[i]["type"] = A.SHAPE_SPHERE
            shapes[i]["radius"] = 0.2
        elif kind == 1:
            shapes[i]["type"] = A.SHAPE_BOX
            shapes[i]["half_extents"] = (0.2, 0.15, 0.25)
        elif kind == 2:
            set_hull(shapes[i], A.SHAPE_CONE, cone_hull(0.2, 0.4, 8), keep)
        elif kind == 3:
            set_hull(shapes[i], A.SHAPE_CAPSULE, capsule_hull(0.12, 0.12, 0.3, 3, 1), keep)
        else:
            set_hull(shapes[i], A.SHAPE_CONVEX, pyramid, keep)
        bodies[i]["mass"] = 0.4 + 0.4 * u[i, 0]
        bodies[i]["position"] = ((k % 4 - 1.5) * 2.6 + 0.4 * u[i, 1], 0.9 + 0.5 * (k // 4), 0.4 + 0.3 * u[i, 2])
        bodies[i]["quaternion"] = shoemake(u[i:i + 1, 3], u[i:i + 1, 1], u[i:i + 1, 2])[0]
        bodies[i]["shape"] = i
        i += 1
    sc = Scene("joints_and_hulls", shapes, bodies, constraints=cons[:c], friction=0.3, restitution=0.0, iterations=12,
               broadphase=broadphase, dt=1 / 60, steps=200)
    sc._keep = keep
    if broadphase == A.BROAD_GRID:
        sc.grid_n = (6, 3, 2)
        sc.grid_min = (-5.0, -1.0, -2.0)
        sc.grid_max = (5.0, 5.0, 2.0)
    return sc


def batch_sizes(n_worlds=4096, seed=1000, lo=8, hi=512):
    """Body counts floor(exp(U[ln lo, ln hi])) of the batched workload, one
    SplitMix64 stream per world (seed+w)."""
    out = np.empty(n_worlds, dtype=np.int64)
    for w in range(n_worlds):
        u = SplitMix64(seed + w).uniform(1)[0]
        out[w] = int(math.floor(math.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))))
    return np.minimum(out, hi)


def batch_worlds(n_worlds=4096, seed=1000, lo=8, hi=512):
    """The batched workload: world w has batch_sizes()[w] bodies plus its plane,
    built from seed (seed+w)*7919+1."""
    sizes = batch_sizes(n_worlds, seed, lo, hi)
    return [column_world(int(sizes[w]), (seed + w) * 7919 + 1, "sphere_box", name=f"batch{w}") for w in range(n_worlds)]


@dataclass
class Request:
    arrival: float
    n_bodies: int
    horizon: int
    seed: int


def serve_requests(rate=2000.0, window=60.0, seed=77, lo=16, hi=4096, max_horizon=240):
    """Poisson arrivals at `rate` req/s over `window` seconds; each request is a
    world of floor(exp(U[ln lo, ln hi])) bodies in the 40/40/20 mix and a
    horizon uniform in 1..max_horizon steps."""
    rng = SplitMix64(seed)
    reqs = []
    t = 0.0
    i = 0
    while True:
        u = rng.uniform(3)
        t += -math.log(1.0 - u[0]) / rate
        if t >= window:
            break
        n = int(math.floor(math.exp(math.log(lo) + u[1] * (math.log(hi) - math.log(lo)))))
        h = 1 + min(max_horizon - 1, int(u[2] * max_horizon))
        reqs.append(Request(t, min(n, hi), h, seed * 1000003 + i))
        i += 1
    return reqs


def request_world(req):
    return column_world(req.n_bodies, req.seed, "mixed", name=f"req{req.seed}")
