"""Seeded synthetic scenes for the rigid-body step.

Headless restatements of the scene recipes the reference's demos use
(ode/demo/demo_boxstack.cpp:130-170 for the near callback and stack,
ode/demo/demo_crash.cpp:119-150 for a wall of boxes), sized to the two
single-world workloads this package measures:

* ``box_stack``   -- 10 unit boxes (1 m, density 1) stacked on the plane z=0,
  x/y jitter U(+-0.01 m), yaw U(+-5 deg); gravity -9.81, dt 0.01, 20 SOR
  iterations, W 1.3, mu 0.5, dContactApprox1, <= 4 contacts per pair,
  ERP 0.2, CFM 1e-5.
* ``pile``        -- N bodies (default 32,768) dropped into an open box made of
  5 static planes: 50 % spheres r~U[0.05,0.25] m, 50 % boxes sides
  ~U[0.1,0.5] m, density ~U[500,2000] kg/m^3, on a jittered 3-D grid with
  random unit quaternions; dt 1/120, 30 iterations, mu 0.6.

Every array is float32 / int32 so that the same bytes feed the reference,
the CPU restatement and the GPU path.

Layouts (shared with tests/golden/gen_golden.cpp):
  bodies  float32 [nb, 20]: pos(3) q(4, w first) lvel(3) avel(3) mass(1)
                            I11 I22 I33 I12 I13 I23 (body frame, about the COM)
  geoms   cls int32 [ng]  (0 sphere, 1 box, 2 capsule, 4 plane: ODE class ids)
          body int32 [ng] (-1 = static geom)
          pos float32 [ng,3], R float32 [ng,12] (3x4 row-major, only for static
          geoms), dims float32 [ng,4] (sphere r | box lx ly lz | capsule r len |
          plane a b c d)
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SPHERE, BOX, CAPSULE, PLANE = 0, 1, 2, 4
JOINT_COLS = 20

# dSurfaceParameters.mode bits (include/ode/contact.h:28-52)
dContactMu2 = 0x001
dContactAxisDep = 0x001
dContactFDir1 = 0x002
dContactBounce = 0x004
dContactSoftERP = 0x008
dContactSoftCFM = 0x010
dContactMotion1 = 0x020
dContactMotion2 = 0x040
dContactMotionN = 0x080
dContactSlip1 = 0x100
dContactSlip2 = 0x200
dContactRolling = 0x400
dContactApprox1_1 = 0x1000
dContactApprox1_2 = 0x2000
dContactApprox1_N = 0x4000
dContactApprox1 = 0x7000


@dataclasses.dataclass
class Scene:
    name: str
    bodies: np.ndarray          # float32 [nb, 20]
    geom_cls: np.ndarray        # int32 [ng]
    geom_body: np.ndarray       # int32 [ng]
    geom_pos: np.ndarray        # float32 [ng, 3]
    geom_R: np.ndarray          # float32 [ng, 12]
    geom_dims: np.ndarray       # float32 [ng, 4]
    dt: float = 0.01
    gravity: tuple = (0.0, 0.0, -9.81)
    erp: float = 0.2
    cfm: float = 1e-5
    w: float = 1.3
    iterations: int = 20
    max_vel: float = float("inf")
    min_depth: float = 0.0
    mu: float = 0.5
    mu2: float = 0.0
    bounce: float = 0.0
    bounce_vel: float = 0.0
    soft_erp: float = 0.0
    soft_cfm: float = 0.0
    surface_mode: int = dContactApprox1
    maxc: int = 4
    hash_levels: tuple = (-3, 10)
    # joints, float32 [nj, JOINT_COLS]: type (1 ball, 2 hinge, 6 hinge2),
    # body1, body2 (-1: the static environment), anchor xyz, axis (hinge) or
    # axis 1 (hinge2) xyz, lo stop, hi stop (axis 1), axis 2 xyz (hinge2),
    # axis-2 motor velocity and max force, suspension ERP and CFM (hinge2),
    # axis-1 motor velocity and max force -- all in the world frame
    joints: np.ndarray | None = None
    # world damping defaults copied into every body: linear scale, angular
    # scale, linear threshold, angular threshold, max angular speed
    damping: tuple = (0.0, 0.0, 0.01, 0.01, float("inf"))
    # world auto-disable defaults copied into every body (None: the reference's
    # defaults, auto-disable off): flag, linear threshold, angular threshold,
    # idle steps, idle time, average samples
    adis: tuple | None = None

    @property
    def nb(self) -> int:
        return int(self.bodies.shape[0])

    @property
    def ng(self) -> int:
        return int(self.geom_cls.shape[0])

    def world_params(self) -> np.ndarray:
        """dt, g(3), erp, cfm, w, max_vel, min_depth as float32[9]."""
        return np.array([self.dt, *self.gravity, self.erp, self.cfm, self.w,
                         self.max_vel, self.min_depth], dtype=np.float32)

    def surface(self) -> np.ndarray:
        """mu, mu2, bounce, bounce_vel, soft_erp, soft_cfm, 0, 0 as float32[8]."""
        return np.array([self.mu, self.mu2, self.bounce, self.bounce_vel,
                         self.soft_erp, self.soft_cfm, 0, 0], dtype=np.float32)


def quat_to_R(q: np.ndarray) -> np.ndarray:
    """Rotation matrix (3x4 row-major, float32) from unit quaternions [...,4]
    (w,x,y,z), by the same formula as dRfromQ (ode/src/rotation.cpp:236-254),
    evaluated in float32 term by term."""
    q = np.asarray(q, dtype=np.float32)
    two = np.float32(2)
    one = np.float32(1)
    q0, q1, q2, q3 = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    qq1 = two * q1 * q1
    qq2 = two * q2 * q2
    qq3 = two * q3 * q3
    R = np.zeros(q.shape[:-1] + (12,), dtype=np.float32)
    R[..., 0] = one - qq2 - qq3
    R[..., 1] = two * (q1 * q2 - q0 * q3)
    R[..., 2] = two * (q1 * q3 + q0 * q2)
    R[..., 4] = two * (q1 * q2 + q0 * q3)
    R[..., 5] = one - qq1 - qq3
    R[..., 6] = two * (q2 * q3 - q0 * q1)
    R[..., 8] = two * (q1 * q3 - q0 * q2)
    R[..., 9] = two * (q2 * q3 + q0 * q1)
    R[..., 10] = one - qq1 - qq2
    return R


def random_quats(rng: np.random.Generator, n: int) -> np.ndarray:
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def mass_box(density, lx, ly, lz):
    """dMassSetBox (ode/src/mass.cpp:182-196): mass and body-frame inertia."""
    density = np.float32(density)
    lx, ly, lz = np.float32(lx), np.float32(ly), np.float32(lz)
    m = lx * ly * lz * density
    k = m / np.float32(12.0)
    return m, k * (ly * ly + lz * lz), k * (lx * lx + lz * lz), k * (lx * lx + ly * ly)


def mass_sphere(density, r):
    """dMassSetSphere (ode/src/mass.cpp:118-130)."""
    r = np.float32(r)
    m = np.float32(4.0) / np.float32(3.0) * np.float32(math.pi) * r * r * r * np.float32(density)
    ii = np.float32(0.4) * m * r * r
    return m, ii, ii, ii


def _body_rows(pos, q, mass, I3):
    n = pos.shape[0]
    b = np.zeros((n, 20), dtype=np.float32)
    b[:, 0:3] = pos
    b[:, 3:7] = q
    b[:, 13] = mass
    b[:, 14:17] = I3
    return b


def box_stack(seed: int = 0, n: int = 10) -> Scene:
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 3), dtype=np.float32)
    pos[:, 0:2] = rng.uniform(-0.01, 0.01, size=(n, 2))
    pos[:, 2] = 0.5 + np.arange(n, dtype=np.float32)
    yaw = np.deg2rad(rng.uniform(-5.0, 5.0, size=n))
    q = np.zeros((n, 4), dtype=np.float32)
    q[:, 0] = np.cos(yaw / 2)
    q[:, 3] = np.sin(yaw / 2)
    m, i1, i2, i3 = mass_box(1.0, 1.0, 1.0, 1.0)
    bodies = _body_rows(pos, q, m, np.array([i1, i2, i3], dtype=np.float32))
    ng = n + 1
    cls = np.full(ng, BOX, dtype=np.int32)
    cls[-1] = PLANE
    gbody = np.arange(ng, dtype=np.int32)
    gbody[-1] = -1
    gdims = np.zeros((ng, 4), dtype=np.float32)
    gdims[:n, 0:3] = 1.0
    gdims[-1] = (0, 0, 1, 0)
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene("box_stack", bodies, cls, gbody, np.zeros((ng, 3), np.float32), gR, gdims,
                 dt=0.01, iterations=20, mu=0.5, maxc=4)


def sleep_stacks(seed: int = 0, adis=(1, 0.15, 0.15, 10, 0.0, 1), drop_height: float = 4.0) -> Scene:
    """Two stacks of three unit boxes 3 m apart on the plane z = 0 and a
    fourth unit box dropped from `drop_height` onto the first stack, slightly
    off-centre: with auto-disable on, both stacks fall asleep before the drop
    lands, the struck stack wakes (the dropped box is never idle while it has
    no contact) and settles again, the other one sleeps throughout."""
    rng = np.random.default_rng(seed)
    n = 7
    pos = np.zeros((n, 3), dtype=np.float32)
    pos[0:3, 0] = 0.0
    pos[3:6, 0] = 3.0
    pos[0:6, 0:2] += rng.uniform(-0.01, 0.01, size=(6, 2)).astype(np.float32)
    pos[0:6, 2] = 0.5 + np.tile(np.arange(3, dtype=np.float32), 2)
    pos[6] = (0.05, 0.02, drop_height)
    yaw = np.deg2rad(rng.uniform(-5.0, 5.0, size=n))
    yaw[6] = np.deg2rad(10.0)
    q = np.zeros((n, 4), dtype=np.float32)
    q[:, 0] = np.cos(yaw / 2)
    q[:, 3] = np.sin(yaw / 2)
    m, i1, i2, i3 = mass_box(1.0, 1.0, 1.0, 1.0)
    bodies = _body_rows(pos, q, m, np.array([i1, i2, i3], dtype=np.float32))
    ng = n + 1
    cls = np.full(ng, BOX, dtype=np.int32)
    cls[-1] = PLANE
    gbody = np.arange(ng, dtype=np.int32)
    gbody[-1] = -1
    gdims = np.zeros((ng, 4), dtype=np.float32)
    gdims[:n, 0:3] = 1.0
    gdims[-1] = (0, 0, 1, 0)
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene("sleep_stacks", bodies, cls, gbody, np.zeros((ng, 3), np.float32), gR, gdims,
                 dt=0.01, iterations=20, mu=0.5, maxc=4, adis=tuple(adis))


def pile(n: int = 32768, seed: int = 1, spacing: float = 0.6, jitter: float = 0.05) -> Scene:
    """Open-box pile: n bodies on a jittered grid of side ceil(cbrt(n)), walls
    at x,y = 0 and x,y = L (L = side*spacing), floor z = 0."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(round(n ** (1.0 / 3.0), 6)))
    L = side * spacing
    idx = np.arange(n)
    gx, gy, gz = idx % side, (idx // side) % side, idx // (side * side)
    pos = np.stack([(gx + 0.5) * spacing, (gy + 0.5) * spacing, (gz + 0.5) * spacing + 0.3], axis=1)
    pos = (pos + rng.uniform(-jitter, jitter, size=(n, 3))).astype(np.float32)
    q = random_quats(rng, n)
    is_sphere = rng.random(n) < 0.5
    radius = rng.uniform(0.05, 0.25, size=n).astype(np.float32)
    sides = rng.uniform(0.1, 0.5, size=(n, 3)).astype(np.float32)
    density = rng.uniform(500.0, 2000.0, size=n).astype(np.float32)
    mass = np.zeros(n, np.float32)
    I3 = np.zeros((n, 3), np.float32)
    for i in range(n):
        if is_sphere[i]:
            r = mass_sphere(density[i], radius[i])
        else:
            r = mass_box(density[i], *sides[i])
        mass[i] = r[0]
        I3[i] = r[1:]
    bodies = _body_rows(pos, q, mass, I3)
    ng = n + 5
    cls = np.where(is_sphere, SPHERE, BOX).astype(np.int32)
    cls = np.concatenate([cls, np.full(5, PLANE, np.int32)])
    gbody = np.concatenate([np.arange(n, dtype=np.int32), np.full(5, -1, np.int32)])
    gdims = np.zeros((ng, 4), dtype=np.float32)
    gdims[:n, 0] = np.where(is_sphere, radius, sides[:, 0])
    gdims[:n, 1] = np.where(is_sphere, 0, sides[:, 1])
    gdims[:n, 2] = np.where(is_sphere, 0, sides[:, 2])
    gdims[n:] = np.array([[0, 0, 1, 0], [1, 0, 0, 0], [-1, 0, 0, -L], [0, 1, 0, 0], [0, -1, 0, -L]],
                         dtype=np.float32)
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene(f"pile{n}", bodies, cls, gbody, np.zeros((ng, 3), np.float32), gR, gdims,
                 dt=1.0 / 120.0, iterations=30, mu=0.6, maxc=4)


def capsule_pile(n: int = 96, seed: int = 2, spacing: float = 0.7) -> Scene:
    """Small mixed pile with capsules (r 0.05-0.2, length 0.1-0.6), spheres and
    boxes, so every pair type of the narrow phase occurs in the loop."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(round(n ** (1.0 / 3.0), 6)))
    L = side * spacing
    idx = np.arange(n)
    gx, gy, gz = idx % side, (idx // side) % side, idx // (side * side)
    pos = np.stack([(gx + 0.5) * spacing, (gy + 0.5) * spacing, (gz + 0.5) * spacing + 0.3], axis=1)
    pos = (pos + rng.uniform(-0.05, 0.05, size=(n, 3))).astype(np.float32)
    q = random_quats(rng, n)
    kind = rng.integers(0, 3, size=n)
    bodies = np.zeros((n, 20), np.float32)
    dims = np.zeros((n, 4), np.float32)
    cls = np.zeros(n, np.int32)
    for i in range(n):
        dens = rng.uniform(500, 2000)
        if kind[i] == 0:
            r = rng.uniform(0.05, 0.25)
            m = mass_sphere(dens, r)
            cls[i] = SPHERE
            dims[i, 0] = r
        elif kind[i] == 1:
            s = rng.uniform(0.1, 0.5, size=3)
            m = mass_box(dens, *s)
            cls[i] = BOX
            dims[i, :3] = s
        else:
            r = rng.uniform(0.05, 0.2)
            ln = rng.uniform(0.1, 0.6)
            # dMassSetCapsule (ode/src/mass.cpp:144-170), axis along z
            r32, l32 = np.float32(r), np.float32(ln)
            M1 = np.float32(math.pi) * r32 * r32 * l32 * np.float32(dens)
            M2 = np.float32(4.0 / 3.0) * np.float32(math.pi) * r32 * r32 * r32 * np.float32(dens)
            mt = M1 + M2
            Ia = M1 * (np.float32(0.25) * r32 * r32 + np.float32(1.0 / 12.0) * l32 * l32) + \
                M2 * (np.float32(0.4) * r32 * r32 + np.float32(0.375) * r32 * l32 + np.float32(0.25) * l32 * l32)
            Iz = (np.float32(0.5) * M1 + np.float32(0.4) * M2) * r32 * r32
            m = (mt, Ia, Ia, Iz)
            cls[i] = CAPSULE
            dims[i, 0] = r
            dims[i, 1] = ln
        bodies[i, 13] = m[0]
        bodies[i, 14:17] = m[1:]
    bodies[:, 0:3] = pos
    bodies[:, 3:7] = q
    ng = n + 5
    gcls = np.concatenate([cls, np.full(5, PLANE, np.int32)])
    gbody = np.concatenate([np.arange(n, dtype=np.int32), np.full(5, -1, np.int32)])
    gdims = np.concatenate([dims, np.array([[0, 0, 1, 0], [1, 0, 0, 0], [-1, 0, 0, -L], [0, 1, 0, 0],
                                            [0, -1, 0, -L]], dtype=np.float32)])
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene(f"capsule_pile{n}", bodies, gcls, gbody, np.zeros((ng, 3), np.float32), gR, gdims,
                 dt=1.0 / 120.0, iterations=20, mu=0.6, maxc=4)


def mass_capsule(density, r, length):
    """dMassSetCapsule (ode/src/mass.cpp:144-170), axis along the body z axis."""
    r32, l32, d32 = np.float32(r), np.float32(length), np.float32(density)
    pi = np.float32(math.pi)
    M1 = pi * r32 * r32 * l32 * d32
    M2 = np.float32(4.0 / 3.0) * pi * r32 * r32 * r32 * d32
    mt = M1 + M2
    Ia = M1 * (np.float32(0.25) * r32 * r32 + np.float32(1.0 / 12.0) * l32 * l32) + \
        M2 * (np.float32(0.4) * r32 * r32 + np.float32(0.375) * r32 * l32 + np.float32(0.25) * l32 * l32)
    Ib = (M1 * np.float32(0.5) + M2 * np.float32(0.4)) * r32 * r32
    return mt, Ia, Ia, Ib


def chains(n_chains: int = 8192, seed: int = 3, nmin: int = 2, nmax: int = 32, spacing: float = 17.0,
           hang: bool = False, density: float = 1000.0) -> Scene:
    """Articulated chains of capsules (radius 0.05 m, length U[0.2, 0.4] m,
    N ~ log-uniform in [nmin, nmax]) linked by alternating hinge and ball
    joints, the hinges limited to +-60 degrees about the chain plane's normal,
    with seeded random joint angles (+-50 degrees).  Independent chains sit on
    a square grid `spacing` m apart.  Dropped onto the plane z = 0 (mu 0.6), or
    with `hang` hanging from a ball joint to the environment at the first
    link's end, with no geoms (a joints-only scene).  dt 1/240, 20 iterations."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(math.sqrt(n_chains)))
    r = 0.05
    pos_l, q_l, mass_l, I_l, dims_l, joints = [], [], [], [], [], []
    nb = 0
    for c in range(n_chains):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        n = min(max(n, nmin), nmax)
        lens = rng.uniform(0.2, 0.4, size=n)
        yaw = rng.uniform(0, 2 * math.pi)
        ex = np.array([math.cos(yaw), math.sin(yaw), 0.0])   # chain direction in plane
        ey = np.array([-math.sin(yaw), math.cos(yaw), 0.0])  # hinge axis (plane normal)
        phi = rng.uniform(-0.3, 0.3)
        ang = np.concatenate([[phi], rng.uniform(-np.deg2rad(50), np.deg2rad(50), size=n - 1)])
        phis = np.cumsum(ang)
        dirs = np.stack([math.cos(p) * ex + math.sin(p) * np.array([0, 0, 1.0]) for p in phis])
        ends = np.zeros((n + 1, 3))
        for k in range(n):
            ends[k + 1] = ends[k] + dirs[k] * (lens[k] + 2 * r)
        base = np.array([(c % side + 0.5) * spacing, (c // side + 0.5) * spacing, 0.0])
        zmin = ends[:, 2].min()
        base[2] = (2.0 + (lens.sum() + 2 * r * n)) if hang else (0.3 - zmin)
        for k in range(n):
            centre = base + 0.5 * (ends[k] + ends[k + 1])
            # body z axis along the link: rotation taking (0,0,1) to dirs[k]
            d = dirs[k] / np.linalg.norm(dirs[k])
            axis = np.cross([0, 0, 1.0], d)
            sa, ca = np.linalg.norm(axis), d[2]
            if sa < 1e-9:
                q = np.array([1.0, 0, 0, 0])
            else:
                t = math.atan2(sa, ca)
                axis = axis / sa
                q = np.array([math.cos(t / 2), *(math.sin(t / 2) * axis)])
            m, i1, i2, i3 = mass_capsule(density, r, lens[k])
            pos_l.append(centre); q_l.append(q); mass_l.append(m); I_l.append((i1, i2, i3))
            dims_l.append((r, lens[k], 0, 0))
            if k == 0:
                if hang:
                    a = base + ends[0]
                    joints.append((1, nb, -1, *a) + (0,) * 14)
            else:
                a = base + ends[k]
                if k % 2 == 1:
                    joints.append((2, nb - 1, nb, *a, *ey, -math.pi / 3, math.pi / 3) + (0,) * 9)
                else:
                    joints.append((1, nb - 1, nb, *a) + (0,) * 14)
            nb += 1
    pos = np.asarray(pos_l, np.float32)
    q = np.asarray(q_l, np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    bodies = _body_rows(pos, q, np.asarray(mass_l, np.float32), np.asarray(I_l, np.float32))
    if hang:
        cls = np.zeros(0, np.int32)
        gbody = np.zeros(0, np.int32)
        gdims = np.zeros((0, 4), np.float32)
    else:
        cls = np.concatenate([np.full(nb, CAPSULE, np.int32), [PLANE]]).astype(np.int32)
        gbody = np.concatenate([np.arange(nb, dtype=np.int32), [-1]]).astype(np.int32)
        gdims = np.concatenate([np.asarray(dims_l, np.float32), [[0, 0, 1, 0]]]).astype(np.float32)
    ng = len(cls)
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene(f"chains{n_chains}" + ("_hanging" if hang else ""), bodies, cls, gbody,
                 np.zeros((ng, 3), np.float32), gR, gdims, dt=1.0 / 240.0, iterations=20, mu=0.6, maxc=4,
                 joints=np.asarray(joints, np.float32).reshape(-1, JOINT_COLS))


def vehicles(n_worlds: int = 65536, seed: int = 4, spacing: float = 12.0, hang: bool = False,
             obstacles: bool = True) -> Scene:
    """Four-wheeled vehicles, one per independent world: a box chassis
    2 x 1 x 0.5 m of 800 kg and four sphere wheels (r 0.3 m, 20 kg) on hinge2
    joints (axis 1 vertical, steering locked with lo = hi stop = 0; axis 2 the
    axle, motored at a seeded velocity U[-20, 20] rad/s with 200 N m), with
    suspension ERP 0.4 / CFM 1e-3, K ~ U{0..16} static box obstacles (sides
    U[0.2, 1] m) around each vehicle, on the plane z = 0; dt 1/120.  The
    worlds sit on a square grid `spacing` m apart.  With `hang` the chassis
    hangs from the environment by a ball joint at its centre top, no geoms
    (a joints-only scene)."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(math.sqrt(n_worlds)))
    pos_l, q_l, mass_l, I_l, cls_l, dims_l, body_l, gpos_l = [], [], [], [], [], [], [], []
    joints = []
    nb = 0
    cm, ci1, ci2, ci3 = mass_box(1.0, 2.0, 1.0, 0.5)
    cm_scale = np.float32(800.0) / cm
    wm, wi, _, _ = mass_sphere(1.0, 0.3)
    wm_scale = np.float32(20.0) / wm
    for c in range(n_worlds):
        base = np.array([(c % side + 0.5) * spacing, (c // side + 0.5) * spacing, 0.0])
        yaw = rng.uniform(0, 2 * math.pi)
        fwd = np.array([math.cos(yaw), math.sin(yaw), 0.0])
        left = np.array([-math.sin(yaw), math.cos(yaw), 0.0])
        zc = (3.0 if hang else 0.6)
        chassis = base + np.array([0, 0, zc])
        q = np.array([math.cos(yaw / 2), 0, 0, math.sin(yaw / 2)])
        pos_l.append(chassis); q_l.append(q); mass_l.append(cm * cm_scale)
        I_l.append((ci1 * cm_scale, ci2 * cm_scale, ci3 * cm_scale))
        cls_l.append(BOX); dims_l.append((2.0, 1.0, 0.5, 0)); body_l.append(nb); gpos_l.append((0, 0, 0))
        cb = nb
        nb += 1
        if hang:
            joints.append((1, cb, -1, *(chassis + np.array([0, 0, 0.25]))) + (0,) * 14)
        vel = rng.uniform(-20, 20)
        for sx in (-0.8, 0.8):
            for sy in (-0.7, 0.7):
                wp = chassis + sx * fwd + sy * left + np.array([0, 0, -0.3])
                pos_l.append(wp); q_l.append((1, 0, 0, 0)); mass_l.append(wm * wm_scale)
                I_l.append((wi * wm_scale,) * 3)
                cls_l.append(SPHERE); dims_l.append((0.3, 0, 0, 0)); body_l.append(nb); gpos_l.append((0, 0, 0))
                joints.append((6, cb, nb, *wp, 0, 0, 1, 0, 0, *left, vel, 200.0, 0.4, 1e-3, 0, 0))
                nb += 1
        if obstacles and not hang:
            for _ in range(int(rng.integers(0, 17))):
                sdim = rng.uniform(0.2, 1.0, size=3)
                r = rng.uniform(3.0, spacing / 2 - 0.8)
                a = rng.uniform(0, 2 * math.pi)
                p = base + np.array([r * math.cos(a), r * math.sin(a), sdim[2] / 2])
                cls_l.append(BOX); dims_l.append((*sdim, 0)); body_l.append(-1); gpos_l.append(p)
    pos = np.asarray(pos_l, np.float32)
    q = np.asarray(q_l, np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    bodies = _body_rows(pos, q, np.asarray(mass_l, np.float32), np.asarray(I_l, np.float32))
    if hang:
        cls = np.zeros(0, np.int32); gbody = np.zeros(0, np.int32)
        gdims = np.zeros((0, 4), np.float32); gpos = np.zeros((0, 3), np.float32)
    else:
        cls = np.asarray(cls_l + [PLANE], np.int32)
        gbody = np.asarray(body_l + [-1], np.int32)
        gdims = np.asarray(dims_l + [(0, 0, 1, 0)], np.float32)
        gpos = np.asarray(gpos_l + [(0, 0, 0)], np.float32)
    ng = len(cls)
    gR = np.zeros((ng, 12), dtype=np.float32)
    gR[:, [0, 5, 10]] = 1.0
    return Scene(f"vehicles{n_worlds}" + ("_hanging" if hang else ""), bodies, cls, gbody, gpos, gR, gdims,
                 dt=1.0 / 120.0, iterations=20, mu=0.8, maxc=4,
                 joints=np.asarray(joints, np.float32).reshape(-1, JOINT_COLS))
