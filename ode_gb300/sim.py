"""Scene drivers over the C API (ode_gb300.ode): build an ODE world from a
seeded Scene and step it the way an ODE program does.

Two loops are offered:
* ``compat`` -- the reference's own user loop (demo_boxstack.cpp:130-170):
  dSpaceCollide with a near callback that calls dCollide and makes one
  dJointCreateContact per point, then dWorldQuickStep and dJointGroupEmpty.
* ``fused``  -- gbodeSpaceCollideContacts (broad + narrow phase + contact
  joints without leaving the device), then dWorldQuickStep.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import ode
from .scenes import BOX, CAPSULE, PLANE, SPHERE, Scene


def make_joint(L, w, bodies, row):
    """Create and attach one joint from a scene joint row (scenes.Scene.joints)
    with the same call sequence an ODE program would use."""
    row = [float(x) for x in row] + [0.0] * (20 - len(row))
    t, b1, b2 = int(row[0]), int(row[1]), int(row[2])
    if t == 1:
        j = L.dJointCreateBall(w, None)
    elif t == 2:
        j = L.dJointCreateHinge(w, None)
    else:
        j = L.dJointCreateHinge2(w, None)
    L.dJointAttach(j, bodies[b1], bodies[b2] if b2 >= 0 else None)
    if t == 1:
        L.dJointSetBallAnchor(j, *row[3:6])
    elif t == 2:
        L.dJointSetHingeAnchor(j, *row[3:6])
        L.dJointSetHingeAxis(j, *row[6:9])
        L.dJointSetHingeParam(j, ode.dParamLoStop, row[9])
        L.dJointSetHingeParam(j, ode.dParamHiStop, row[10])
        if row[19] > 0:
            L.dJointSetHingeParam(j, ode.dParamVel, row[18])
            L.dJointSetHingeParam(j, ode.dParamFMax, row[19])
    else:
        L.dJointSetHinge2Anchor(j, *row[3:6])
        a1 = np.array(row[6:9] + [0.0], np.float32)
        a2 = np.array(row[11:14] + [0.0], np.float32)
        L.dJointSetHinge2Axes(j, ode.fptr(a1), ode.fptr(a2))
        L.dJointSetHinge2Param(j, ode.dParamLoStop, row[9])
        L.dJointSetHinge2Param(j, ode.dParamHiStop, row[10])
        L.dJointSetHinge2Param(j, ode.dParamVel2, row[14])
        L.dJointSetHinge2Param(j, ode.dParamFMax2, row[15])
        L.dJointSetHinge2Param(j, ode.dParamSuspensionERP, row[16])
        L.dJointSetHinge2Param(j, ode.dParamSuspensionCFM, row[17])
    return j


BULK_BODIES = 20000  # larger scenes are built through the bulk builders


class GBWorld:
    def __init__(self, scene: Scene, solver: int = ode.GBODE_SOLVER_COLOURED, dyn: bool = False,
                 iterations: int | None = None, stream=None):
        L = self.L = ode.load()
        self.scene = scene
        L.dInitODE2(0)
        self.w = L.dWorldCreate()
        if stream is not None:
            L.gbodeWorldSetStream(self.w, stream)
        L.dWorldSetGravity(self.w, *scene.gravity)
        L.dWorldSetERP(self.w, scene.erp)
        L.dWorldSetCFM(self.w, scene.cfm)
        L.dWorldSetQuickStepNumIterations(self.w, iterations or scene.iterations)
        L.dWorldSetQuickStepW(self.w, scene.w)
        L.dWorldSetContactMaxCorrectingVel(self.w, scene.max_vel)
        L.dWorldSetContactSurfaceLayer(self.w, scene.min_depth)
        if not dyn:
            zero = (ctypes.c_float * 1)(0.0)
            L.dWorldSetQuickStepDynamicIterationParameters(self.w, zero, zero, None)
        L.gbodeWorldSetSolver(self.w, solver)
        ls, as_, lt, at, mw = scene.damping
        L.dWorldSetDamping(self.w, ls, as_)
        L.dWorldSetLinearDampingThreshold(self.w, lt)
        L.dWorldSetAngularDampingThreshold(self.w, at)
        L.dWorldSetMaxAngularSpeed(self.w, mw)
        if scene.adis is not None:
            flag, lin, ang, steps, t, samples = scene.adis
            L.dWorldSetAutoDisableFlag(self.w, int(flag))
            L.dWorldSetAutoDisableLinearThreshold(self.w, lin)
            L.dWorldSetAutoDisableAngularThreshold(self.w, ang)
            L.dWorldSetAutoDisableSteps(self.w, int(steps))
            L.dWorldSetAutoDisableTime(self.w, t)
            L.dWorldSetAutoDisableAverageSamplesCount(self.w, int(samples))
        self.space = None
        if scene.nb > BULK_BODIES:
            self._build_bulk(scene)
        else:
            self._build_calls(scene)
        self.group = L.dJointGroupCreate(0)
        self.surface = ode.dSurfaceParameters()
        self.surface.mode = scene.surface_mode
        self.surface.mu = scene.mu
        self.surface.mu2 = scene.mu2
        self.surface.bounce = scene.bounce
        self.surface.bounce_vel = scene.bounce_vel
        self.surface.soft_erp = scene.soft_erp
        self.surface.soft_cfm = scene.soft_cfm
        self.body_index = {int(b): k for k, b in enumerate(self.bodies)}
        self._contacts = (ode.dContact * 16)()
        self.made = []   # contacts made by the last compat step: (b1, b2, dContact copy)
        self._cb = ode.dNearCallback(self._near)

    def _build_calls(self, scene):
        """One ODE call per object, as an ODE program builds a world."""
        L = self.L
        self.bodies = []
        m = ode.dMass()
        for row in scene.bodies:
            b = L.dBodyCreate(self.w)
            L.dBodySetPosition(b, *row[0:3])
            q = np.ascontiguousarray(row[3:7], np.float32)
            L.dBodySetQuaternion(b, ode.fptr(q))
            L.dBodySetLinearVel(b, *row[7:10])
            L.dBodySetAngularVel(b, *row[10:13])
            L.dMassSetParameters(ctypes.byref(m), row[13], 0, 0, 0, row[14], row[15], row[16], row[17], row[18],
                                 row[19])
            L.dBodySetMass(b, ctypes.byref(m))
            self.bodies.append(b)
        self.space = L.dHashSpaceCreate(None)
        L.dHashSpaceSetLevels(self.space, scene.hash_levels[0], scene.hash_levels[1])
        self.geoms = []
        for i in range(scene.ng):
            c, d = int(scene.geom_cls[i]), scene.geom_dims[i]
            if c == SPHERE:
                g = L.dCreateSphere(self.space, d[0])
            elif c == BOX:
                g = L.dCreateBox(self.space, d[0], d[1], d[2])
            elif c == CAPSULE:
                g = L.dCreateCapsule(self.space, d[0], d[1])
            elif c == PLANE:
                g = L.dCreatePlane(self.space, d[0], d[1], d[2], d[3])
            else:
                raise ValueError(c)
            bi = int(scene.geom_body[i])
            if bi >= 0:
                L.dGeomSetBody(g, self.bodies[bi])
            elif c != PLANE:
                L.dGeomSetPosition(g, *scene.geom_pos[i])
                R = np.ascontiguousarray(scene.geom_R[i], np.float32)
                L.dGeomSetRotation(g, ode.fptr(R))
            L.dGeomSetData(g, ctypes.c_void_p(i))
            self.geoms.append(g)
        self.joints = []
        if scene.joints is not None:
            for row in scene.joints:
                self.joints.append(make_joint(L, self.w, self.bodies, row))

    def _build_bulk(self, scene):
        """The same objects through the bulk builders (gbodeCreateBodies,
        gbodeCreateGeoms, gbodeCreateJoints): one call per kind."""
        L = self.L
        nb, ng = scene.nb, scene.ng
        ids = (ctypes.c_void_p * max(nb, 1))()
        rows = np.ascontiguousarray(scene.bodies, np.float32)
        if L.gbodeCreateBodies(self.w, nb, ode.fptr(rows), ids) != 1:
            raise RuntimeError(L.gbodeGetLastError().decode())
        self.bodies = list(ids[:nb])
        self.space = L.dHashSpaceCreate(None)
        L.dHashSpaceSetLevels(self.space, scene.hash_levels[0], scene.hash_levels[1])
        gb = (ctypes.c_void_p * max(ng, 1))()
        for i in range(ng):
            bi = int(scene.geom_body[i])
            gb[i] = ids[bi] if bi >= 0 else None
        gids = (ctypes.c_void_p * max(ng, 1))()
        cls = np.ascontiguousarray(scene.geom_cls, np.int32)
        dims = np.ascontiguousarray(scene.geom_dims, np.float32)
        pos = np.ascontiguousarray(scene.geom_pos, np.float32)
        R = np.ascontiguousarray(scene.geom_R, np.float32)
        if L.gbodeCreateGeoms(self.space, ng, cls.ctypes.data, ode.fptr(dims), ode.fptr(pos), ode.fptr(R), gb,
                              gids) != 1:
            raise RuntimeError(L.gbodeGetLastError().decode())
        self.geoms = list(gids[:ng])
        for i, g in enumerate(self.geoms):
            L.dGeomSetData(g, ctypes.c_void_p(i))
        self.joints = []
        if scene.joints is not None and len(scene.joints):
            jr = np.zeros((len(scene.joints), 20), np.float32)
            jr[:, :scene.joints.shape[1]] = scene.joints
            jids = (ctypes.c_void_p * len(jr))()
            if L.gbodeCreateJoints(self.w, len(jr), ode.fptr(jr), ids, jids) != 1:
                raise RuntimeError(L.gbodeGetLastError().decode())
            self.joints = list(jids)

    # ---------------------------------------------------------------- loops
    def _near(self, data, o1, o2):
        L = self.L
        maxc = self.scene.maxc
        for i in range(maxc):
            self._contacts[i].surface = self.surface
        b1, b2 = L.dGeomGetBody(o1), L.dGeomGetBody(o2)
        # demo_boxstack.cpp:140: bodies joined by a (non-contact) joint do not collide
        if b1 and b2 and L.dAreConnectedExcluding(b1, b2, ode.dJointTypeContact):
            return
        n = L.dCollide(o1, o2, maxc, ctypes.addressof(self._contacts[0].geom), ctypes.sizeof(ode.dContact))
        for i in range(n):
            j = L.dJointCreateContact(self.w, self.group, ctypes.byref(self._contacts[i]))
            L.dJointAttach(j, b1, b2)
            c = self._contacts[i]
            self.made.append((self.body_index.get(b1, -1) if b1 else -1, self.body_index.get(b2, -1) if b2 else -1,
                              np.array(c.geom.pos[:3]), np.array(c.geom.normal[:3]), float(c.geom.depth)))

    def step_compat(self):
        self.made = []
        self.L.dSpaceCollide(self.space, None, self._cb)
        ok = self.L.dWorldQuickStep(self.w, self.scene.dt)
        self.L.dJointGroupEmpty(self.group)
        return ok

    def step_graph(self):
        """A fused step replayed from a CUDA graph (gbodeWorldStepFused)."""
        L = self.L
        if not L.gbodeWorldStepFused(self.w, self.space, self.group, ctypes.byref(self.surface), self.scene.maxc,
                                     self.scene.dt, 1):
            raise RuntimeError(L.gbodeGetLastError().decode())
        return 1

    def step_dantzig(self, collide: str | None = None):
        """One dWorldStep (a dense LCP per island).  `collide`: None steps the
        joints alone (jointed scenes without geoms); "host" makes contact
        joints through dSpaceCollide and dCollide; "device" makes the contacts
        on the device (gbodeSpaceCollideContacts)."""
        L = self.L
        if collide == "host":
            self.made = []
            L.dSpaceCollide(self.space, None, self._cb)
        elif collide == "device":
            if not L.gbodeSpaceCollideContacts(self.space, self.w, self.group, ctypes.byref(self.surface),
                                               self.scene.maxc):
                raise RuntimeError(L.gbodeGetLastError().decode())
        elif collide is not None:
            raise ValueError(f"collide: {collide!r}")
        ok = L.dWorldStep(self.w, self.scene.dt)
        if collide is not None:
            L.dJointGroupEmpty(self.group)
        return ok

    def autotune(self, steps: int = 3, graph: bool = True) -> ode.gbodeTuning:
        """gbodeWorldAutotune on the fused step (the tuning steps advance the world)."""
        t = ode.gbodeTuning()
        if not self.L.gbodeWorldAutotune(self.w, self.space, self.group, ctypes.byref(self.surface), self.scene.maxc,
                                         self.scene.dt, steps, 1 if graph else 0, ctypes.byref(t)):
            raise RuntimeError(self.L.gbodeGetLastError().decode())
        return t

    def step_fused(self):
        L = self.L
        if not L.gbodeSpaceCollideContacts(self.space, self.w, self.group, ctypes.byref(self.surface),
                                           self.scene.maxc):
            raise RuntimeError(L.gbodeGetLastError().decode())
        ok = L.dWorldQuickStep(self.w, self.scene.dt)
        L.dJointGroupEmpty(self.group)
        return ok

    # ---------------------------------------------------------------- state
    def state(self) -> np.ndarray:
        out = np.zeros((len(self.bodies), 25), np.float32)
        self.L.gbodeWorldGetState(self.w, ode.fptr(out))
        return out

    def set_state(self, st: np.ndarray):
        st = np.ascontiguousarray(st, np.float32)
        self.L.gbodeWorldSetState(self.w, ode.fptr(st))

    def stats(self) -> ode.gbodeStepStats:
        s = ode.gbodeStepStats()
        self.L.gbodeWorldGetStepStats(self.w, ctypes.byref(s))
        return s

    def sync(self):
        if not self.L.gbodeWorldSynchronize(self.w):
            raise RuntimeError(self.L.gbodeGetLastError().decode())

    def last_rows(self) -> np.ndarray:
        n = self.L.gbodeWorldGetLastRows(self.w, None, 0)
        rows = np.zeros((max(n, 1), 20), np.float32)
        self.L.gbodeWorldGetLastRows(self.w, ode.fptr(rows), n)
        return rows[:n]

    def contacts(self) -> np.ndarray:
        n = self.L.gbodeWorldGetContacts(self.w, None, 0)
        out = np.zeros((max(n, 1), 12), np.float32)
        self.L.gbodeWorldGetContacts(self.w, ode.fptr(out), n)
        return out[:n]

    def last_residual(self):
        ce, ml = ctypes.c_double(0), ctypes.c_double(0)
        r = self.L.gbodeWorldLastResidual(self.w, ctypes.byref(ce), ctypes.byref(ml))
        return r, ce.value, ml.value

    def close(self):
        L = self.L
        L.dJointGroupDestroy(self.group)
        L.dSpaceDestroy(self.space)
        L.dWorldDestroy(self.w)


def step_contacts(world: GBWorld, cb: np.ndarray, cs: np.ndarray, mode: int, stepper: bool = False):
    """One dWorldQuickStep (dWorldStep with `stepper`) on an explicit contact
    list (the golden snapshots' contact joints, created and attached in their
    recorded order)."""
    L = world.L
    c = ode.dContact()
    for k in range(cb.shape[0]):
        c.surface.mode = mode
        c.surface.mu, c.surface.mu2 = float(cs[k, 7]), float(cs[k, 8])
        c.surface.bounce, c.surface.bounce_vel = float(cs[k, 9]), float(cs[k, 10])
        c.surface.soft_erp, c.surface.soft_cfm = float(cs[k, 11]), float(cs[k, 12])
        c.surface.slip1, c.surface.slip2 = float(cs[k, 13]), float(cs[k, 14])
        for q in range(3):
            c.geom.pos[q] = float(cs[k, q])
            c.geom.normal[q] = float(cs[k, 3 + q])
        c.geom.depth = float(cs[k, 6])
        j = L.dJointCreateContact(world.w, world.group, ctypes.byref(c))
        b1 = world.bodies[cb[k, 0]] if cb[k, 0] >= 0 else None
        b2 = world.bodies[cb[k, 1]] if cb[k, 1] >= 0 else None
        L.dJointAttach(j, b1, b2)
    ok = (L.dWorldStep if stepper else L.dWorldQuickStep)(world.w, world.scene.dt)
    return ok
