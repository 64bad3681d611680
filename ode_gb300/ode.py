"""ctypes binding of libgbode.so: ODE's C API for the rigid-body hot path.

This is the same interface the reference exposes (include/ode/*.h) with the
same names and argument meaning, so Python code here reads like an ODE
program: create a world and a hash space, add bodies and geoms, call
dSpaceCollide with a near callback that calls dCollide and
dJointCreateContact, then dWorldQuickStep and dJointGroupEmpty.

Loading fails loudly when the CUDA library is missing: there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbode.so")

dReal = ctypes.c_float
dVector3 = dReal * 4
dMatrix3 = dReal * 12
dQuaternion = dReal * 4
ID = ctypes.c_void_p


class dSurfaceParameters(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("mu", dReal), ("mu2", dReal), ("rho", dReal), ("rho2", dReal),
                ("rhoN", dReal), ("bounce", dReal), ("bounce_vel", dReal), ("soft_erp", dReal),
                ("soft_cfm", dReal), ("motion1", dReal), ("motion2", dReal), ("motionN", dReal),
                ("slip1", dReal), ("slip2", dReal)]


class dContactGeom(ctypes.Structure):
    _fields_ = [("pos", dVector3), ("normal", dVector3), ("depth", dReal), ("g1", ID), ("g2", ID),
                ("side1", ctypes.c_int), ("side2", ctypes.c_int)]


class dContact(ctypes.Structure):
    _fields_ = [("surface", dSurfaceParameters), ("geom", dContactGeom), ("fdir1", dVector3)]


class dMass(ctypes.Structure):
    _fields_ = [("mass", dReal), ("c", dVector3), ("I", dMatrix3)]


class dJointFeedback(ctypes.Structure):
    _fields_ = [("f1", dVector3), ("t1", dVector3), ("f2", dVector3), ("t2", dVector3)]


class gbodeTuning(ctypes.Structure):
    _fields_ = [("blocks", ctypes.c_int), ("passes", ctypes.c_int), ("check_every", ctypes.c_int),
                ("ms_per_step", ctypes.c_float), ("candidates", ctypes.c_int), ("threads", ctypes.c_int),
                ("chunk_rows", ctypes.c_int), ("two_level", ctypes.c_int), ("momentum", ctypes.c_float)]


class gbodeStepStats(ctypes.Structure):
    _fields_ = [("contacts", ctypes.c_int), ("rows", ctypes.c_int), ("colours", ctypes.c_int),
                ("iterations", ctypes.c_int), ("residual", ctypes.c_float), ("pairs", ctypes.c_int),
                ("solve_ms", ctypes.c_float), ("step_ms", ctypes.c_float), ("sleeping", ctypes.c_int),
                ("interior_colours", ctypes.c_int), ("interior_rows", ctypes.c_int),
                ("neighbour_waits", ctypes.c_int), ("cross_classes", ctypes.c_int),
                ("momentum", ctypes.c_float)]


dNearCallback = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ID, ID)

# (name, restype, argtypes) for every exported function declared in include/gbode.h
_F = ctypes.POINTER(ctypes.c_float)
_PROTOS = [
    ("dInitODE2", ctypes.c_int, [ctypes.c_uint]), ("dInitODE", None, []),
    ("dAllocateODEDataForThread", ctypes.c_int, [ctypes.c_uint]), ("dCloseODE", None, []),
    ("dWorldCreate", ID, []), ("dWorldDestroy", None, [ID]),
    ("dWorldSetGravity", None, [ID, dReal, dReal, dReal]), ("dWorldGetGravity", None, [ID, _F]),
    ("dWorldSetERP", None, [ID, dReal]), ("dWorldGetERP", dReal, [ID]),
    ("dWorldSetCFM", None, [ID, dReal]), ("dWorldGetCFM", dReal, [ID]),
    ("dWorldQuickStep", ctypes.c_int, [ID, dReal]), ("dWorldStep", ctypes.c_int, [ID, dReal]),
    ("dWorldSetQuickStepNumIterations", None, [ID, ctypes.c_int]),
    ("dWorldGetQuickStepNumIterations", ctypes.c_int, [ID]),
    ("dWorldSetQuickStepW", None, [ID, dReal]), ("dWorldGetQuickStepW", dReal, [ID]),
    ("dWorldSetQuickStepDynamicIterationParameters", None, [ID, _F, _F, _F]),
    ("dWorldGetQuickStepDynamicIterationParameters", None, [ID, _F, _F, _F]),
    ("dWorldSetContactMaxCorrectingVel", None, [ID, dReal]), ("dWorldGetContactMaxCorrectingVel", dReal, [ID]),
    ("dWorldSetContactSurfaceLayer", None, [ID, dReal]), ("dWorldGetContactSurfaceLayer", dReal, [ID]),
    ("dWorldSetLinearDamping", None, [ID, dReal]), ("dWorldSetAngularDamping", None, [ID, dReal]),
    ("dWorldSetDamping", None, [ID, dReal, dReal]),
    ("dWorldSetLinearDampingThreshold", None, [ID, dReal]), ("dWorldSetAngularDampingThreshold", None, [ID, dReal]),
    ("dWorldGetLinearDamping", dReal, [ID]), ("dWorldGetAngularDamping", dReal, [ID]),
    ("dWorldGetLinearDampingThreshold", dReal, [ID]), ("dWorldGetAngularDampingThreshold", dReal, [ID]),
    ("dWorldSetMaxAngularSpeed", None, [ID, dReal]), ("dWorldGetMaxAngularSpeed", dReal, [ID]),
    ("dWorldSetAutoDisableFlag", None, [ID, ctypes.c_int]), ("dWorldGetAutoDisableFlag", ctypes.c_int, [ID]),
    ("dWorldSetAutoDisableLinearThreshold", None, [ID, dReal]), ("dWorldGetAutoDisableLinearThreshold", dReal, [ID]),
    ("dWorldSetAutoDisableAngularThreshold", None, [ID, dReal]), ("dWorldGetAutoDisableAngularThreshold", dReal, [ID]),
    ("dWorldSetAutoDisableAverageSamplesCount", None, [ID, ctypes.c_uint]),
    ("dWorldGetAutoDisableAverageSamplesCount", ctypes.c_int, [ID]),
    ("dWorldSetAutoDisableSteps", None, [ID, ctypes.c_int]), ("dWorldGetAutoDisableSteps", ctypes.c_int, [ID]),
    ("dWorldSetAutoDisableTime", None, [ID, dReal]), ("dWorldGetAutoDisableTime", dReal, [ID]),
    ("dBodyCreate", ID, [ID]), ("dBodyDestroy", None, [ID]),
    ("dBodySetData", None, [ID, ctypes.c_void_p]), ("dBodyGetData", ctypes.c_void_p, [ID]),
    ("dBodySetPosition", None, [ID, dReal, dReal, dReal]), ("dBodySetRotation", None, [ID, _F]),
    ("dBodySetQuaternion", None, [ID, _F]), ("dBodySetLinearVel", None, [ID, dReal, dReal, dReal]),
    ("dBodySetAngularVel", None, [ID, dReal, dReal, dReal]),
    ("dBodyGetPosition", _F, [ID]), ("dBodyGetRotation", _F, [ID]), ("dBodyGetQuaternion", _F, [ID]),
    ("dBodyGetLinearVel", _F, [ID]), ("dBodyGetAngularVel", _F, [ID]),
    ("dBodySetMass", None, [ID, ctypes.POINTER(dMass)]), ("dBodyGetMass", None, [ID, ctypes.POINTER(dMass)]),
    ("dBodyAddForce", None, [ID, dReal, dReal, dReal]), ("dBodyAddTorque", None, [ID, dReal, dReal, dReal]),
    ("dBodyGetForce", _F, [ID]), ("dBodyGetTorque", _F, [ID]),
    ("dBodySetGyroscopicMode", None, [ID, ctypes.c_int]), ("dBodyGetGyroscopicMode", ctypes.c_int, [ID]),
    ("dBodyGetNumJoints", ctypes.c_int, [ID]),
    ("dBodySetLinearDamping", None, [ID, dReal]), ("dBodySetAngularDamping", None, [ID, dReal]),
    ("dBodySetDamping", None, [ID, dReal, dReal]),
    ("dBodySetLinearDampingThreshold", None, [ID, dReal]), ("dBodySetAngularDampingThreshold", None, [ID, dReal]),
    ("dBodySetDampingDefaults", None, [ID]),
    ("dBodyGetLinearDamping", dReal, [ID]), ("dBodyGetAngularDamping", dReal, [ID]),
    ("dBodyGetLinearDampingThreshold", dReal, [ID]), ("dBodyGetAngularDampingThreshold", dReal, [ID]),
    ("dBodySetMaxAngularSpeed", None, [ID, dReal]), ("dBodyGetMaxAngularSpeed", dReal, [ID]),
    ("dBodyEnable", None, [ID]), ("dBodyDisable", None, [ID]), ("dBodyIsEnabled", ctypes.c_int, [ID]),
    ("dBodySetAutoDisableFlag", None, [ID, ctypes.c_int]), ("dBodyGetAutoDisableFlag", ctypes.c_int, [ID]),
    ("dBodySetAutoDisableLinearThreshold", None, [ID, dReal]), ("dBodyGetAutoDisableLinearThreshold", dReal, [ID]),
    ("dBodySetAutoDisableAngularThreshold", None, [ID, dReal]), ("dBodyGetAutoDisableAngularThreshold", dReal, [ID]),
    ("dBodySetAutoDisableAverageSamplesCount", None, [ID, ctypes.c_uint]),
    ("dBodyGetAutoDisableAverageSamplesCount", ctypes.c_int, [ID]),
    ("dBodySetAutoDisableSteps", None, [ID, ctypes.c_int]), ("dBodyGetAutoDisableSteps", ctypes.c_int, [ID]),
    ("dBodySetAutoDisableTime", None, [ID, dReal]), ("dBodyGetAutoDisableTime", dReal, [ID]),
    ("dBodySetAutoDisableDefaults", None, [ID]),
    ("dMassSetZero", None, [ctypes.POINTER(dMass)]),
    ("dMassSetParameters", None, [ctypes.POINTER(dMass), dReal, dReal, dReal, dReal, dReal, dReal, dReal, dReal,
                                  dReal, dReal]),
    ("dMassSetSphere", None, [ctypes.POINTER(dMass), dReal, dReal]),
    ("dMassSetSphereTotal", None, [ctypes.POINTER(dMass), dReal, dReal]),
    ("dMassSetCapsule", None, [ctypes.POINTER(dMass), dReal, ctypes.c_int, dReal, dReal]),
    ("dMassSetBox", None, [ctypes.POINTER(dMass), dReal, dReal, dReal, dReal]),
    ("dMassSetBoxTotal", None, [ctypes.POINTER(dMass), dReal, dReal, dReal, dReal]),
    ("dHashSpaceCreate", ID, [ID]), ("dHashSpaceSetLevels", None, [ID, ctypes.c_int, ctypes.c_int]),
    ("dHashSpaceGetLevels", None, [ID, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("dSpaceDestroy", None, [ID]), ("dSpaceSetCleanup", None, [ID, ctypes.c_int]),
    ("dSpaceGetNumGeoms", ctypes.c_int, [ID]), ("dSpaceCollide", None, [ID, ctypes.c_void_p, dNearCallback]),
    ("dCreateSphere", ID, [ID, dReal]), ("dCreateBox", ID, [ID, dReal, dReal, dReal]),
    ("dCreateCapsule", ID, [ID, dReal, dReal]), ("dCreatePlane", ID, [ID, dReal, dReal, dReal, dReal]),
    ("dGeomDestroy", None, [ID]), ("dGeomSetData", None, [ID, ctypes.c_void_p]),
    ("dGeomGetData", ctypes.c_void_p, [ID]), ("dGeomSetBody", None, [ID, ID]), ("dGeomGetBody", ID, [ID]),
    ("dGeomSetPosition", None, [ID, dReal, dReal, dReal]), ("dGeomSetRotation", None, [ID, _F]),
    ("dGeomGetPosition", _F, [ID]), ("dGeomGetRotation", _F, [ID]), ("dGeomGetClass", ctypes.c_int, [ID]),
    ("dGeomGetAABB", None, [ID, _F]),
    ("dCollide", ctypes.c_int, [ID, ID, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    ("dBoxBox", ctypes.c_int, [_F, _F, _F, _F, _F, _F, _F, _F, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                               ctypes.c_void_p, ctypes.c_int]),
    ("dJointGroupCreate", ID, [ctypes.c_int]), ("dJointGroupDestroy", None, [ID]),
    ("dJointGroupEmpty", None, [ID]), ("dJointCreateContact", ID, [ID, ID, ctypes.POINTER(dContact)]),
    ("dJointAttach", None, [ID, ID, ID]), ("dJointDestroy", None, [ID]),
    ("dJointSetFeedback", None, [ID, ctypes.POINTER(dJointFeedback)]),
    ("dJointGetFeedback", ctypes.POINTER(dJointFeedback), [ID]), ("dJointGetBody", ID, [ID, ctypes.c_int]),
    ("dAreConnectedExcluding", ctypes.c_int, [ID, ID, ctypes.c_int]),
    ("dRand", ctypes.c_ulong, []), ("dRandInt", ctypes.c_int, [ctypes.c_int]),
    ("dRandSetSeed", None, [ctypes.c_ulong]), ("dRandGetSeed", ctypes.c_ulong, []), ("dTestRand", ctypes.c_int, []),
    ("dRSetIdentity", None, [_F]), ("dRFromAxisAndAngle", None, [_F, dReal, dReal, dReal, dReal]),
    ("dRfromQ", None, [_F, _F]), ("dQFromAxisAndAngle", None, [_F, dReal, dReal, dReal, dReal]),
    ("gbodeWorldSetSolver", None, [ID, ctypes.c_int]), ("gbodeWorldGetSolver", ctypes.c_int, [ID]),
    ("gbodeWorldSetResidualTarget", None, [ID, dReal, ctypes.c_int, ctypes.c_int]),
    ("gbodeWorldSetWarmStart", None, [ID, ctypes.c_int, dReal]),
    ("gbodeWorldSetSolverBlocks", None, [ID, ctypes.c_int]), ("gbodeWorldGetSolverBlocks", ctypes.c_int, [ID]),
    ("gbodeWorldSetManifoldPasses", None, [ID, ctypes.c_int]), ("gbodeWorldGetManifoldPasses", ctypes.c_int, [ID]),
    ("gbodeWorldSetTwoLevelSweep", None, [ID, ctypes.c_int]), ("gbodeWorldGetTwoLevelSweep", ctypes.c_int, [ID]),
    ("gbodeWorldSetSweepSync", None, [ID, ctypes.c_int]), ("gbodeWorldGetSweepSync", ctypes.c_int, [ID]),
    ("gbodeWorldSetResidualChecks", None, [ID, ctypes.c_int, ctypes.c_int]),
    ("gbodeWorldSetCrossClasses", None, [ID, ctypes.c_int]), ("gbodeWorldGetCrossClasses", ctypes.c_int, [ID]),
    ("gbodeWorldSetSweepMomentum", None, [ID, ctypes.c_float]), ("gbodeWorldGetSweepMomentum", ctypes.c_float, [ID]),
    ("gbodeTestInject", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("gbodeWorldSetSolverTiles", None, [ID, ctypes.c_int, ctypes.c_int]),
    ("gbodeWorldGetSolverTiles", None, [ID, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("gbodeSolveLCPBatch", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    ("gbodeWorldAutotune", ctypes.c_int, [ID, ID, ID, ctypes.c_void_p, ctypes.c_int, dReal, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p]),
    ("gbodeWorldSaveSnapshot", ctypes.c_int, [ID]), ("gbodeWorldRestoreSnapshot", ctypes.c_int, [ID]),
    ("gbodeWorldDropSnapshot", None, [ID]),
    ("gbodeSpaceCollideContacts", ctypes.c_int, [ID, ID, ID, ctypes.POINTER(dSurfaceParameters), ctypes.c_int]),
    ("gbodeHashSpaceSetExactPairs", None, [ID, ctypes.c_int]),
    ("gbodeWorldSetStream", None, [ID, ctypes.c_void_p]), ("gbodeWorldGetStream", ctypes.c_void_p, [ID]),
    ("gbodeWorldSynchronize", ctypes.c_int, [ID]),
    ("gbodeWorldGetStepStats", None, [ID, ctypes.POINTER(gbodeStepStats)]),
    ("gbodeWorldSetTiming", None, [ID, ctypes.c_int]),
    ("gbodeWorldLastResidual", ctypes.c_double, [ID, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.POINTER(ctypes.c_double)]),
    ("gbodeWorldGetLastRows", ctypes.c_int, [ID, _F, ctypes.c_int]),
    ("gbodeWorldGetContacts", ctypes.c_int, [ID, _F, ctypes.c_int]),
    ("gbodeWorldGetResidualHistory", ctypes.c_int, [ID, _F, ctypes.c_int]),
    ("gbodeWorldGetResidualSweeps", ctypes.c_int, [ID, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    ("gbodeGetLastError", ctypes.c_char_p, []), ("gbodeKernelLaunchCount", ctypes.c_longlong, []),
    ("gbodeWorldGetBodyCount", ctypes.c_int, [ID]), ("gbodeWorldGetState", None, [ID, _F]),
    ("gbodeWorldSetState", None, [ID, _F]),
    ("dAreConnected", ctypes.c_int, [ID, ID]),
    ("dJointCreateBall", ID, [ID, ID]), ("dJointCreateHinge", ID, [ID, ID]),
    ("dJointGetType", ctypes.c_int, [ID]),
    ("dJointSetBallAnchor", None, [ID, dReal, dReal, dReal]),
    ("dJointSetBallParam", None, [ID, ctypes.c_int, dReal]),
    ("dJointSetHingeAnchor", None, [ID, dReal, dReal, dReal]),
    ("dJointSetHingeAxis", None, [ID, dReal, dReal, dReal]),
    ("dJointSetHingeAxisOffset", None, [ID, dReal, dReal, dReal, dReal]),
    ("dJointGetHinge2Axis1", None, [ID, _F]), ("dJointGetHinge2Axis2", None, [ID, _F]),
    ("dSafeNormalize3", ctypes.c_int, [_F]), ("dNormalize3", None, [_F]),
    ("dJointSetHingeParam", None, [ID, ctypes.c_int, dReal]),
    ("dJointGetBallAnchor", None, [ID, _F]), ("dJointGetBallParam", dReal, [ID, ctypes.c_int]),
    ("dJointGetHingeAnchor", None, [ID, _F]), ("dJointGetHingeAxis", None, [ID, _F]),
    ("dJointGetHingeParam", dReal, [ID, ctypes.c_int]), ("dJointGetHingeAngle", dReal, [ID]),
    ("dJointCreateHinge2", ID, [ID, ID]),
    ("dJointSetHinge2Anchor", None, [ID, dReal, dReal, dReal]),
    ("dJointSetHinge2Axes", None, [ID, _F, _F]),
    ("dJointSetHinge2Axis1", None, [ID, dReal, dReal, dReal]),
    ("dJointSetHinge2Axis2", None, [ID, dReal, dReal, dReal]),
    ("dJointSetHinge2Param", None, [ID, ctypes.c_int, dReal]),
    ("dJointGetHinge2Anchor", None, [ID, _F]), ("dJointGetHinge2Param", dReal, [ID, ctypes.c_int]),
    ("dJointGetHinge2Angle1", dReal, [ID]),
    ("gbodeCreateBodies", ctypes.c_int, [ID, ctypes.c_int, _F, ctypes.c_void_p]),
    ("gbodeCreateGeoms", ctypes.c_int, [ID, ctypes.c_int, ctypes.c_void_p, _F, _F, _F, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    ("gbodeCreateJoints", ctypes.c_int, [ID, ctypes.c_int, _F, ctypes.c_void_p, ctypes.c_void_p]),
    ("gbodeWorldStepFused", ctypes.c_int, [ID, ID, ID, ctypes.c_void_p, ctypes.c_int, dReal, ctypes.c_int]),
    ("gbodeMlpParamCount", ctypes.c_int, []),
    ("gbodeMlpLossGrad", ctypes.c_int, [_F, _F, _F, ctypes.c_int, _F, _F]),
    ("gbodeMlpTrain", ctypes.c_int, [_F, _F, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_uint, _F, _F]),
    ("gbodeMlpPredict", ctypes.c_int, [_F, _F, ctypes.c_int, _F]),
    ("gbodeWorldSetLearnedWarmStart", ctypes.c_int, [ID, _F, ctypes.c_int]),
    ("gbodeWorldSetLearnCapture", None, [ID, ctypes.c_int]),
    ("gbodeWorldGetLearnSamples", ctypes.c_int, [ID, _F, ctypes.c_int]),
    ("gbodeWorldGetLearnedStats", None, [ID, _F]),
    ("gbodeCollidePairsNoAlloc", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_void_p]),
]

GBODE_NOALLOC_MAX_PAIRS = 8192  # gbodeCollidePairsNoAlloc's largest batch
GBODE_TEST_OFF, GBODE_TEST_BARRIER, GBODE_TEST_STAGE, GBODE_TEST_ALLOC = 0, 1, 2, 3
GBODE_TEST_CONTACT_CAP, GBODE_TEST_ROW_CAP, GBODE_TEST_COLOUR_CAP, GBODE_TEST_ALLOC_PENDING = 4, 5, 6, 7
GBODE_MLP_NPARAMS = 35099       # learned warm start parameters

dJointTypeBall, dJointTypeHinge, dJointTypeContact, dJointTypeHinge2 = 1, 2, 4, 6
dParamLoStop, dParamHiStop, dParamVel, dParamFMax, dParamCFM, dParamERP = 0, 1, 2, 5, 8, 13
dParamSuspensionERP, dParamSuspensionCFM = 11, 12
dParamVel2, dParamFMax2 = 0x102, 0x105

GBODE_SYNC_NEIGHBOURS, GBODE_SYNC_GRID = 0, 1  # gbodeWorldSetSweepSync
GBODE_CHECKS_PREDICTED, GBODE_CHECKS_FIXED = 0, 1  # gbodeWorldSetResidualChecks
GBODE_SOLVER_COLOURED = 0
GBODE_SOLVER_REFERENCE_ORDER = 1

_lib = None


def load(path: str = LIB_PATH):
    """Load libgbode.so and declare every exported prototype.  Raises if the
    library has not been built: the GPU path has no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgbode.so not found at {path}; build it with ode_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, res, args in _PROTOS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_names():
    return [p[0] for p in _PROTOS]


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)


def vec(p, n=3):
    return np.ctypeslib.as_array(p, shape=(n,)).copy()
