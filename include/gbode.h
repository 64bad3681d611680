/* gbode -- GB300-native rigid-body step behind ODE's C API.
 *
 * libgbode.so exports the subset of the Open Dynamics Engine 0.16 C API that
 * the rigid-body hot path uses (hash-space broad phase -> dCollide contact
 * generation for sphere/box/capsule/plane -> contact joints -> dWorldQuickStep
 * -> body integration), with ODE's exact names, argument meanings, struct
 * layouts and return conventions (dReal = float, i.e. ODE's dSINGLE build), so
 * an ODE program that uses only this subset links against it unchanged.  The
 * numerical work runs in hand-written CUDA kernels on one GPU; host code keeps
 * only handles, parameters and the near-callback loop.
 *
 * Each declaration cites the reference declaration it replaces
 * (include/ode/<file>:<line> in the reference tree).  The gbode* functions at
 * the end have no ODE counterpart: they expose the fused GPU path (contacts
 * that never leave the device) and GPU-only controls.
 */
#ifndef GBODE_H
#define GBODE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar and vector types: include/ode/common.h:270-275, odeconfig.h */
typedef float dReal;
typedef dReal dVector3[4];
typedef dReal dVector4[4];
typedef dReal dMatrix3[4 * 3];
typedef dReal dQuaternion[4];

/* ---- opaque handles: include/ode/common.h:330-345 */
typedef struct dxWorld *dWorldID;
typedef struct dxSpace *dSpaceID;
typedef struct dxBody *dBodyID;
typedef struct dxGeom *dGeomID;
typedef struct dxJoint *dJointID;
typedef struct dxJointGroup *dJointGroupID;

/* ---- geom classes: include/ode/collision.h:881-905 */
enum { dSphereClass = 0, dBoxClass, dCapsuleClass, dCylinderClass, dPlaneClass };

/* ---- contact records: include/ode/contact.h:28-103 (identical layout) */
enum {
    dContactMu2 = 0x001, dContactAxisDep = 0x001, dContactFDir1 = 0x002, dContactBounce = 0x004,
    dContactSoftERP = 0x008, dContactSoftCFM = 0x010, dContactMotion1 = 0x020, dContactMotion2 = 0x040,
    dContactMotionN = 0x080, dContactSlip1 = 0x100, dContactSlip2 = 0x200, dContactRolling = 0x400,
    dContactApprox0 = 0x0000, dContactApprox1_1 = 0x1000, dContactApprox1_2 = 0x2000,
    dContactApprox1_N = 0x4000, dContactApprox1 = 0x7000
};
typedef struct dSurfaceParameters {
    int mode;
    dReal mu, mu2, rho, rho2, rhoN, bounce, bounce_vel, soft_erp, soft_cfm;
    dReal motion1, motion2, motionN, slip1, slip2;
} dSurfaceParameters;
typedef struct dContactGeom {
    dVector3 pos;
    dVector3 normal;
    dReal depth;
    dGeomID g1, g2;
    int side1, side2;
} dContactGeom;
typedef struct dContact {
    dSurfaceParameters surface;
    dContactGeom geom;
    dVector3 fdir1;
} dContact;

/* ---- mass: include/ode/mass.h:31-96 */
typedef struct dMass {
    dReal mass;
    dVector3 c;
    dMatrix3 I;
} dMass;

/* ---- joint feedback: include/ode/common.h:389-396 */
typedef struct dJointFeedback {
    dVector3 f1, t1, f2, t2;
} dJointFeedback;

/* near callback: include/ode/collision_space.h:49 */
typedef void dNearCallback(void *data, dGeomID o1, dGeomID o2);

/* ---- init: include/ode/odeinit.h:119, :177, :227 */
int dInitODE2(unsigned int uiInitFlags);
void dInitODE(void);
int dAllocateODEDataForThread(unsigned int uiAllocateFlags);
void dCloseODE(void);

/* ---- world: include/ode/objects.h:77-560 */
dWorldID dWorldCreate(void);
void dWorldDestroy(dWorldID w);
void dWorldSetGravity(dWorldID w, dReal x, dReal y, dReal z);
void dWorldGetGravity(dWorldID w, dVector3 gravity);
void dWorldSetERP(dWorldID w, dReal erp);
dReal dWorldGetERP(dWorldID w);
void dWorldSetCFM(dWorldID w, dReal cfm);
dReal dWorldGetCFM(dWorldID w);
int dWorldQuickStep(dWorldID w, dReal stepsize);
/* dWorldStep (ode.cpp:1828-1845, step.cpp): the rows as dWorldQuickStep forms
 * them, then for every island (bodies connected by this step's contact joints
 * and ball/hinge/hinge2 joints) the dense mixed LCP A lambda = b + w,
 * A = J M^-1 J^T + diag(cfm), solved exactly on the device as the reference's
 * Dantzig solver defines it (friction rows bounded by the normal multipliers
 * of the problem without them), FP64 with FP32 factorisations; one thread
 * block per island, at most 2048 rows an island.  The contacts are the
 * attached contact joints (dJointCreateContact) or the device's own from
 * gbodeSpaceCollideContacts, not both in one step.  Returns 0 on failure
 * (gbodeGetLastError). */
int dWorldStep(dWorldID w, dReal stepsize);

/* The dense LCP solver of dWorldStep for a batch of problems given directly
 * (the role of the reference's internal dSolveLCP, lcp.cpp:836-1160): for
 * each problem p, A x = b + w with A = A[p] (n x n, row-major, symmetric
 * positive definite), the first nub variables unbounded, the rest in
 * [lo, hi] with x = lo => w >= 0, x = hi => w <= 0, else w = 0; findex
 * (optional) as in dWorldStep.  FP64 in and out, one thread block a problem,
 * n <= 2048.  Host arrays; returns 0 if a problem did not solve. */
int gbodeSolveLCPBatch(int count, int n, const double *A, const double *b, const double *lo, const double *hi, int nub,
                       const int *findex, double *x, double *w);
void dWorldSetQuickStepNumIterations(dWorldID w, int num);
int dWorldGetQuickStepNumIterations(dWorldID w);
void dWorldSetQuickStepW(dWorldID w, dReal over_relaxation);
dReal dWorldGetQuickStepW(dWorldID w);
void dWorldSetQuickStepDynamicIterationParameters(dWorldID w, const dReal *ptr_iteration_premature_exit_delta,
                                                  const dReal *ptr_max_num_extra_factor,
                                                  const dReal *ptr_extra_iteration_requirement_delta);
void dWorldGetQuickStepDynamicIterationParameters(dWorldID w, dReal *out_iteration_premature_exit_delta,
                                                  dReal *out_max_num_extra_factor,
                                                  dReal *out_extra_iteration_requirement_delta);
void dWorldSetContactMaxCorrectingVel(dWorldID w, dReal vel);
dReal dWorldGetContactMaxCorrectingVel(dWorldID w);
void dWorldSetContactSurfaceLayer(dWorldID w, dReal depth);
dReal dWorldGetContactSurfaceLayer(dWorldID w);
/* damping and the angular speed cap, world defaults copied into bodies by
 * dBodyCreate: include/ode/objects.h:430-520, ode/src/ode.cpp:1950-2048.
 * Applied in the integration step (ode/src/util.cpp:583-593, :675-691):
 * angular speed above the cap is scaled down to it before the move; after
 * the move a velocity whose squared norm exceeds the squared threshold is
 * multiplied by (1 - scale).  Thresholds are stored squared; scale 0 and an
 * infinite cap switch the terms off. */
void dWorldSetLinearDamping(dWorldID w, dReal scale);
void dWorldSetAngularDamping(dWorldID w, dReal scale);
void dWorldSetDamping(dWorldID w, dReal linear_scale, dReal angular_scale);
void dWorldSetLinearDampingThreshold(dWorldID w, dReal threshold);
void dWorldSetAngularDampingThreshold(dWorldID w, dReal threshold);
dReal dWorldGetLinearDamping(dWorldID w);
dReal dWorldGetAngularDamping(dWorldID w);
dReal dWorldGetLinearDampingThreshold(dWorldID w);
dReal dWorldGetAngularDampingThreshold(dWorldID w);
void dWorldSetMaxAngularSpeed(dWorldID w, dReal max_speed);
dReal dWorldGetMaxAngularSpeed(dWorldID w);
/* auto-disable defaults copied into bodies by dBodyCreate: include/ode/
 * objects.h:185-320, ode/src/ode.cpp:1880-1965.  Thresholds are stored
 * squared.  dWorldGetAutoDisableFlag returns the reference's flag bit (16)
 * when on. */
void dWorldSetAutoDisableFlag(dWorldID w, int do_auto_disable);
int dWorldGetAutoDisableFlag(dWorldID w);
void dWorldSetAutoDisableLinearThreshold(dWorldID w, dReal linear_average_threshold);
dReal dWorldGetAutoDisableLinearThreshold(dWorldID w);
void dWorldSetAutoDisableAngularThreshold(dWorldID w, dReal angular_average_threshold);
dReal dWorldGetAutoDisableAngularThreshold(dWorldID w);
void dWorldSetAutoDisableAverageSamplesCount(dWorldID w, unsigned int average_samples_count);
int dWorldGetAutoDisableAverageSamplesCount(dWorldID w);
void dWorldSetAutoDisableSteps(dWorldID w, int steps);
int dWorldGetAutoDisableSteps(dWorldID w);
void dWorldSetAutoDisableTime(dWorldID w, dReal time);
dReal dWorldGetAutoDisableTime(dWorldID w);

/* ---- bodies: include/ode/objects.h:700-1400 */
dBodyID dBodyCreate(dWorldID w);
void dBodyDestroy(dBodyID b);
void dBodySetData(dBodyID b, void *data);
void *dBodyGetData(dBodyID b);
void dBodySetPosition(dBodyID b, dReal x, dReal y, dReal z);
void dBodySetRotation(dBodyID b, const dMatrix3 R);
void dBodySetQuaternion(dBodyID b, const dQuaternion q);
void dBodySetLinearVel(dBodyID b, dReal x, dReal y, dReal z);
void dBodySetAngularVel(dBodyID b, dReal x, dReal y, dReal z);
const dReal *dBodyGetPosition(dBodyID b);
const dReal *dBodyGetRotation(dBodyID b);
const dReal *dBodyGetQuaternion(dBodyID b);
const dReal *dBodyGetLinearVel(dBodyID b);
const dReal *dBodyGetAngularVel(dBodyID b);
void dBodySetMass(dBodyID b, const dMass *mass);
void dBodyGetMass(dBodyID b, dMass *mass);
void dBodyAddForce(dBodyID b, dReal fx, dReal fy, dReal fz);
void dBodyAddTorque(dBodyID b, dReal fx, dReal fy, dReal fz);
const dReal *dBodyGetForce(dBodyID b);
const dReal *dBodyGetTorque(dBodyID b);
void dBodySetGyroscopicMode(dBodyID b, int enabled);
int dBodyGetGyroscopicMode(dBodyID b);
/* per-body damping and angular speed cap: ode/src/ode.cpp:1025-1113 */
void dBodySetLinearDamping(dBodyID b, dReal scale);
void dBodySetAngularDamping(dBodyID b, dReal scale);
void dBodySetDamping(dBodyID b, dReal linear_scale, dReal angular_scale);
void dBodySetLinearDampingThreshold(dBodyID b, dReal threshold);
void dBodySetAngularDampingThreshold(dBodyID b, dReal threshold);
void dBodySetDampingDefaults(dBodyID b);
dReal dBodyGetLinearDamping(dBodyID b);
dReal dBodyGetAngularDamping(dBodyID b);
dReal dBodyGetLinearDampingThreshold(dBodyID b);
dReal dBodyGetAngularDampingThreshold(dBodyID b);
void dBodySetMaxAngularSpeed(dBodyID b, dReal max_speed);
dReal dBodyGetMaxAngularSpeed(dBodyID b);
/* enable state and auto-disable per body: ode/src/ode.cpp:850-1020.  Each
 * step, before the solve (util.cpp:427-561), a body with auto-disable on, no
 * disabled flag and at least one joint (contacts of the step count) samples
 * its velocities; when the average of the last `average samples` samples is
 * within both thresholds for `steps` steps and `time` seconds the body is
 * disabled and its velocities zeroed.  A step processes every body connected
 * through contacts and joints to an enabled body and enables it again
 * (util.cpp:724-860); components of disabled bodies only are not stepped. */
void dBodyEnable(dBodyID b);
void dBodyDisable(dBodyID b);
int dBodyIsEnabled(dBodyID b);
void dBodySetAutoDisableFlag(dBodyID b, int do_auto_disable);
int dBodyGetAutoDisableFlag(dBodyID b);
void dBodySetAutoDisableLinearThreshold(dBodyID b, dReal linear_average_threshold);
dReal dBodyGetAutoDisableLinearThreshold(dBodyID b);
void dBodySetAutoDisableAngularThreshold(dBodyID b, dReal angular_average_threshold);
dReal dBodyGetAutoDisableAngularThreshold(dBodyID b);
void dBodySetAutoDisableAverageSamplesCount(dBodyID b, unsigned int average_samples_count);
int dBodyGetAutoDisableAverageSamplesCount(dBodyID b);
void dBodySetAutoDisableSteps(dBodyID b, int steps);
int dBodyGetAutoDisableSteps(dBodyID b);
void dBodySetAutoDisableTime(dBodyID b, dReal time);
dReal dBodyGetAutoDisableTime(dBodyID b);
void dBodySetAutoDisableDefaults(dBodyID b);
int dBodyGetNumJoints(dBodyID b);

/* ---- mass helpers: include/ode/mass.h:40-96 */
void dMassSetZero(dMass *m);
void dMassSetParameters(dMass *m, dReal themass, dReal cgx, dReal cgy, dReal cgz, dReal I11, dReal I22,
                        dReal I33, dReal I12, dReal I13, dReal I23);
void dMassSetSphere(dMass *m, dReal density, dReal radius);
void dMassSetSphereTotal(dMass *m, dReal total_mass, dReal radius);
void dMassSetCapsule(dMass *m, dReal density, int direction, dReal radius, dReal length);
void dMassSetBox(dMass *m, dReal density, dReal lx, dReal ly, dReal lz);
void dMassSetBoxTotal(dMass *m, dReal total_mass, dReal lx, dReal ly, dReal lz);

/* ---- spaces: include/ode/collision_space.h:60-120 */
dSpaceID dHashSpaceCreate(dSpaceID space);
void dHashSpaceSetLevels(dSpaceID space, int minlevel, int maxlevel);
void dHashSpaceGetLevels(dSpaceID space, int *minlevel, int *maxlevel);
void dSpaceDestroy(dSpaceID space);
void dSpaceSetCleanup(dSpaceID space, int mode);
int dSpaceGetNumGeoms(dSpaceID space);
/* include/ode/collision.h:822 */
void dSpaceCollide(dSpaceID space, void *data, dNearCallback *callback);

/* ---- geoms: include/ode/collision.h:100-1000 */
dGeomID dCreateSphere(dSpaceID space, dReal radius);
dGeomID dCreateBox(dSpaceID space, dReal lx, dReal ly, dReal lz);
dGeomID dCreateCapsule(dSpaceID space, dReal radius, dReal length);
dGeomID dCreatePlane(dSpaceID space, dReal a, dReal b, dReal c, dReal d);
void dGeomDestroy(dGeomID geom);
void dGeomSetData(dGeomID geom, void *data);
void *dGeomGetData(dGeomID geom);
void dGeomSetBody(dGeomID geom, dBodyID body);
dBodyID dGeomGetBody(dGeomID geom);
void dGeomSetPosition(dGeomID geom, dReal x, dReal y, dReal z);
void dGeomSetRotation(dGeomID geom, const dMatrix3 R);
const dReal *dGeomGetPosition(dGeomID geom);
const dReal *dGeomGetRotation(dGeomID geom);
int dGeomGetClass(dGeomID geom);
/* minx maxx miny maxy minz maxz; a plane is unbounded except below an
 * axis-aligned one (plane.cpp:80-107) */
void dGeomGetAABB(dGeomID geom, dReal aabb[6]);
/* include/ode/collision.h:792 */
int dCollide(dGeomID o1, dGeomID o2, int flags, dContactGeom *contact, int skip);
/* include/ode/collision.h:1478 */
int dBoxBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2, const dMatrix3 R2,
            const dVector3 side2, dVector3 normal, dReal *depth, int *return_code, int flags,
            dContactGeom *contact, int skip);

/* ---- joints: include/ode/objects.h:1500-1700 */
dJointGroupID dJointGroupCreate(int max_size);
void dJointGroupDestroy(dJointGroupID group);
void dJointGroupEmpty(dJointGroupID group);
dJointID dJointCreateContact(dWorldID w, dJointGroupID group, const dContact *c);
/* attaching a ball, hinge or hinge2 joint re-derives its body-frame anchor
 * and axes from their world values with the new bodies (the reference's
 * setRelativeValues, ode.cpp:1434-1438) */
void dJointAttach(dJointID j, dBodyID body1, dBodyID body2);
void dJointDestroy(dJointID j);
void dJointSetFeedback(dJointID j, dJointFeedback *fb);
dJointFeedback *dJointGetFeedback(dJointID j);
dBodyID dJointGetBody(dJointID j, int index);
int dAreConnectedExcluding(dBodyID body1, dBodyID body2, int joint_type);  /* objects.h:3499 */
int dAreConnected(dBodyID body1, dBodyID body2);                          /* objects.h:3484 */

/* ---- ball and hinge joints: include/ode/common.h:384-403 (types),
 * :439-455 (parameters), objects.h:1693-2618 */
enum {
    dJointTypeNone = 0, dJointTypeBall, dJointTypeHinge, dJointTypeSlider, dJointTypeContact, dJointTypeUniversal,
    dJointTypeHinge2
};
enum {
    dParamLoStop = 0, dParamHiStop, dParamVel, dParamLoVel, dParamHiVel, dParamFMax, dParamFudgeFactor,
    dParamBounce, dParamCFM, dParamStopERP, dParamStopCFM, dParamSuspensionERP, dParamSuspensionCFM, dParamERP,
    dParamGroup2 = 0x100, dParamLoStop2 = 0x100, dParamHiStop2, dParamVel2, dParamLoVel2, dParamHiVel2, dParamFMax2,
    dParamFudgeFactor2, dParamBounce2, dParamCFM2, dParamStopERP2, dParamStopCFM2
};
dJointID dJointCreateBall(dWorldID w, dJointGroupID group);    /* objects.h:1693 */
dJointID dJointCreateHinge(dWorldID w, dJointGroupID group);   /* objects.h:1701 */
int dJointGetType(dJointID j);                                  /* objects.h:1929 */
void dJointSetBallAnchor(dJointID j, dReal x, dReal y, dReal z);        /* objects.h:1965 */
void dJointSetBallParam(dJointID j, int parameter, dReal value);         /* objects.h:1977 */
void dJointSetHingeAnchor(dJointID j, dReal x, dReal y, dReal z);       /* objects.h:1983 */
void dJointSetHingeAxis(dJointID j, dReal x, dReal y, dReal z);         /* objects.h:1991 */
/* the axis, with the current relative rotation taken as the given angle */
void dJointSetHingeAxisOffset(dJointID j, dReal x, dReal y, dReal z, dReal angle); /* objects.h:2021 */
void dJointSetHingeParam(dJointID j, int parameter, dReal value);        /* objects.h:2027 */
void dJointGetBallAnchor(dJointID j, dVector3 result);                   /* objects.h:2555 */
dReal dJointGetBallParam(dJointID j, int parameter);                      /* objects.h:2573 */
void dJointGetHingeAnchor(dJointID j, dVector3 result);                  /* objects.h:2582 */
void dJointGetHingeAxis(dJointID j, dVector3 result);                    /* objects.h:2598 */
dReal dJointGetHingeParam(dJointID j, int parameter);                     /* objects.h:2604 */
dReal dJointGetHingeAngle(dJointID j);                                    /* objects.h:2618 */
dJointID dJointCreateHinge2(dWorldID w, dJointGroupID group);                  /* objects.h:1725 */
void dJointSetHinge2Anchor(dJointID j, dReal x, dReal y, dReal z);            /* objects.h:2070 */
void dJointSetHinge2Axes(dJointID j, const dReal *axis1, const dReal *axis2); /* objects.h:2084 */
void dJointSetHinge2Axis1(dJointID j, dReal x, dReal y, dReal z);             /* objects.h:2094 */
void dJointSetHinge2Axis2(dJointID j, dReal x, dReal y, dReal z);             /* objects.h:2104 */
void dJointSetHinge2Param(dJointID j, int parameter, dReal value);             /* objects.h:2110 */
void dJointGetHinge2Anchor(dJointID j, dVector3 result);                       /* objects.h:2663 */
void dJointGetHinge2Axis1(dJointID j, dVector3 result);                        /* objects.h:2679 */
void dJointGetHinge2Axis2(dJointID j, dVector3 result);                        /* objects.h:2685 */
dReal dJointGetHinge2Param(dJointID j, int parameter);                          /* objects.h:2691 */
dReal dJointGetHinge2Angle1(dJointID j);                                        /* objects.h:2697 */

/* ---- misc: include/ode/misc.h:35-50, rotation.h:40-70 */
unsigned long dRand(void);
int dRandInt(int n);
void dRandSetSeed(unsigned long s);
unsigned long dRandGetSeed(void);
int dTestRand(void);
void dRSetIdentity(dMatrix3 R);
void dRFromAxisAndAngle(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal angle);
void dRfromQ(dMatrix3 R, const dQuaternion q);
void dQFromAxisAndAngle(dQuaternion q, dReal ax, dReal ay, dReal az, dReal angle);
/* odemath.h:521-523: scale to unit length by the largest component; a zero
 * vector is left as it is (dSafeNormalize3 returns 0 for it) */
int dSafeNormalize3(dVector3 a);
void dNormalize3(dVector3 a);

/* ======================================================================
 * gbode extensions (no ODE counterpart)
 * ====================================================================== */

/* Solver schedule used by dWorldQuickStep. */
enum {
    /* Graph-coloured projected Gauss-Seidel over all rows of the world: rows of
     * one colour share no body and are relaxed in parallel; colours run in
     * sequence.  The default. */
    GBODE_SOLVER_COLOURED = 0,
    /* The reference's own row order: islands built as ODE builds them, rows in
     * joint order with findex<0 rows first, one island per thread block, rows
     * relaxed one after another (ODE with row reordering disabled). */
    GBODE_SOLVER_REFERENCE_ORDER = 1,
};
void gbodeWorldSetSolver(dWorldID w, int solver);
int gbodeWorldGetSolver(dWorldID w);

/* Iterate until the LCP residual (projected natural map, FP32, relative to
 * max(1, max|lambda|)) is <= target, checking at least check_every
 * iterations apart (see gbodeWorldSetResidualChecks), up to max_iterations.
 * target <= 0 restores the fixed iteration count. */
void gbodeWorldSetResidualTarget(dWorldID w, dReal target, int check_every, int max_iterations);

/* When residual-target mode checks.  GBODE_CHECKS_PREDICTED (the default):
 * from the last two checks' residuals the sweeps still needed are predicted
 * (geometric decay) and the next check comes after half of them -- at least
 * check_every, at most 64 sweeps later; check_every sweeps after a check
 * whose residual did not fall.  GBODE_CHECKS_FIXED: every check_every sweeps.
 * Either way the body accumulators are re-formed from the multipliers every
 * reform_every sweeps (<= 0: 500) and before the check that ends the solve,
 * so that check's residual is the multipliers' own. */
#define GBODE_CHECKS_PREDICTED 0
#define GBODE_CHECKS_FIXED 1
void gbodeWorldSetResidualChecks(dWorldID w, int mode, int reform_every);

/* Warm start: 0 = cold (lambda = 0, the reference default), 1 = previous-step
 * lambda of the same (geom pair, contact slot) scaled by `scale`. */
void gbodeWorldSetWarmStart(dWorldID w, int mode, dReal scale);

/* Thread blocks of the coloured solver's persistent kernel (256 threads
 * each; 0 or more than the SM count: one per SM).  Fewer blocks make each
 * colour's grid barrier cheaper; a colour with more manifolds than the
 * blocks' threads relaxes the rest from global memory. */
void gbodeWorldSetSolverBlocks(dWorldID w, int blocks);
int gbodeWorldGetSolverBlocks(dWorldID w);

/* Passes over a constraint group's rows (a contact manifold's normal rows,
 * then its friction rows; a joint's rows in order) each time the coloured
 * solver visits it in a sweep (1 to 16; default 1).  Repeating the strongly
 * coupled rows of one manifold while they are in registers is a Gauss-Seidel
 * order with repetition; it can lower the sweeps a residual target needs. */
void gbodeWorldSetManifoldPasses(dWorldID w, int passes);
int gbodeWorldGetManifoldPasses(dWorldID w);

/* Tiles of the coloured solver: threads a block of the sweep kernels (128
 * or 256, default 256) -- the colour-group tile: a colour's slots of a block
 * are relaxed in waves of this many -- and staged rows a shared-memory buffer
 * of the one-level sweep (64 to 800, default 800; a wave also ends when its
 * rows would not fit).  Other values select the defaults. */
void gbodeWorldSetSolverTiles(dWorldID w, int threads, int chunk_rows);
void gbodeWorldGetSolverTiles(dWorldID w, int *threads, int *chunk_rows);

/* Two-level sweep of the coloured solver (0 off; k >= 1 on, up to 8).  The
 * bodies are split into one spatial column per solver block; contact
 * manifolds inside one column are relaxed from the block's shared memory,
 * colour by colour with block barriers only, and only the manifolds that
 * cross columns are coloured globally with a grid barrier per colour.  A
 * sweep relaxes the interior manifolds k times (interior passes cost no grid
 * barrier), then the crossing ones once.  Same LCP, another Gauss-Seidel
 * order (deterministic).  Columns whose manifolds do not fit in shared memory
 * fall back to the global colours. */
void gbodeWorldSetTwoLevelSweep(dWorldID w, int interior_phases);
int gbodeWorldGetTwoLevelSweep(dWorldID w);

/* How the two-level sweep orders the blocks' steps (the interior phase, then
 * each crossing colour).  GBODE_SYNC_NEIGHBOURS (the default): a crossing
 * manifold is relaxed by the block whose column holds its first body, and a
 * block waits only for the blocks that touch one of the same bodies to finish
 * the previous step (nothing, in a colour where it has no manifold).
 * GBODE_SYNC_GRID: a grid barrier after every step.  Both give the same
 * multipliers and bodies to the bit. */
#define GBODE_SYNC_NEIGHBOURS 0
#define GBODE_SYNC_GRID 1
void gbodeWorldSetSweepSync(dWorldID w, int mode);
int gbodeWorldGetSweepSync(dWorldID w);

/* Cross classes of the two-level sweep (0 or 1: off).  With k >= 2 the
 * crossing manifolds' colours are merged into k classes (colour c into class
 * c mod k), each relaxed as one step instead of one step per colour.  Inside a
 * class a body can be shared by several manifolds; they are relaxed at once
 * (Jacobi within the class) with mass splitting: a body shared by n manifolds
 * of the class enters each of them with 1/n of its mass, and each adds 1/n of
 * its copy's change of the body's velocities (as fixed-point integers, so the
 * sum does not depend on the order).  The fixed point is the same LCP
 * solution; fewer steps a sweep, usually a few more sweeps.  The result does
 * not depend on timing (the same to the bit run after run, and under either
 * gbodeWorldSetSweepSync mode).  A crossing group that is not a staged
 * manifold or joint, or that touches a body outside the columns' lists, keeps
 * the exact colours for that step (gbodeStepStats.cross_classes reads 0). */
#define GBODE_MAX_CROSS_CLASSES 8
void gbodeWorldSetCrossClasses(dWorldID w, int classes);
int gbodeWorldGetCrossClasses(dWorldID w);

/* Momentum between the sweeps of the coloured solver (no counterpart in the
 * reference; 0: off, the default; clamped to [0, 0.95]).  After each sweep
 * every multiplier moves on from the sweep's projected Gauss-Seidel result
 * y_k to y_k + beta (y_k - y_{k-1}), and every body's velocity accumulators
 * by the same rule, before the next sweep starts from them (the fixed-
 * coefficient extrapolation of Nesterov's accelerated gradient method, applied
 * to the sweep's iterates).  A solution of the LCP is a fixed point of both,
 * so the solution is the same; on deep piles beta = 0.5 reaches a residual
 * target in fewer sweeps.  The first and the last sweep, and every sweep that
 * ends in a residual check, are plain, so every check and the final
 * multipliers are Gauss-Seidel results; a check whose residual rose halves
 * beta for the rest of the step (gbodeStepStats.momentum reads the value at
 * the end).  On the two-level sweep a step whose crossing manifolds touch a
 * body outside the columns' lists runs without it (momentum reads 0).  The
 * result does not depend on timing. */
void gbodeWorldSetSweepMomentum(dWorldID w, dReal beta);
dReal gbodeWorldGetSweepMomentum(dWorldID w);

/* The fused GPU path: hash-space broad phase, narrow phase and contact-joint
 * creation without leaving the device.  Equivalent to dSpaceCollide with a near
 * callback that calls dCollide(o1, o2, maxc, ...) and makes one contact joint
 * per point with surface *s (fdir1 unused), attached to the geoms' bodies.
 * The contacts belong to `group` and are cleared by dJointGroupEmpty.  Runs
 * asynchronously on the world's stream.  Returns 1, or 0 on a bad argument. */
int gbodeSpaceCollideContacts(dSpaceID space, dWorldID w, dJointGroupID group, const dSurfaceParameters *s,
                              int maxc);

/* Bulk builders for large batched scenes (no counterpart in the reference):
 * the same creation calls an ODE program makes per object, looped inside the
 * library.  Returns 1, or 0 on a bad argument.
 *   gbodeCreateBodies: rows [n][20] = pos(3) q(4, w first) lvel(3) avel(3)
 *     mass I11 I22 I33 I12 I13 I23 (dMassSetParameters with the COM at 0)
 *   gbodeCreateGeoms: cls [n] (dSphereClass, dBoxClass, dCapsuleClass,
 *     dPlaneClass), dims [n][4], body [n] (NULL entry or array: static geom,
 *     placed by pos [n][3] and R [n][12])
 *   gbodeCreateJoints: rows [n][GBODE_JOINT_COLS] = type (dJointTypeBall,
 *     Hinge, Hinge2), body1, body2 (indices into `bodies`, -1: none),
 *     anchor(3), axis or axis 1 (3), lo stop, hi stop, axis 2 (3), axis-2
 *     motor velocity, max force, suspension ERP, CFM, axis-1 motor velocity,
 *     max force -- world frame */
#define GBODE_JOINT_COLS 20
int gbodeCreateBodies(dWorldID w, int n, const float *rows, dBodyID *out);
int gbodeCreateGeoms(dSpaceID space, int n, const int *cls, const float *dims, const float *pos, const float *R,
                     const dBodyID *body, dGeomID *out);
int gbodeCreateJoints(dWorldID w, int n, const float *rows, const dBodyID *bodies, dJointID *out);

/* One fused step (no counterpart in the reference): gbodeSpaceCollideContacts
 * + dWorldQuickStep(w, dt) + dJointGroupEmpty(group).  With use_graph != 0
 * the step is recorded once into a CUDA graph -- on the second call after
 * anything that changes the recorded work (body, geom or joint edits on the
 * host, parameters, sizes) -- and later calls replay it with a single
 * cudaGraphLaunch on the world's stream.  The world needs its own stream (the
 * default) and step timing off.  Returns 1, or 0 on error. */
int gbodeWorldStepFused(dWorldID w, dSpaceID space, dJointGroupID group, const dSurfaceParameters *s, int maxc,
                        dReal dt, int use_graph);

/* Pair rule of a hash space.  0 (default): exactly the pairs the reference's
 * dHashSpace reports, including its blind spot -- the bucket of a cell is
 * computed in unsigned arithmetic that wraps for negative z in columns near
 * the origin (collision_space.cpp:358-361), so some overlapping pairs there
 * are never reported.  1: every pair whose AABBs overlap. */
void gbodeHashSpaceSetExactPairs(dSpaceID space, int exact);

/* CUDA stream (cudaStream_t) the world enqueues its work on; NULL = the
 * library's own stream. */
void gbodeWorldSetStream(dWorldID w, void *stream);
void *gbodeWorldGetStream(dWorldID w);
/* Wait for the world's stream. Returns 1, or 0 if a device error was recorded. */
int gbodeWorldSynchronize(dWorldID w);

/* Statistics of the last dWorldQuickStep (synchronises the stream). */
typedef struct gbodeStepStats {
    int contacts;          /* contact joints stepped */
    int rows;              /* constraint rows */
    int colours;           /* colours (coloured solver) */
    int iterations;        /* PGS sweeps performed */
    float residual;        /* final FP32 relative residual (0 if not computed) */
    int pairs;             /* candidate pairs of the last broad phase */
    float solve_ms;        /* device time of the PGS sweeps, if timing is on */
    float step_ms;         /* device time of the whole dWorldQuickStep, if timing is on */
    int sleeping;          /* bodies not stepped: their component is disabled (auto-disable) */
    int interior_colours;  /* two-level sweep: colours of the columns' interior manifolds (0: off) */
    int interior_rows;     /* two-level sweep: rows relaxed from shared memory (0: off) */
    int neighbour_waits;   /* two-level sweep: the blocks waited only on their neighbours (1), or on grid
                              barriers (0: GBODE_SYNC_GRID, or a body touched by too many blocks) */
    int cross_classes;     /* two-level sweep: split classes of the crossing manifolds (0: exact colours) */
    float momentum;        /* momentum between sweeps at the end of the solve (0: off or not used) */
} gbodeStepStats;
void gbodeWorldGetStepStats(dWorldID w, gbodeStepStats *out);
/* Record CUDA events around the solver and the step (adds no host syncs). */
void gbodeWorldSetTiming(dWorldID w, int enabled);

/* A device-side copy of the world's simulation state -- bodies, the
 * warm-start cache, the joints' multipliers, the auto-disable state -- to
 * rerun the same steps (benchmarks, tuning, rollback).  Save replaces the
 * world's one snapshot; Restore puts it back (0 with gbodeGetLastError when
 * bodies were added or removed, a device buffer grew, or the host changed a
 * body, since the save); Drop frees it (dWorldDestroy does too).  Contacts,
 * rows and space state are rebuilt by every step and are not part of it. */
int gbodeWorldSaveSnapshot(dWorldID w);
int gbodeWorldRestoreSnapshot(dWorldID w);
void gbodeWorldDropSnapshot(dWorldID w);

/* Solver settings tuned on the running world.  gbodeWorldAutotune makes one
 * plain fused step, copies the device-side state aside, and for each
 * candidate -- threads a solver block (128 or 256: the colour-group tile, the
 * slots one wave of a colour relaxes at once), staged rows a shared-memory
 * buffer (400 or 800), the two-level sweep (off, or two interior passes),
 * residual checks every 5 or 10 sweeps when a residual target is set, and
 * also half the solver blocks or two passes over a group's rows; each with
 * and without the sweep momentum when a residual target and a momentum are
 * set -- restores that state and times
 * `steps` gbodeWorldStepFused steps (after two untimed ones) with CUDA
 * events.  It keeps the candidate with the lowest median step time, leaves
 * it set, and restores the state once more: the world continues from the
 * one plain step.  Returns 1 and the choice in *best, or 0
 * (gbodeGetLastError). */
typedef struct gbodeTuning {
    int blocks;       /* gbodeWorldSetSolverBlocks */
    int passes;       /* gbodeWorldSetManifoldPasses */
    int check_every;  /* residual checks every this many sweeps (0: no residual target) */
    float ms_per_step;
    int candidates;   /* candidates timed */
    int threads;      /* gbodeWorldSetSolverTiles: threads a block */
    int chunk_rows;   /* gbodeWorldSetSolverTiles: staged rows a buffer */
    int two_level;    /* gbodeWorldSetTwoLevelSweep */
    float momentum;   /* gbodeWorldSetSweepMomentum: the value set, or 0 if the sweeps were faster without */
} gbodeTuning;
int gbodeWorldAutotune(dWorldID w, dSpaceID space, dJointGroupID group, const dSurfaceParameters *s, int maxc,
                       dReal dt, int steps, int use_graph, gbodeTuning *best);

/* FP64 LCP residual and complementarity error of the last step's solution,
 * evaluated on the device from the step's FP32 rows (unscaled) and lambda:
 * max_i |lambda_i - proj_[lo,hi](lambda_i - (A lambda - b)_i / A_ii)|, not
 * normalised; *complementarity receives the min-map complementarity error
 * max_i max(min(lambda_i - lo_i, w_i+ / A_ii), min(hi_i - lambda_i, w_i- / A_ii))
 * with w_i = (A lambda - b)_i, w+ = max(w, 0), w- = max(-w, 0) -- in the units
 * of lambda, like the residual; *max_lambda receives max|lambda|.  Divide the first two by
 * max(1, max|lambda_ref|) for relative figures.  Synchronises the stream. */
double gbodeWorldLastResidual(dWorldID w, double *complementarity, double *max_lambda);

/* Copies of the last step's rows and lambda for checking: rows [nrows][20]
 * (J1(6) J2(6) rhs cfm lo hi b1 b2 findex lambda, world body indices), in the
 * solver's row order.  Returns nrows (writes at most cap rows). */
int gbodeWorldGetLastRows(dWorldID w, float *rows, int cap);

/* Copies of the contacts the last gbodeSpaceCollideContacts (or the host
 * contact joints of the last step) produced: [n][12] pos(3) normal(3) depth
 * g1 g2 b1 b2 slot (geom indices are positions in the space's geom list,
 * body indices creation order among live bodies).  Returns n (writes at most
 * cap).  Synchronises the stream. */
int gbodeWorldGetContacts(dWorldID w, float *out, int cap);

/* The FP32 relative residual at each residual check of the last solve
 * (residual-target mode), oldest first.  Returns the number of checks (at
 * most 256 are kept).  Synchronises the stream. */
int gbodeWorldGetResidualHistory(dWorldID w, float *out, int cap);
/* The sweeps done at each of those checks (0 for the checks of the start),
 * oldest first; returns the number of checks.  Synchronises the stream. */
int gbodeWorldGetResidualSweeps(dWorldID w, int *out, int cap);

/* Last error message ("" if none) and clear. */
const char *gbodeGetLastError(void);
/* Number of kernel launches the library has issued since load. */
long long gbodeKernelLaunchCount(void);

/* Fault injection for error-path tests (no counterpart in the reference).
 * Process-wide, host-side; nothing is made to fault:
 *   GBODE_TEST_BARRIER   value != 0: the next solver launch's grid-barrier
 *                        counter starts one arrival short, so its bounded
 *                        wait runs out (a second or two): the kernel returns
 *                        and gbodeWorldSynchronize reports ERR bit 0x1
 *   GBODE_TEST_STAGE     value != 0: the next solver launch's first staging
 *                        wait names a copy that is never issued (bounded):
 *                        ERR bit 0x100 (and 0x1 from blocks left waiting)
 *   GBODE_TEST_ALLOC     after `value` more device allocations succeed, the
 *                        next `count` fail as cudaMalloc would
 *   GBODE_TEST_CONTACT_CAP, GBODE_TEST_ROW_CAP, GBODE_TEST_COLOUR_CAP
 *                        capacities the kernels see, below what is allocated
 *                        (0: off): contacts of the narrow phase, contact rows
 *                        of the assembly (worlds without ball/hinge joints),
 *                        colours of the colouring; the kernels clamp and set
 *                        ERR bits 0x4 / 0x8 / 0x10
 *   GBODE_TEST_ALLOC_PENDING  returns 1 while an injected allocation
 *                        failure has not happened yet, else 0
 *   GBODE_TEST_OFF       clears everything
 * Returns 1, or 0 for an unknown kind. */
#define GBODE_TEST_OFF 0
#define GBODE_TEST_BARRIER 1
#define GBODE_TEST_STAGE 2
#define GBODE_TEST_ALLOC 3
#define GBODE_TEST_CONTACT_CAP 4
#define GBODE_TEST_ROW_CAP 5
#define GBODE_TEST_COLOUR_CAP 6
#define GBODE_TEST_ALLOC_PENDING 7
int gbodeTestInject(int kind, int value, int count);

/* Bulk state access for batched drivers: [nb][25] pos q R lvel avel in body
 * creation order (index = order of dBodyCreate among live bodies). */
int gbodeWorldGetBodyCount(dWorldID w);
void gbodeWorldGetState(dWorldID w, float *out);
void gbodeWorldSetState(dWorldID w, const float *in);

/* ---- Learned warm start (extension; the reference has no counterpart).
 *
 * A small MLP predicts each contact's three starting multipliers (normal and
 * two friction rows, dContactApprox1) from twelve local features:
 *   normal (3), contact-point relative velocity in the contact frame
 *   (normal, t1, t2), depth, effective mass of the normal row, the
 *   previous step's three multipliers in units of s, and 1 if a previous
 *   step's contact was matched
 * where s = effective mass * |gravity| is the contact's weight scale.  The
 * network is 12 -> 128 -> 128 -> 128 -> 3 with SiLU; its outputs are
 * multipliers in units of s.  Parameters: GBODE_MLP_NPARAMS floats, in the
 * order mean[12] std[12] (input standardisation), W1[128][12] b1[128]
 * W2[128][128] b2[128] W3[128][128] b3[128] W4[3][128] b4[3].
 *
 * With the learned start enabled, dWorldQuickStep predicts the start on the
 * tensor cores (BF16 operands, FP32 accumulation), projects it onto the
 * rows' bounds, and compares its LCP residual with the plain start's (the
 * previous-step multipliers when gbodeWorldSetWarmStart is on, else zero):
 * the lower residual starts the sweeps, so the network can only help. */
#define GBODE_MLP_NPARAMS 35099
int gbodeMlpParamCount(void);
/* Loss (mean squared error over the three outputs) and its gradient for n
 * samples X[n][12] (raw features), Y[n][3] (targets in units of s), on the
 * device.  Host arrays.  Returns 1, or 0 on error. */
int gbodeMlpLossGrad(const float *params, const float *X, const float *Y, int n, float *grad, float *loss);
/* Adam training on the device (mini-batches of `batch` shuffled samples);
 * params is read as the starting point (its standardisation entries are kept
 * fixed) and overwritten with the result; loss_per_epoch (may be NULL) gets
 * each epoch's mean batch loss.  Host arrays.  Returns 1, or 0 on error. */
int gbodeMlpTrain(const float *X, const float *Y, int n, int epochs, int batch, float lr, unsigned seed,
                  float *params, float *loss_per_epoch);
/* Inference with the tensor-core kernel: Y[n][3] = MLP(X[n][12]).  Host
 * arrays.  Returns 1, or 0 on error. */
int gbodeMlpPredict(const float *params, const float *X, int n, float *Y);
/* Enable (params != NULL, enabled != 0) or disable the learned start. */
int gbodeWorldSetLearnedWarmStart(dWorldID w, const float *params, int enabled);
/* Record the features of every contact of each step (for training data). */
void gbodeWorldSetLearnCapture(dWorldID w, int enabled);
/* Samples of the last step (with capture or the learned start on):
 * [n][17] = 12 features, s, the three rows' multipliers after the solve,
 * 1 if the contact has the three-row (normal + 2 friction) shape.  Returns n
 * (writes at most cap).  Synchronises the stream. */
int gbodeWorldGetLearnSamples(dWorldID w, float *out, int cap);
/* Last step with the learned start: out[0] = 1 if the network's start was
 * used, out[1] its relative residual, out[2] the plain start's. */
void gbodeWorldGetLearnedStats(dWorldID w, float *out3);

/* ---- Narrow phase that allocates nothing (no counterpart in the reference).
 *
 * For callers that must not allocate device memory once they run: programs
 * that reserve all their GPU memory up front and hand out pieces of it
 * themselves (engines, robot controllers, simulators embedded in a larger
 * GPU application), where a cudaMalloc or cudaFree in the middle of a frame
 * would synchronise the device, could fail under their memory budget, or is
 * simply forbidden by the host program's allocator.
 *
 * gbodeCollidePairsNoAlloc runs dCollide on every pair of a batch on the
 * device: for pair p, geoms[pairs[2p]] against geoms[pairs[2p+1]], with the
 * same colliders, rejections (a geom with itself, two geoms on one body) and
 * normal orientation as dCollide, and at most flags & 0xffff contacts per
 * pair (capped at 8).  Only those low 16 bits of flags are used; higher flag
 * bits are ignored.  All pointers are DEVICE pointers the caller owns:
 *   geoms     [ngeoms] gbodePairGeom records
 *   pairs     [npairs][2] geom indices, 8-byte aligned (a pair is read as
 *             one 8-byte load; a misaligned pointer is rejected)
 *   contacts  [capacity][8] out: pos xyz, depth, normal xyz, 0 -- pair p's
 *             contacts are rows first[p] .. first[p+1]-1 (rows at or beyond
 *             capacity are not written)
 *   first     [npairs+1] out: exclusive prefix sum of the per-pair counts;
 *             first[npairs] is the total (compare it with capacity)
 * The work is enqueued on `stream` (a cudaStream_t, NULL = the legacy default
 * stream); read the outputs after that stream has reached this point.
 *
 * Limit: npairs <= GBODE_NOALLOC_MAX_PAIRS.  A larger batch is rejected:
 * nothing is launched, the call returns 0 and gbodeGetLastError() says why;
 * split it into several calls.  The temporaries (8 contact slots and a count
 * per pair) live in one fixed array of 2.03 MiB in device memory that every
 * GPU which loads this library holds until the process exits.  Each call
 * writes every part of that array it later reads, so no state carries over
 * between calls; but all calls share the one array, so two calls whose work
 * can overlap on the GPU (different streams, or different host threads, with
 * no ordering between them) race and corrupt each other's results.  Order
 * them on one stream or wait in between.
 *
 * The first call on each device (with that device current) looks up the
 * array's device address with cudaGetSymbolAddress, which can load the
 * library's device code on that device; make that first call before any
 * stream capture begins.
 *
 * An error already pending on the calling thread from earlier, unrelated CUDA
 * work is cleared before the launches, so that a launch error reported here
 * is this call's own.
 *
 * Returns 1 when the work was enqueued, 0 on a rejected argument or launch
 * error (gbodeGetLastError() has the message). */
#define GBODE_NOALLOC_MAX_PAIRS 8192
typedef struct gbodePairGeom {
    int cls;          /* dSphereClass, dBoxClass, dCapsuleClass or dPlaneClass */
    int body;         /* any id of the geom's body, -1 for none */
    int pad[2];
    dReal dims[4];    /* sphere: radius; box: side lengths; capsule: radius,
                         length; plane: unit normal and offset (a, b, c, d) */
    dReal pos[4];     /* position (xyz) */
    dReal R[12];      /* rotation, dMatrix3 layout (3 rows of 4) */
} gbodePairGeom;      /* 96 bytes */
int gbodeCollidePairsNoAlloc(const gbodePairGeom *geoms, int ngeoms, const int *pairs, int npairs, int flags,
                             float *contacts, int capacity, int *first, void *stream);

#ifdef __cplusplus
}
#endif
#endif
