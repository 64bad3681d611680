// Golden-vector generator: runs the reference ODE library (built from its own
// sources by oracle/ref_build/Makefile into oracle/_ref/<variant>/libode.a) on
// inputs written by tests/golden/make_golden.py and writes the reference's
// outputs back as raw little-endian arrays.  Test infrastructure only.
//
// Modes (argv[1]):
//   colliders IN OUT   dCollide on single geom pairs (collision_kernel.cpp:292)
//                      plus dBoxBox's return_code for box-box (box.cpp:356)
//   space IN OUT       dSpaceCollide on a dHashSpace (collision_space.cpp:421):
//                      the set of candidate pairs handed to the near callback
//   step IN OUT        one dWorldQuickStep (ode.cpp:1847) or dWorldStep
//                      (ode.cpp:1828) on bodies + a given contact list; lambda
//                      recovered from dJointFeedback
//   loop IN OUT        the full user loop (dSpaceCollide -> near callback ->
//                      dCollide -> dJointCreateContact -> dWorldQuickStep ->
//                      dJointGroupEmpty) with per-step states and snapshots
//   timing IN OUT      the full user loop on a large scene with the reference's
//                      opt-in multi-threaded stepping (built-in thread pool,
//                      dWorldSetStepThreadingImplementation): wall-clock seconds
//                      of dSpaceCollide + contact joints and of dWorldQuickStep
//                      per step (a timing of the reference itself, not a golden)
//   chain IN OUT       bodies linked by ball and hinge joints (hinge limits),
//                      no geoms, stepped with dWorldQuickStep: per-step body
//                      poses and hinge angles (dJointGetHingeAngle)
#include <ode/ode.h>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>

static FILE *fin, *fout;
template <class T> static void rd(T *p, size_t n) {
    if (fread(p, sizeof(T), n, fin) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
template <class T> static void wr(const T *p, size_t n) { fwrite(p, sizeof(T), n, fout); }
static int rdi() { int v; rd(&v, 1); return v; }

enum { CLS_SPHERE = 0, CLS_BOX = 1, CLS_CAPSULE = 2, CLS_PLANE = 4 };

static dGeomID make_geom(dSpaceID space, int cls, const float *pos, const float *R, const float *dims) {
    dGeomID g = 0;
    switch (cls) {
    case CLS_SPHERE: g = dCreateSphere(space, dims[0]); break;
    case CLS_BOX: g = dCreateBox(space, dims[0], dims[1], dims[2]); break;
    case CLS_CAPSULE: g = dCreateCapsule(space, dims[0], dims[1]); break;
    case CLS_PLANE: return dCreatePlane(space, dims[0], dims[1], dims[2], dims[3]);
    default: fprintf(stderr, "bad class %d\n", cls); exit(2);
    }
    dGeomSetPosition(g, pos[0], pos[1], pos[2]);
    dMatrix3 m;
    for (int i = 0; i < 12; i++) m[i] = R[i];
    dGeomSetRotation(g, m);
    return g;
}

// ---------------------------------------------------------------- colliders
static void mode_colliders() {
    int n = rdi();
    std::vector<int> cls(2 * n), flags(n);
    std::vector<float> pos(6 * n), R(24 * n), dims(8 * n);
    rd(cls.data(), cls.size()); rd(flags.data(), n);
    rd(pos.data(), pos.size()); rd(R.data(), R.size()); rd(dims.data(), dims.size());
    std::vector<int> count(n), code(n, -1), swap(8 * n, 0), side(16 * n, 0);
    std::vector<float> cpos(24 * n, 0), cnrm(24 * n, 0), cdep(8 * n, 0);
    for (int k = 0; k < n; k++) {
        dGeomID a = make_geom(0, cls[2 * k], &pos[6 * k], &R[24 * k], &dims[8 * k]);
        dGeomID b = make_geom(0, cls[2 * k + 1], &pos[6 * k + 3], &R[24 * k + 12], &dims[8 * k + 4]);
        dContactGeom c[8];
        memset(c, 0, sizeof c);
        int num = dCollide(a, b, flags[k], c, sizeof(dContactGeom));
        count[k] = num;
        for (int i = 0; i < num; i++) {
            for (int j = 0; j < 3; j++) { cpos[24 * k + 3 * i + j] = c[i].pos[j]; cnrm[24 * k + 3 * i + j] = c[i].normal[j]; }
            cdep[8 * k + i] = c[i].depth;
            swap[8 * k + i] = (c[i].g1 == b) ? 1 : 0;
            side[16 * k + 2 * i] = c[i].side1; side[16 * k + 2 * i + 1] = c[i].side2;
        }
        if (cls[2 * k] == CLS_BOX && cls[2 * k + 1] == CLS_BOX) {
            dVector3 p1, p2, s1, s2, nrm; dMatrix3 R1, R2; dReal depth; int rc = 0;
            for (int j = 0; j < 3; j++) { p1[j] = pos[6 * k + j]; p2[j] = pos[6 * k + 3 + j]; s1[j] = dims[8 * k + j]; s2[j] = dims[8 * k + 4 + j]; }
            p1[3] = p2[3] = s1[3] = s2[3] = 0;
            for (int j = 0; j < 12; j++) { R1[j] = R[24 * k + j]; R2[j] = R[24 * k + 12 + j]; }
            dContactGeom cc[8];
            int m2 = dBoxBox(p1, R1, s1, p2, R2, s2, nrm, &depth, &rc, flags[k], cc, sizeof(dContactGeom));
            code[k] = m2 ? rc : 0;
        }
        dGeomDestroy(a); dGeomDestroy(b);
    }
    wr(count.data(), n); wr(code.data(), n); wr(cpos.data(), cpos.size()); wr(cnrm.data(), cnrm.size());
    wr(cdep.data(), cdep.size()); wr(swap.data(), swap.size()); wr(side.data(), side.size());
}

// ---------------------------------------------------------------- space
struct PairSink { std::vector<dGeomID> *geoms; std::vector<int> pairs; };
static int geom_index(std::vector<dGeomID> &v, dGeomID g) {
    return (int)(std::find(v.begin(), v.end(), g) - v.begin());
}
static void space_cb(void *data, dGeomID a, dGeomID b) {
    PairSink *s = (PairSink *)data;
    int i = (int)(size_t)dGeomGetData(a), j = (int)(size_t)dGeomGetData(b);
    s->pairs.push_back(std::min(i, j)); s->pairs.push_back(std::max(i, j));
}
static void mode_space() {
    int n = rdi();
    int minlevel = rdi(), maxlevel = rdi();
    std::vector<int> cls(n);
    std::vector<float> pos(3 * n), R(12 * n), dims(4 * n);
    rd(cls.data(), n); rd(pos.data(), pos.size()); rd(R.data(), R.size()); rd(dims.data(), dims.size());
    dSpaceID sp = dHashSpaceCreate(0);
    dHashSpaceSetLevels(sp, minlevel, maxlevel);
    std::vector<dGeomID> geoms(n);
    for (int i = 0; i < n; i++) {
        geoms[i] = make_geom(sp, cls[i], &pos[3 * i], &R[12 * i], &dims[4 * i]);
        dGeomSetData(geoms[i], (void *)(size_t)i);
    }
    PairSink sink; sink.geoms = &geoms;
    dSpaceCollide(sp, &sink, &space_cb);
    int np = (int)sink.pairs.size() / 2;
    wr(&np, 1); wr(sink.pairs.data(), sink.pairs.size());
    dSpaceDestroy(sp);
}

// ---------------------------------------------------------------- world helpers
struct WorldParams { float dt, g[3], erp, cfm, w, max_vel, min_depth; };
static const int BODY_IN = 20;   // pos3 q4 lvel3 avel3 mass1 I6
static const int BODY_OUT = 25;  // pos3 q4 R12 lvel3 avel3
static const int CONTACT_IN = 16;  // pos3 normal3 depth mu mu2 bounce bounce_vel soft_erp soft_cfm slip1 slip2 pad

static void set_body(dBodyID b, const float *s) {
    dBodySetPosition(b, s[0], s[1], s[2]);
    dQuaternion q = {s[3], s[4], s[5], s[6]};
    dBodySetQuaternion(b, q);
    dBodySetLinearVel(b, s[7], s[8], s[9]);
    dBodySetAngularVel(b, s[10], s[11], s[12]);
    dMass m;
    dMassSetParameters(&m, s[13], 0, 0, 0, s[14], s[15], s[16], s[17], s[18], s[19]);
    dBodySetMass(b, &m);
}
static void get_body(dBodyID b, float *o) {
    const dReal *p = dBodyGetPosition(b), *q = dBodyGetQuaternion(b), *R = dBodyGetRotation(b);
    const dReal *lv = dBodyGetLinearVel(b), *av = dBodyGetAngularVel(b);
    for (int j = 0; j < 3; j++) o[j] = (float)p[j];
    for (int j = 0; j < 4; j++) o[3 + j] = (float)q[j];
    for (int j = 0; j < 12; j++) o[7 + j] = (float)R[j];
    for (int j = 0; j < 3; j++) { o[19 + j] = (float)lv[j]; o[22 + j] = (float)av[j]; }
}
static void fill_contact(dContact &c, int mode, const float *s) {
    memset(&c, 0, sizeof c);
    c.surface.mode = mode;
    c.surface.mu = s[7]; c.surface.mu2 = s[8]; c.surface.bounce = s[9]; c.surface.bounce_vel = s[10];
    c.surface.soft_erp = s[11]; c.surface.soft_cfm = s[12]; c.surface.slip1 = s[13]; c.surface.slip2 = s[14];
    for (int j = 0; j < 3; j++) { c.geom.pos[j] = s[j]; c.geom.normal[j] = s[3 + j]; }
    c.geom.depth = s[6];
}
// Recover per-row lambda of a contact joint from its feedback: the three J1
// linear rows are the orthonormal frame (n, t1, t2) (contact.cpp:169-293), so
// lambda_k = f1 . dir_k.  The frame is rebuilt exactly as getInfo2 does.
static void contact_lambda(const dContact &c, bool reversed, const dJointFeedback &fb, float *lam) {
    dVector3 n, t1, t2;
    for (int j = 0; j < 3; j++) n[j] = reversed ? -c.geom.normal[j] : c.geom.normal[j];
    n[3] = 0;
    dPlaneSpace(n, t1, t2);
    lam[0] = (float)dCalcVectorDot3(fb.f1, n);
    lam[1] = (float)dCalcVectorDot3(fb.f1, t1);
    lam[2] = (float)dCalcVectorDot3(fb.f1, t2);
}

// dyn 0: the dynamic iteration rule off; 1: on at the reference's defaults;
// 2: on with the parameters in g_dynp (premature exit delta, extra factor,
// extra iteration delta), read by the step mode
static dReal g_dynp[3] = {0, 0, 0};
static void apply_params(dWorldID w, const WorldParams &P, int iters, int dyn) {
    dWorldSetGravity(w, P.g[0], P.g[1], P.g[2]);
    dWorldSetERP(w, P.erp);
    dWorldSetCFM(w, P.cfm);
    dWorldSetQuickStepNumIterations(w, iters);
    dWorldSetQuickStepW(w, P.w);
    dWorldSetContactMaxCorrectingVel(w, P.max_vel);
    dWorldSetContactSurfaceLayer(w, P.min_depth);
    if (!dyn) {
        dReal zero = 0;
        dWorldSetQuickStepDynamicIterationParameters(w, &zero, &zero, NULL);
    } else if (dyn == 2) {
        dWorldSetQuickStepDynamicIterationParameters(w, &g_dynp[0], &g_dynp[1], &g_dynp[2]);
    }
}

// ---------------------------------------------------------------- step
static void mode_step() {
    int nb = rdi(), nc = rdi(), iters = rdi(), dyn = rdi(), stepper = rdi();
    WorldParams P; rd((float *)&P, sizeof(P) / sizeof(float));
    if (dyn == 2) {
        float d3[3];
        rd(d3, 3);
        for (int i = 0; i < 3; i++) g_dynp[i] = d3[i];
    }
    std::vector<float> bodies(BODY_IN * nb);
    rd(bodies.data(), bodies.size());
    std::vector<int> cb(2 * nc), cmode(nc);
    std::vector<float> cs(CONTACT_IN * nc);
    rd(cb.data(), cb.size()); rd(cmode.data(), nc); rd(cs.data(), cs.size());

    dWorldID w = dWorldCreate();
    apply_params(w, P, iters, dyn);
    std::vector<dBodyID> b(nb);
    for (int i = 0; i < nb; i++) { b[i] = dBodyCreate(w); set_body(b[i], &bodies[BODY_IN * i]); }
    dJointGroupID grp = dJointGroupCreate(0);
    std::vector<dJointFeedback> fb(nc);
    std::vector<dContact> cc(nc);
    for (int k = 0; k < nc; k++) {
        fill_contact(cc[k], cmode[k], &cs[CONTACT_IN * k]);
        dJointID j = dJointCreateContact(w, grp, &cc[k]);
        dJointAttach(j, cb[2 * k] >= 0 ? b[cb[2 * k]] : 0, cb[2 * k + 1] >= 0 ? b[cb[2 * k + 1]] : 0);
        dJointSetFeedback(j, &fb[k]);
    }
    int ok = stepper ? dWorldStep(w, P.dt) : dWorldQuickStep(w, P.dt);
    std::vector<float> lam(3 * nc), raw(12 * nc), out(BODY_OUT * nb);
    for (int k = 0; k < nc; k++) {
        contact_lambda(cc[k], cb[2 * k] < 0, fb[k], &lam[3 * k]);
        for (int j = 0; j < 3; j++) {
            raw[12 * k + j] = fb[k].f1[j]; raw[12 * k + 3 + j] = fb[k].t1[j];
            raw[12 * k + 6 + j] = fb[k].f2[j]; raw[12 * k + 9 + j] = fb[k].t2[j];
        }
    }
    for (int i = 0; i < nb; i++) get_body(b[i], &out[BODY_OUT * i]);
    wr(&ok, 1); wr(lam.data(), lam.size()); wr(raw.data(), raw.size()); wr(out.data(), out.size());
    dJointGroupDestroy(grp);
    dWorldDestroy(w);
}

// ---------------------------------------------------------------- loop
struct LoopCtx {
    dWorldID world; dJointGroupID group; int maxc; int mode; float surf[8];
    std::vector<dContact> made; std::vector<int> made_b;
    std::vector<dBodyID> *bodies; bool record;
};
static int body_index(LoopCtx *L, dBodyID b) {
    if (!b) return -1;
    return (int)(std::find(L->bodies->begin(), L->bodies->end(), b) - L->bodies->begin());
}
static void loop_cb(void *data, dGeomID o1, dGeomID o2) {
    LoopCtx *L = (LoopCtx *)data;
    dBodyID b1 = dGeomGetBody(o1), b2 = dGeomGetBody(o2);
    dContact contact[16];
    for (int i = 0; i < L->maxc; i++) {
        memset(&contact[i], 0, sizeof(dContact));
        contact[i].surface.mode = L->mode;
        contact[i].surface.mu = L->surf[0]; contact[i].surface.mu2 = L->surf[1];
        contact[i].surface.bounce = L->surf[2]; contact[i].surface.bounce_vel = L->surf[3];
        contact[i].surface.soft_erp = L->surf[4]; contact[i].surface.soft_cfm = L->surf[5];
    }
    int n = dCollide(o1, o2, L->maxc, &contact[0].geom, sizeof(dContact));
    for (int i = 0; i < n; i++) {
        dJointID c = dJointCreateContact(L->world, L->group, &contact[i]);
        dJointAttach(c, b1, b2);
        L->made.push_back(contact[i]);
        L->made_b.push_back(body_index(L, b1));
        L->made_b.push_back(body_index(L, b2));
    }
}
static void mode_loop() {
    int nb = rdi(), ng = rdi(), nsteps = rdi(), iters = rdi(), dyn = rdi(), maxc = rdi(), mode = rdi(), nsnap = rdi();
    int minlevel = rdi(), maxlevel = rdi();
    WorldParams P; rd((float *)&P, sizeof(P) / sizeof(float));
    float surf[8]; rd(surf, 8);
    std::vector<int> snap(nsnap); rd(snap.data(), nsnap);
    std::vector<float> bodies(BODY_IN * nb); rd(bodies.data(), bodies.size());
    std::vector<int> gcls(ng), gbody(ng);
    std::vector<float> gpos(3 * ng), gR(12 * ng), gdims(4 * ng);
    rd(gcls.data(), ng); rd(gbody.data(), ng); rd(gpos.data(), gpos.size()); rd(gR.data(), gR.size()); rd(gdims.data(), gdims.size());

    dWorldID w = dWorldCreate();
    apply_params(w, P, iters, dyn);
    std::vector<dBodyID> b(nb);
    for (int i = 0; i < nb; i++) { b[i] = dBodyCreate(w); set_body(b[i], &bodies[BODY_IN * i]); }
    dSpaceID sp = dHashSpaceCreate(0);
    dHashSpaceSetLevels(sp, minlevel, maxlevel);
    for (int i = 0; i < ng; i++) {
        dGeomID g = make_geom(sp, gcls[i], &gpos[3 * i], &gR[12 * i], &gdims[4 * i]);
        if (gbody[i] >= 0) dGeomSetBody(g, b[gbody[i]]);
    }
    LoopCtx L; L.world = w; L.group = dJointGroupCreate(0); L.maxc = maxc; L.mode = mode;
    memcpy(L.surf, surf, sizeof surf); L.bodies = &b;
    std::vector<float> traj((size_t)nsteps * nb * 7);
    int si = 0;
    for (int s = 0; s < nsteps; s++) {
        bool snapnow = si < nsnap && snap[si] == s;
        std::vector<float> pre(BODY_OUT * nb);
        if (snapnow) for (int i = 0; i < nb; i++) get_body(b[i], &pre[BODY_OUT * i]);
        L.made.clear(); L.made_b.clear();
        dSpaceCollide(sp, &L, &loop_cb);
        int nc = (int)L.made.size();
        dWorldQuickStep(w, P.dt);
        if (snapnow) {
            std::vector<float> post(BODY_OUT * nb);
            for (int i = 0; i < nb; i++) get_body(b[i], &post[BODY_OUT * i]);
            int step = s;
            wr(&step, 1); wr(&nc, 1);
            wr(pre.data(), pre.size());
            std::vector<float> cs(CONTACT_IN * nc, 0.f);
            for (int k = 0; k < nc; k++) {
                const dContact &c = L.made[k];
                for (int j = 0; j < 3; j++) { cs[CONTACT_IN * k + j] = c.geom.pos[j]; cs[CONTACT_IN * k + 3 + j] = c.geom.normal[j]; }
                cs[CONTACT_IN * k + 6] = c.geom.depth;
                cs[CONTACT_IN * k + 7] = c.surface.mu; cs[CONTACT_IN * k + 8] = c.surface.mu2;
                cs[CONTACT_IN * k + 9] = c.surface.bounce; cs[CONTACT_IN * k + 10] = c.surface.bounce_vel;
                cs[CONTACT_IN * k + 11] = c.surface.soft_erp; cs[CONTACT_IN * k + 12] = c.surface.soft_cfm;
            }
            wr(L.made_b.data(), L.made_b.size());
            wr(cs.data(), cs.size());
            wr(post.data(), post.size());
            si++;
        }
        dJointGroupEmpty(L.group);
        for (int i = 0; i < nb; i++) {
            const dReal *p = dBodyGetPosition(b[i]), *q = dBodyGetQuaternion(b[i]);
            float *o = &traj[((size_t)s * nb + i) * 7];
            for (int j = 0; j < 3; j++) o[j] = (float)p[j];
            for (int j = 0; j < 4; j++) o[3 + j] = (float)q[j];
        }
    }
    wr(traj.data(), traj.size());
    dJointGroupDestroy(L.group);
    dSpaceDestroy(sp);
    dWorldDestroy(w);
}

// ---------------------------------------------------------------- sleep
// The loop of mode_loop with auto-disable on in the world (flag, linear and
// angular thresholds, steps, time, average samples, read after the geoms):
// per step the poses and every body's dBodyIsEnabled.
static void mode_sleep() {
    int nb = rdi(), ng = rdi(), nsteps = rdi(), iters = rdi(), dyn = rdi(), maxc = rdi(), mode = rdi();
    int minlevel = rdi(), maxlevel = rdi();
    WorldParams P; rd((float *)&P, sizeof(P) / sizeof(float));
    float surf[8]; rd(surf, 8);
    std::vector<float> bodies(BODY_IN * nb); rd(bodies.data(), bodies.size());
    std::vector<int> gcls(ng), gbody(ng);
    std::vector<float> gpos(3 * ng), gR(12 * ng), gdims(4 * ng);
    rd(gcls.data(), ng); rd(gbody.data(), ng); rd(gpos.data(), gpos.size()); rd(gR.data(), gR.size()); rd(gdims.data(), gdims.size());
    float adis[6]; rd(adis, 6);
    dWorldID w = dWorldCreate();
    apply_params(w, P, iters, dyn);
    dWorldSetAutoDisableFlag(w, adis[0] != 0);
    dWorldSetAutoDisableLinearThreshold(w, adis[1]);
    dWorldSetAutoDisableAngularThreshold(w, adis[2]);
    dWorldSetAutoDisableSteps(w, (int)adis[3]);
    dWorldSetAutoDisableTime(w, adis[4]);
    dWorldSetAutoDisableAverageSamplesCount(w, (unsigned)adis[5]);
    std::vector<dBodyID> b(nb);
    for (int i = 0; i < nb; i++) { b[i] = dBodyCreate(w); set_body(b[i], &bodies[BODY_IN * i]); }
    dSpaceID sp = dHashSpaceCreate(0);
    dHashSpaceSetLevels(sp, minlevel, maxlevel);
    for (int i = 0; i < ng; i++) {
        dGeomID g = make_geom(sp, gcls[i], &gpos[3 * i], &gR[12 * i], &gdims[4 * i]);
        if (gbody[i] >= 0) dGeomSetBody(g, b[gbody[i]]);
    }
    LoopCtx L; L.world = w; L.group = dJointGroupCreate(0); L.maxc = maxc; L.mode = mode;
    memcpy(L.surf, surf, sizeof surf); L.bodies = &b;
    std::vector<float> traj((size_t)nsteps * nb * 7);
    std::vector<int> en((size_t)nsteps * nb);
    for (int s = 0; s < nsteps; s++) {
        L.made.clear(); L.made_b.clear();
        dSpaceCollide(sp, &L, &loop_cb);
        dWorldQuickStep(w, P.dt);
        dJointGroupEmpty(L.group);
        for (int i = 0; i < nb; i++) {
            const dReal *p = dBodyGetPosition(b[i]), *q = dBodyGetQuaternion(b[i]);
            float *o = &traj[((size_t)s * nb + i) * 7];
            for (int j = 0; j < 3; j++) o[j] = (float)p[j];
            for (int j = 0; j < 4; j++) o[3 + j] = (float)q[j];
            en[(size_t)s * nb + i] = dBodyIsEnabled(b[i]);
        }
    }
    wr(traj.data(), traj.size());
    wr(en.data(), en.size());
    dJointGroupDestroy(L.group);
    dSpaceDestroy(sp);
    dWorldDestroy(w);
}

// ---------------------------------------------------------------- chain
static void mode_chain() {
    // dyn bit 0: the reference's dynamic iteration rule; bit 1: dWorldStep instead of dWorldQuickStep
    int nb = rdi(), nj = rdi(), nsteps = rdi(), iters = rdi(), dyn = rdi();
    const bool stepper = (dyn & 2) != 0;
    dyn &= 1;
    WorldParams P; rd((float *)&P, sizeof(P) / sizeof(float));
    std::vector<float> bodies(BODY_IN * nb); rd(bodies.data(), bodies.size());
    const int JC = 20;
    std::vector<float> jt(JC * nj); rd(jt.data(), jt.size());
    float damp[5]; rd(damp, 5);  // linear/angular scale, linear/angular threshold, max angular speed
    dWorldID w = dWorldCreate();
    apply_params(w, P, iters, dyn);
    dWorldSetDamping(w, damp[0], damp[1]);
    dWorldSetLinearDampingThreshold(w, damp[2]);
    dWorldSetAngularDampingThreshold(w, damp[3]);
    dWorldSetMaxAngularSpeed(w, damp[4]);
    std::vector<dBodyID> b(nb);
    for (int i = 0; i < nb; i++) { b[i] = dBodyCreate(w); set_body(b[i], &bodies[BODY_IN * i]); }
    std::vector<dJointID> hinges;
    std::vector<dJointID> hinge2s;
    for (int k = 0; k < nj; k++) {
        const float *r = &jt[JC * k];
        const int t = (int)r[0], b1 = (int)r[1], b2 = (int)r[2];
        dJointID j = t == 1 ? dJointCreateBall(w, 0) : (t == 2 ? dJointCreateHinge(w, 0) : dJointCreateHinge2(w, 0));
        dJointAttach(j, b[b1], b2 >= 0 ? b[b2] : 0);
        if (t == 1) {
            dJointSetBallAnchor(j, r[3], r[4], r[5]);
        } else if (t == 2) {
            dJointSetHingeAnchor(j, r[3], r[4], r[5]);
            dJointSetHingeAxis(j, r[6], r[7], r[8]);
            dJointSetHingeParam(j, dParamLoStop, r[9]);
            dJointSetHingeParam(j, dParamHiStop, r[10]);
            if (r[19] > 0) { dJointSetHingeParam(j, dParamVel, r[18]); dJointSetHingeParam(j, dParamFMax, r[19]); }
            hinges.push_back(j);
        } else {
            dJointSetHinge2Anchor(j, r[3], r[4], r[5]);
            const dReal a1[4] = {r[6], r[7], r[8], 0}, a2[4] = {r[11], r[12], r[13], 0};
            dJointSetHinge2Axes(j, a1, a2);
            dJointSetHinge2Param(j, dParamLoStop, r[9]);
            dJointSetHinge2Param(j, dParamHiStop, r[10]);
            dJointSetHinge2Param(j, dParamVel2, r[14]);
            dJointSetHinge2Param(j, dParamFMax2, r[15]);
            dJointSetHinge2Param(j, dParamSuspensionERP, r[16]);
            dJointSetHinge2Param(j, dParamSuspensionCFM, r[17]);
            hinge2s.push_back(j);
        }
    }
    // angles: the hinges' dJointGetHingeAngle, then the hinge2s' dJointGetHinge2Angle1
    for (dJointID j : hinge2s) hinges.push_back(j);
    const int nh = (int)hinges.size(), nh1 = nh - (int)hinge2s.size();
    std::vector<float> traj((size_t)nsteps * nb * 7), ang((size_t)nsteps * nh);
    for (int s = 0; s < nsteps; s++) {
        if (stepper) dWorldStep(w, P.dt);
        else dWorldQuickStep(w, P.dt);
        for (int i = 0; i < nb; i++) {
            const dReal *p = dBodyGetPosition(b[i]), *q = dBodyGetQuaternion(b[i]);
            float *o = &traj[((size_t)s * nb + i) * 7];
            for (int j = 0; j < 3; j++) o[j] = (float)p[j];
            for (int j = 0; j < 4; j++) o[3 + j] = (float)q[j];
        }
        for (int h = 0; h < nh; h++)
            ang[(size_t)s * nh + h] =
                (float)(h < nh1 ? dJointGetHingeAngle(hinges[h]) : dJointGetHinge2Angle1(hinges[h]));
    }
    wr(traj.data(), traj.size());
    wr(ang.data(), ang.size());
    dWorldDestroy(w);
}

// ---------------------------------------------------------------- timing
struct TimingCtx { dWorldID world; dJointGroupID group; int maxc; int mode; float surf[8]; int made; };
static void timing_cb(void *data, dGeomID o1, dGeomID o2) {
    TimingCtx *T = (TimingCtx *)data;
    dBodyID b1 = dGeomGetBody(o1), b2 = dGeomGetBody(o2);
    dContact contact[16];
    for (int i = 0; i < T->maxc; i++) {
        memset(&contact[i], 0, sizeof(dContact));
        contact[i].surface.mode = T->mode;
        contact[i].surface.mu = T->surf[0]; contact[i].surface.mu2 = T->surf[1];
        contact[i].surface.bounce = T->surf[2]; contact[i].surface.bounce_vel = T->surf[3];
        contact[i].surface.soft_erp = T->surf[4]; contact[i].surface.soft_cfm = T->surf[5];
    }
    int n = dCollide(o1, o2, T->maxc, &contact[0].geom, sizeof(dContact));
    for (int i = 0; i < n; i++) {
        dJointID c = dJointCreateContact(T->world, T->group, &contact[i]);
        dJointAttach(c, b1, b2);
    }
    T->made += n;
}
static void mode_timing() {
    int nb = rdi(), ng = rdi(), nsteps = rdi(), iters = rdi(), threads = rdi(), maxc = rdi(), mode = rdi();
    int minlevel = rdi(), maxlevel = rdi();
    WorldParams P; rd((float *)&P, sizeof(P) / sizeof(float));
    float surf[8]; rd(surf, 8);
    std::vector<float> bodies(BODY_IN * nb); rd(bodies.data(), bodies.size());
    std::vector<int> gcls(ng), gbody(ng);
    std::vector<float> gpos(3 * ng), gR(12 * ng), gdims(4 * ng);
    rd(gcls.data(), ng); rd(gbody.data(), ng); rd(gpos.data(), gpos.size()); rd(gR.data(), gR.size()); rd(gdims.data(), gdims.size());

    dWorldID w = dWorldCreate();
    apply_params(w, P, iters, 0);
    dThreadingImplementationID impl = 0;
    dThreadingThreadPoolID pool = 0;
    if (threads > 1) {
        impl = dThreadingAllocateMultiThreadedImplementation();
        pool = dThreadingAllocateThreadPool(threads, 0, dAllocateFlagBasicData, NULL);
        dThreadingThreadPoolServeMultiThreadedImplementation(pool, impl);
        dWorldSetStepIslandsProcessingMaxThreadCount(w, threads);
        dWorldSetStepThreadingImplementation(w, dThreadingImplementationGetFunctions(impl), impl);
    }
    std::vector<dBodyID> b(nb);
    for (int i = 0; i < nb; i++) { b[i] = dBodyCreate(w); set_body(b[i], &bodies[BODY_IN * i]); }
    dSpaceID sp = dHashSpaceCreate(0);
    dHashSpaceSetLevels(sp, minlevel, maxlevel);
    for (int i = 0; i < ng; i++) {
        dGeomID g = make_geom(sp, gcls[i], &gpos[3 * i], &gR[12 * i], &gdims[4 * i]);
        if (gbody[i] >= 0) dGeomSetBody(g, b[gbody[i]]);
    }
    TimingCtx T; T.world = w; T.group = dJointGroupCreate(0); T.maxc = maxc; T.mode = mode;
    memcpy(T.surf, surf, sizeof surf);
    std::vector<double> out;
    typedef std::chrono::steady_clock clk;
    for (int s = 0; s < nsteps; s++) {
        T.made = 0;
        const clk::time_point t0 = clk::now();
        dSpaceCollide(sp, &T, &timing_cb);
        const clk::time_point t1 = clk::now();
        dWorldQuickStep(w, P.dt);
        dJointGroupEmpty(T.group);
        const clk::time_point t2 = clk::now();
        out.push_back(std::chrono::duration<double>(t1 - t0).count());
        out.push_back(std::chrono::duration<double>(t2 - t1).count());
        out.push_back((double)T.made);
    }
    wr(out.data(), out.size());
    std::vector<float> st(BODY_OUT * nb);
    for (int i = 0; i < nb; i++) get_body(b[i], &st[BODY_OUT * i]);
    wr(st.data(), st.size());
    dJointGroupDestroy(T.group);
    if (impl) {
        dThreadingImplementationShutdownProcessing(impl);
        dThreadingFreeThreadPool(pool);
        dWorldSetStepThreadingImplementation(w, NULL, NULL);
        dThreadingFreeImplementation(impl);
    }
    dSpaceDestroy(sp);
    dWorldDestroy(w);
}

int main(int argc, char **argv) {
    if (argc != 4) { fprintf(stderr, "usage: gen_golden MODE IN OUT\n"); return 2; }
    fin = fopen(argv[2], "rb"); fout = fopen(argv[3], "wb");
    if (!fin || !fout) { fprintf(stderr, "cannot open files\n"); return 2; }
    dInitODE2(0);
    if (!strcmp(argv[1], "colliders")) mode_colliders();
    else if (!strcmp(argv[1], "space")) mode_space();
    else if (!strcmp(argv[1], "step")) mode_step();
    else if (!strcmp(argv[1], "loop")) mode_loop();
    else if (!strcmp(argv[1], "chain")) mode_chain();
    else if (!strcmp(argv[1], "sleep")) mode_sleep();
    else if (!strcmp(argv[1], "timing")) mode_timing();
    else { fprintf(stderr, "bad mode\n"); return 2; }
    dCloseODE();
    fclose(fin); fclose(fout);
    return 0;
}
