// The C-ABI layer: ODE's public functions for the rigid-body hot path, backed
// by the device pipeline in collide.cu / solve.cu.
//
// Host objects keep only what ODE's API exposes (handles, parameters, user
// data, the bodies' host-visible state) and a dirty/valid protocol against the
// device copy: setters mark the world's device state dirty and it is uploaded
// whole before the next device step; getters download the whole body state
// once after a step.  Argument checking follows ODE's release build: invalid
// handles are the caller's responsibility, device failures are reported
// through the return value (0) and gbodeGetLastError(), never by aborting.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <algorithm>
#include <vector>

#include "../../include/gbode.h"
#include "gbode_internal.h"

using namespace gb;

// ------------------------------------------------------------------ infrastructure
namespace gb {
static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }
int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}
TestFaults g_test;

// an injected allocation failure (gbodeTestInject), as cudaMalloc failing
static bool injected_alloc_failure() {
    if (g_test.alloc_skip < 0) return false;
    if (g_test.alloc_skip > 0) { --g_test.alloc_skip; return false; }
    if (--g_test.alloc_fail <= 0) g_test.alloc_skip = -1;
    return true;
}

// The new block is allocated before the old one is released: a failed grow
// leaves the buffer (and its contents) as it was.
bool DBuf::ensure(size_t want) {
    if (want <= bytes && p) return true;
    size_t nb = bytes ? bytes : 256;
    while (nb < want) nb = nb + nb / 2 + 256;
    if (injected_alloc_failure()) return false;
    void *np = nullptr;
    if (cudaMalloc(&np, nb) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (p) cudaFree(p);
    p = np;
    bytes = nb;
    return true;
}
void DBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}
void Workspace::release() {
    DBuf *all[] = {&g_cls, &g_body, &g_dims, &g_spos, &g_sR, &g_pos, &g_R, &g_amin, &g_amax, &g_level, &g_dblo, &g_dbhi,
                   &g_big, &h_keys, &h_count, &h_start, &h_fill, &h_members, &h_entry, &p_count, &p_start, &pairs,
                   &c_slots, &c_count, &c_start, &contacts, &surfaces, &c_mcount, &c_rstart, &c_code, &b_pos, &b_q,
                   &b_R, &b_lvel, &b_avel, &b_facc, &b_tacc, &b_Ib, &b_invIb, &b_invIw, &b_fc, &b_rt, &b_fa, &r_J1l,
                   &r_J1a, &r_J2l, &r_J2a, &r_M1l, &r_M1a, &r_M2l, &r_M2a, &r_lambda, &r_Ad, &r_findex, &r_contact,
                   &r_body, &m_head, &m_id, &m_start, &m_colour, &m_mask, &m_claim, &m_tent, &col_count, &col_start,
                   &col_fill, &col_list, &m_desc, &p_rows, &chunk_rows, &chunk_start, &wv_count, &wv_base, &wv_col, &wv_sched, &l_feat, &l_scale, &l_pred, &l_alt, &mlp_P, &mlp_wb, &j_info, &j_a1, &j_a2, &j_x1, &j_x2, &j_qrel, &j_l0, &j_l1, &j_l2, &j_m, &j_rstart, &j_limit, &j_lerr, &j_lam, &grp_body, &j_pairs, &b_damp, &b_maxw, &b_adis_i, &b_adis_f, &b_adis_buf, &b_touch, &b_parent, &b_awake, &b_asleep, &c_keep, &c_kpos, &c_awake, &c_orig, &j_v1, &j_v2, &j_m0, &j_m1, &j_m2, &i_order, &i_start, &i_bodies, &i_bstart, &i_normals, &d_off, &d_scr, &d_iscr, &d_rloc, &w_keys, &w_lambda,
                   &w_keys_prev, &w_lambda_prev, &res_f, &res_v, &scan_tmp, &s_bw, &s_part, &s_blocal, &s_pbcount,
                   &s_pbody, &s_prow, &s_pgrp, &s_gpart, &s_gdesc, &s_pccount, &s_pcstart, &s_pcfill, &s_ilist,
                   &s_irown, &s_irowoff, &s_idesc, &s_ipack, &s_hist, &s_binpart, &n_perm, &n_key, &x_cnt,
                   &x_start, &x_fill, &x_accn, &x_acc, &x_adj, &x_prog, &x_nsplit, &x_dacc, &x_smask, &m_lprev,
                   &b_fcprev, &p_cache};
    for (DBuf *b : all) b->release();
    if (dc) cudaFree(dc);
    if (hc) cudaFreeHost(hc);
    dc = nullptr;
    hc = nullptr;
}
}  // namespace gb

static thread_local std::string g_err;
static void set_error(const char *where, cudaError_t e = cudaSuccess) {
    char buf[256];
    if (e != cudaSuccess) snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
    else snprintf(buf, sizeof buf, "%s", where);
    g_err = buf;
}
namespace gb {
void report_error(const char *msg) { set_error(msg); }
}  // namespace gb

// ------------------------------------------------------------------ objects
struct dxJoint;
struct dxGeom;

struct dxBody {
    dxWorld *world;
    int index;
    void *data = nullptr;
    float pos[4] = {0, 0, 0, 0}, q[4] = {1, 0, 0, 0}, R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    float lvel[4] = {0, 0, 0, 0}, avel[4] = {0, 0, 0, 0}, facc[4] = {0, 0, 0, 0}, tacc[4] = {0, 0, 0, 0};
    dMass mass;
    float invI[12];
    float invMass = 1;
    int gyro = 1;  // ode.cpp:283 -- dBodyCreate enables the implicit gyroscopic term
    // damping (objects.h:100-108: scales, squared thresholds; scale 0 = off) and angular speed cap
    float damp[4] = {0, 0, 0.01f * 0.01f, 0.01f * 0.01f};
    float max_w = INFINITY;
    int njoints = 0;
    // auto-disable (objects.h:73-84 dxAutoDisable, ode.cpp:240-285, :887-1020):
    // GB_ADIS_* flags, countdowns, squared thresholds, velocity ring buffer
    int adis_flags = 0, adis_counter = 0;
    int adis_idle_steps = 10, adis_steps_left = 10, adis_samples = 1;
    float adis_lin = 0.01f * 0.01f, adis_ang = 0.01f * 0.01f, adis_idle_time = 0, adis_time_left = 0;
    std::vector<float> adis_buf;  // adis_samples x (lvel xyz_, avel xyz_)
};

struct dxSpace;
struct dxGeom {
    int cls;
    dxSpace *space = nullptr;
    dxBody *body = nullptr;
    void *data = nullptr;
    float dims[4] = {0, 0, 0, 0};
    float pos[4] = {0, 0, 0, 0};
    float R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    int index = -1;  // position in its space
    int uid = 0;     // creation serial (warm-start keys of contact joints)
};
static int g_geom_uid = 0;

struct dxSpace {
    std::vector<dxGeom *> geoms;
    int minlevel = -3, maxlevel = 10;  // collision_space.cpp:371-376
    int cleanup = 1;
    int exact_pairs = 0;               // 1: report every overlapping pair (see gbodeHashSpaceSetExactPairs)
    bool dirty = true;                 // geom set or static poses changed since the last upload
};

struct dxJointGroup {
    std::vector<dxJoint *> joints;
    dxWorld *device_world = nullptr;   // world holding this group's device-resident contacts
};

// joints/joint.cpp:495-509 dxJointLimitMotor::init (set from the world's ERP/CFM at creation)
struct Limot {
    float vel = 0, fmax = 0, lostop = -INFINITY, histop = INFINITY, fudge_factor = 1, normal_cfm = 0,
          stop_erp = 0, stop_cfm = 0, bounce = 0;
};

struct dxJoint {
    dxWorld *world;
    dxJointGroup *group;
    int type = dJointTypeContact;
    dContact contact;
    dxBody *b1 = nullptr, *b2 = nullptr;  // as attached; node[0] is b1, or b2 when b1 is null
    bool attached = false;
    dJointFeedback *feedback = nullptr;
    // ball and hinge (joints/ball.cpp, joints/hinge.cpp): anchors and axes in
    // the bodies' frames, hinge reference orientation, ball ERP/CFM, hinge limit/motor
    float anchor1[4] = {0, 0, 0, 0}, anchor2[4] = {0, 0, 0, 0};
    float axis1[4] = {1, 0, 0, 0}, axis2[4] = {1, 0, 0, 0}, qrel[4] = {0, 0, 0, 0};
    float erp = 0, cfm = 0;
    Limot limot;
    // hinge2 (joints/hinge2.cpp): angle-measuring vectors in body 1's frame,
    // sin/cos of the rest angle between the axes, suspension, axis-2 motor
    float v1[4] = {1, 0, 0, 0}, v2[4] = {0, 1, 0, 0}, s0 = 0, c0 = 0, susp_erp = 0, susp_cfm = 0;
    Limot limot2;
    dxBody *node0() const { return b1 ? b1 : b2; }
    dxBody *node1() const { return b1 ? b2 : nullptr; }
};

struct dxWorld {
    Workspace ws;
    SolverParams P;
    std::vector<dxBody *> bodies;
    std::vector<dxJoint *> joints;
    bool joints_dirty = false;  // ball/hinge joints changed since the last upload
    // defaults copied into bodies at creation (objects.cpp:63-69, ode.cpp:265-285)
    float damp[4] = {0, 0, 0.01f * 0.01f, 0.01f * 0.01f};
    float max_w = INFINITY;
    // auto-disable defaults (objects.cpp:55-60) and the world's flag
    int adis_on = 0, adis_idle_steps = 10, adis_samples = 1;
    float adis_lin = 0.01f * 0.01f, adis_ang = 0.01f * 0.01f, adis_idle_time = 0;
    // gbodeWorldStepFused's CUDA graph of one fused step
    int graph_state = 0;  // 0 none, 1 capture on the next call, 2 replaying
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> graph_key;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool dev_dirty = true;    // host body state newer than device
    bool host_valid = true;   // host body state equals device
    dxSpace *uploaded_space = nullptr;
    bool device_contacts = false;
    int device_surfaces = 0;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    gbodeStepStats stats{};
    bool stats_pending = false;
    int last_host_contacts = 0;
    std::vector<dxJoint *> table_joints;  // the ball/hinge/hinge2 joints in device-table order
    struct DevSnapshot *snapshot = nullptr;  // gbodeWorldSaveSnapshot
    // pinned staging of the bulk state calls (pos, q, R rows, lvel, avel: 112 B a body)
    float4 *stage_up = nullptr, *stage_down = nullptr;
    size_t stage_up_n = 0, stage_down_n = 0;  // bodies each holds
    cudaEvent_t stage_up_done = nullptr;      // the last upload from stage_up has been copied
};

// Pinned staging for n bodies (112 B each); false when it cannot be allocated
// (the callers then take the path through the body records).
static bool stage_ensure(float4 *&p, size_t &cap, size_t n, cudaEvent_t pending) {
    if (cap >= n && p) return true;
    if (pending) cudaEventSynchronize(pending);
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, 112 * (n > 0 ? n : 1)) != cudaSuccess) {
        (void)cudaGetLastError();
        p = nullptr;
        return false;
    }
    cap = n;
    return true;
}

// A copy of a world's device-side simulation state: bodies, the warm-start
// tables, the joints' multipliers, the auto-disable state and the counters.
// Everything else on the device is rebuilt by every step.
struct DevSnapshot {
    std::vector<DBuf> copies;
    std::vector<size_t> sizes;  // each source buffer's size at the save (0: not allocated)
    int nbodies = 0;
    bool warm_valid = false;
    unsigned warm_mask = 0;
    bool valid = false;
    void release() {
        for (DBuf &c : copies) c.release();
        copies.clear();
        sizes.clear();
        valid = false;
    }
};

static int snapshot_sources(Workspace &ws, DBuf **out) {
    DBuf *keep[] = {&ws.b_pos, &ws.b_q, &ws.b_R, &ws.b_lvel, &ws.b_avel, &ws.b_facc, &ws.b_tacc, &ws.w_keys,
                    &ws.w_lambda, &ws.j_lam, &ws.b_adis_i, &ws.b_adis_f, &ws.b_adis_buf};
    const int n = (int)(sizeof keep / sizeof keep[0]);
    for (int k = 0; k < n; k++) out[k] = keep[k];
    return n;
}
static const int SNAP_MAX = 16;

// Copies the state aside on the world's stream and waits for the copies.
static bool snapshot_save(dxWorld *w, DevSnapshot &S) {
    Workspace &ws = w->ws;
    DBuf *src[SNAP_MAX];
    const int n = snapshot_sources(ws, src);
    S.valid = false;
    S.copies.resize(n + 1);
    S.sizes.assign(n, 0);
    for (int k = 0; k < n; k++) {
        if (!src[k]->p) continue;
        S.sizes[k] = src[k]->bytes;
        if (!S.copies[k].ensure(src[k]->bytes)) return false;
        cudaMemcpyAsync(S.copies[k].p, src[k]->p, src[k]->bytes, cudaMemcpyDeviceToDevice, w->stream);
    }
    if (!S.copies[n].ensure(sizeof(DevCounters))) return false;
    cudaMemcpyAsync(S.copies[n].p, ws.dc, sizeof(DevCounters), cudaMemcpyDeviceToDevice, w->stream);
    S.nbodies = (int)w->bodies.size();
    S.warm_valid = ws.warm_valid;
    S.warm_mask = ws.warm_mask;
    S.valid = cudaStreamSynchronize(w->stream) == cudaSuccess;
    return S.valid;
}

// false (nothing restored) when a buffer was allocated or resized since the save
static bool snapshot_fits(dxWorld *w, const DevSnapshot &S) {
    DBuf *src[SNAP_MAX];
    const int n = snapshot_sources(w->ws, src);
    if (!S.valid || (int)S.sizes.size() != n || S.nbodies != (int)w->bodies.size()) return false;
    for (int k = 0; k < n; k++)
        if ((src[k]->p ? src[k]->bytes : 0) != S.sizes[k]) return false;
    return true;
}

static bool snapshot_restore(dxWorld *w, const DevSnapshot &S) {
    if (!snapshot_fits(w, S)) return false;
    Workspace &ws = w->ws;
    DBuf *src[SNAP_MAX];
    const int n = snapshot_sources(ws, src);
    for (int k = 0; k < n; k++)
        if (S.sizes[k]) cudaMemcpyAsync(src[k]->p, S.copies[k].p, S.sizes[k], cudaMemcpyDeviceToDevice, w->stream);
    cudaMemcpyAsync(ws.dc, S.copies[n].p, sizeof(DevCounters), cudaMemcpyDeviceToDevice, w->stream);
    if (cudaStreamSynchronize(w->stream) != cudaSuccess) return false;
    ws.warm_valid = S.warm_valid && ws.warm_mask == S.warm_mask;
    w->host_valid = false;
    return true;
}

static dxWorld *g_default_world = nullptr;
static std::vector<dxWorld *> g_worlds;

// ------------------------------------------------------------------ small math (host)
// rotation.cpp:236-254 dRfromQ
static void r_from_q(float *R, const float *q) {
    float qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
    R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]); R[3] = 0;
    R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]); R[7] = 0;
    R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2; R[11] = 0;
}
// odemath.cpp:200-218 dxSafeNormalize4 with the dxNormalize4 fallback
static void normalize4(float *a) {
    float l = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3];
    if (l > 0) { l = 1.0f / sqrtf(l); a[0] *= l; a[1] *= l; a[2] *= l; a[3] *= l; }
    else { a[0] = 1; a[1] = a[2] = a[3] = 0; }
}
// rotation.cpp:257-307 dQfromR
static void q_from_r(float *q, const float *Rm) {
#define RR(i, j) Rm[(i) * 4 + (j)]
    float tr = RR(0, 0) + RR(1, 1) + RR(2, 2), s;
    if (tr >= 0) {
        s = sqrtf(tr + 1); q[0] = 0.5f * s; s = 0.5f * (1.0f / s);
        q[1] = (RR(2, 1) - RR(1, 2)) * s; q[2] = (RR(0, 2) - RR(2, 0)) * s; q[3] = (RR(1, 0) - RR(0, 1)) * s;
    } else if (RR(1, 1) > RR(0, 0) && !(RR(2, 2) > RR(1, 1))) {
        s = sqrtf((RR(1, 1) - (RR(2, 2) + RR(0, 0))) + 1); q[2] = 0.5f * s; s = 0.5f * (1.0f / s);
        q[3] = (RR(1, 2) + RR(2, 1)) * s; q[1] = (RR(0, 1) + RR(1, 0)) * s; q[0] = (RR(0, 2) - RR(2, 0)) * s;
    } else if ((RR(1, 1) > RR(0, 0) && RR(2, 2) > RR(1, 1)) || (!(RR(1, 1) > RR(0, 0)) && RR(2, 2) > RR(0, 0))) {
        s = sqrtf((RR(2, 2) - (RR(0, 0) + RR(1, 1))) + 1); q[3] = 0.5f * s; s = 0.5f * (1.0f / s);
        q[1] = (RR(2, 0) + RR(0, 2)) * s; q[2] = (RR(1, 2) + RR(2, 1)) * s; q[0] = (RR(1, 0) - RR(0, 1)) * s;
    } else {
        s = sqrtf((RR(0, 0) - (RR(1, 1) + RR(2, 2))) + 1); q[1] = 0.5f * s; s = 0.5f * (1.0f / s);
        q[2] = (RR(0, 1) + RR(1, 0)) * s; q[3] = (RR(2, 0) + RR(0, 2)) * s; q[0] = (RR(2, 1) - RR(1, 2)) * s;
    }
#undef RR
}
// matrix.cpp dxFactorCholesky + dxSolveCholesky + dxInvertPDMatrix for n = 3
// (row stride 4), the inversion dBodySetMass uses (ode.cpp:488-505).
static int invert_pd3(const float *A, float *Ainv) {
    float L[12], recip[3], X[3], y[3];
    memcpy(L, A, sizeof L);
    for (int i = 0; i < 3; i++) {
        float *aa = L + 4 * i;
        for (int j = 0; j < i; j++) {
            float sum = aa[j];
            const float *bb = L + 4 * j;
            for (int k = 0; k < j; k++) sum -= aa[k] * bb[k];
            aa[j] = sum * recip[j];
        }
        float sum = aa[i];
        for (int k = 0; k < i; k++) sum -= aa[k] * aa[k];
        if (sum <= 0.0f) return 0;
        float sq = sqrtf(sum);
        aa[i] = sq;
        recip[i] = 1.0f / sq;
    }
    memset(Ainv, 0, 12 * sizeof(float));
    for (int c = 0; c < 3; c++) {
        X[0] = X[1] = X[2] = 0; X[c] = 1.0f;
        for (int i = 0; i < 3; i++) {
            float sum = 0.0f;
            for (int k = 0; k < i; k++) sum += L[4 * i + k] * y[k];
            y[i] = (X[i] - sum) / L[4 * i + i];
        }
        for (int i = 2; i >= 0; i--) {
            float sum = 0.0f;
            for (int k = i + 1; k < 3; k++) sum += L[4 * k + i] * X[k];
            X[i] = (y[i] - sum) / L[4 * i + i];
        }
        for (int k = 0; k < 3; k++) Ainv[4 * k + c] = X[k];
    }
    return 1;
}

// ------------------------------------------------------------------ world plumbing
static bool world_init_device(dxWorld *w) {
    if (w->ws.dc) return true;
    cudaError_t e = cudaMalloc(&w->ws.dc, sizeof(DevCounters));
    if (e != cudaSuccess) { set_error("cudaMalloc(counters)", e); return false; }
    cudaMemset(w->ws.dc, 0, sizeof(DevCounters));
    e = cudaMallocHost(&w->ws.hc, sizeof(DevCounters));
    if (e != cudaSuccess) { set_error("cudaMallocHost", e); return false; }
    memset(w->ws.hc, 0, sizeof(DevCounters));
    if (!w->stream) {
        e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { set_error("cudaStreamCreate", e); return false; }
        w->own_stream = true;
    }
    for (int i = 0; i < 4; i++) cudaEventCreate(&w->ev[i]);
    return true;
}

static void world_download(dxWorld *w) {
    if (w->host_valid) return;
    int nb = (int)w->bodies.size();
    if (nb > 0) {
        std::vector<float4> pos(nb), q(nb), R(3 * nb), lv(nb), av(nb);
        cudaStream_t s = w->stream;
        cudaMemcpyAsync(pos.data(), w->ws.b_pos.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(q.data(), w->ws.b_q.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(R.data(), w->ws.b_R.p, 48 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(lv.data(), w->ws.b_lvel.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(av.data(), w->ws.b_avel.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        // sleeping bodies keep their force accumulators and auto-disable state
        const bool sl = w->ws.sleep_on;
        const int S = w->ws.adis_S;
        std::vector<float4> fa(sl ? nb : 0), ta(sl ? nb : 0), af(sl ? nb : 0), buf(sl ? (size_t)nb * S * 2 : 0);
        std::vector<int4> ai(sl ? nb : 0);
        if (sl) {
            cudaMemcpyAsync(fa.data(), w->ws.b_facc.p, 16 * nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(ta.data(), w->ws.b_tacc.p, 16 * nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(ai.data(), w->ws.b_adis_i.p, 16 * nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(af.data(), w->ws.b_adis_f.p, 16 * nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(buf.data(), w->ws.b_adis_buf.p, buf.size() * 16, cudaMemcpyDeviceToHost, s);
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { set_error("download bodies", e); return; }
        for (int i = 0; i < nb; i++) {
            dxBody *b = w->bodies[i];
            b->pos[0] = pos[i].x; b->pos[1] = pos[i].y; b->pos[2] = pos[i].z;
            b->q[0] = q[i].x; b->q[1] = q[i].y; b->q[2] = q[i].z; b->q[3] = q[i].w;
            for (int r = 0; r < 3; r++) {
                b->R[4 * r] = R[3 * i + r].x; b->R[4 * r + 1] = R[3 * i + r].y; b->R[4 * r + 2] = R[3 * i + r].z; b->R[4 * r + 3] = 0;
            }
            b->lvel[0] = lv[i].x; b->lvel[1] = lv[i].y; b->lvel[2] = lv[i].z;
            b->avel[0] = av[i].x; b->avel[1] = av[i].y; b->avel[2] = av[i].z;
            if (sl) {
                b->facc[0] = fa[i].x; b->facc[1] = fa[i].y; b->facc[2] = fa[i].z;
                b->tacc[0] = ta[i].x; b->tacc[1] = ta[i].y; b->tacc[2] = ta[i].z;
                b->adis_flags = ai[i].x & (GB_ADIS_ON | GB_ADIS_DISABLED | GB_ADIS_READY);
                b->adis_counter = (ai[i].x >> 8) & 0xffff;
                b->adis_steps_left = ai[i].z;
                b->adis_time_left = af[i].w;
                for (int k = 0; k < b->adis_samples && k < S; k++) {
                    const float4 l = buf[((size_t)i * S + k) * 2], a = buf[((size_t)i * S + k) * 2 + 1];
                    float *o = &b->adis_buf[8 * k];
                    o[0] = l.x; o[1] = l.y; o[2] = l.z; o[4] = a.x; o[5] = a.y; o[6] = a.z;
                }
            } else {
                // the device consumed the force accumulators
                b->facc[0] = b->facc[1] = b->facc[2] = 0;
                b->tacc[0] = b->tacc[1] = b->tacc[2] = 0;
            }
        }
    }
    w->host_valid = true;
}

static void mark_host_changed(dxBody *b) {
    dxWorld *w = b->world;
    world_download(w);  // keep the other bodies' device state
    w->dev_dirty = true;
}

static bool world_upload(dxWorld *w) {
    if (!world_init_device(w)) return false;
    int nb = (int)w->bodies.size();
    if (!ensure_bodies(w->ws, nb)) { set_error("device allocation (bodies)"); return false; }
    if (!w->dev_dirty) return true;
    std::vector<float4> pos(nb), q(nb), R(3 * nb), lv(nb), av(nb), fa(nb), ta(nb), Ib(3 * nb), iIb(3 * nb), dm(nb);
    std::vector<float> mw(nb);
    for (int i = 0; i < nb; i++) {
        dxBody *b = w->bodies[i];
        b->index = i;
        pos[i] = make_float4(b->pos[0], b->pos[1], b->pos[2], b->invMass);
        q[i] = make_float4(b->q[0], b->q[1], b->q[2], b->q[3]);
        for (int r = 0; r < 3; r++) {
            R[3 * i + r] = make_float4(b->R[4 * r], b->R[4 * r + 1], b->R[4 * r + 2], 0.f);
            Ib[3 * i + r] = make_float4(b->mass.I[4 * r], b->mass.I[4 * r + 1], b->mass.I[4 * r + 2], 0.f);
            iIb[3 * i + r] = make_float4(b->invI[4 * r], b->invI[4 * r + 1], b->invI[4 * r + 2], 0.f);
        }
        lv[i] = make_float4(b->lvel[0], b->lvel[1], b->lvel[2], b->mass.mass);
        int flags = b->gyro ? 1 : 0;
        float ff;
        memcpy(&ff, &flags, 4);
        av[i] = make_float4(b->avel[0], b->avel[1], b->avel[2], ff);
        fa[i] = make_float4(b->facc[0], b->facc[1], b->facc[2], 0.f);
        ta[i] = make_float4(b->tacc[0], b->tacc[1], b->tacc[2], 0.f);
        dm[i] = make_float4(b->damp[0], b->damp[1], b->damp[2], b->damp[3]);
        mw[i] = b->max_w;
    }
    // auto-disable state: uploaded while some body has it on or is disabled
    bool sleep_on = false;
    int S = 1;
    for (int i = 0; i < nb; i++) {
        const dxBody *b = w->bodies[i];
        if (b->adis_flags & (GB_ADIS_ON | GB_ADIS_DISABLED)) sleep_on = true;
        if (b->adis_samples > S) S = b->adis_samples;
    }
    w->ws.sleep_on = sleep_on;
    std::vector<int4> ai;
    std::vector<float4> af, abuf;
    if (sleep_on) {
        if (!ensure_sleep(w->ws, nb, S)) { set_error("device allocation (auto-disable)"); return false; }
        w->ws.adis_S = S;
        ai.resize(nb);
        af.resize(nb);
        abuf.assign((size_t)nb * S * 2, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int i = 0; i < nb; i++) {
            const dxBody *b = w->bodies[i];
            ai[i] = make_int4((b->adis_flags & 0xff) | (b->adis_counter << 8), b->adis_idle_steps, b->adis_steps_left,
                              b->adis_samples);
            af[i] = make_float4(b->adis_lin, b->adis_ang, b->adis_idle_time, b->adis_time_left);
            for (int k = 0; k < b->adis_samples; k++) {
                const float *o = &b->adis_buf[8 * k];
                abuf[((size_t)i * S + k) * 2] = make_float4(o[0], o[1], o[2], 0.f);
                abuf[((size_t)i * S + k) * 2 + 1] = make_float4(o[4], o[5], o[6], 0.f);
            }
        }
    }
    if (nb > 0) {
        cudaStream_t s = w->stream;
        cudaMemcpyAsync(w->ws.b_pos.p, pos.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_q.p, q.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_R.p, R.data(), 48 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_lvel.p, lv.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_avel.p, av.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_facc.p, fa.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_tacc.p, ta.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_Ib.p, Ib.data(), 48 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_invIb.p, iIb.data(), 48 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_damp.p, dm.data(), 16 * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(w->ws.b_maxw.p, mw.data(), 4 * nb, cudaMemcpyHostToDevice, s);
        if (sleep_on) {
            cudaMemcpyAsync(w->ws.b_adis_i.p, ai.data(), 16 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_adis_f.p, af.data(), 16 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_adis_buf.p, abuf.data(), abuf.size() * 16, cudaMemcpyHostToDevice, s);
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { set_error("upload bodies", e); return false; }
    }
    w->dev_dirty = false;
    w->host_valid = true;
    return true;
}

static dxWorld *space_world(dxSpace *sp) {
    for (dxGeom *g : sp->geoms)
        if (g->body) return g->body->world;
    if (!g_default_world) g_default_world = dWorldCreate();
    return g_default_world;
}

static bool space_upload(dxSpace *sp, dxWorld *w) {
    if (!world_upload(w)) return false;
    if (w->uploaded_space == sp && !sp->dirty) return true;
    std::vector<GeomHost> gh(sp->geoms.size());
    for (size_t i = 0; i < sp->geoms.size(); i++) {
        dxGeom *g = sp->geoms[i];
        g->index = (int)i;
        gh[i].cls = g->cls;
        gh[i].body = g->body ? g->body->index : -1;
        memcpy(gh[i].dims, g->dims, sizeof g->dims);
        memcpy(gh[i].pos, g->pos, sizeof g->pos);
        memcpy(gh[i].R, g->R, sizeof g->R);
    }
    if (!upload_geoms(w->ws, gh, w->stream)) { set_error("upload geoms"); return false; }
    w->uploaded_space = sp;
    sp->dirty = false;
    return true;
}

// ------------------------------------------------------------------ init / misc
extern "C" {
static void drop_graph(dxWorld *w);

int dInitODE2(unsigned int) { return 1; }
void dInitODE(void) {}
int dAllocateODEDataForThread(unsigned int) { return 1; }
void dCloseODE(void) {}

const char *gbodeGetLastError(void) { return g_err.c_str(); }
long long gbodeKernelLaunchCount(void) { return g_launches.load(); }

int gbodeTestInject(int kind, int value, int count) {
    switch (kind) {
    case GBODE_TEST_OFF: g_test = TestFaults(); return 1;
    case GBODE_TEST_BARRIER: g_test.barrier = value != 0; return 1;
    case GBODE_TEST_STAGE: g_test.stage = value != 0; return 1;
    case GBODE_TEST_ALLOC:
        g_test.alloc_skip = count > 0 && value >= 0 ? value : -1;
        g_test.alloc_fail = count > 0 ? count : 0;
        return 1;
    case GBODE_TEST_CONTACT_CAP: g_test.contact_cap = value > 0 ? value : 0; return 1;
    case GBODE_TEST_ROW_CAP: g_test.row_cap = value > 0 ? value : 0; return 1;
    case GBODE_TEST_COLOUR_CAP: g_test.colour_cap = value > 0 ? value : 0; return 1;
    case GBODE_TEST_ALLOC_PENDING: return g_test.alloc_skip >= 0 ? 1 : 0;
    default: set_error("gbodeTestInject: unknown kind"); return 0;
    }
}

// misc.cpp:35-135 dRand / dRandInt
static uint32_t g_seed = 0;
unsigned long dRand(void) {
    g_seed = (uint32_t)(1664525u * g_seed + 1013904223u);
    return g_seed;
}
unsigned long dRandGetSeed(void) { return g_seed; }
void dRandSetSeed(unsigned long s) { g_seed = (uint32_t)s; }
int dTestRand(void) {
    uint32_t old = g_seed;
    int ok = 1;
    g_seed = 0;
    if (dRand() != 0x3c6ef35f || dRand() != 0x47502932 || dRand() != 0xd1ccf6e9 || dRand() != 0xaaf95334 ||
        dRand() != 0x6252e503)
        ok = 0;
    g_seed = old;
    return ok;
}
int dRandInt(int n) {
    uint32_t r = (uint32_t)dRand(), un = (uint32_t)n;
    if (un <= 0x10u) {
        r ^= (r >> 16); r ^= (r >> 8); r ^= (r >> 4);
        if (un <= 0x2u) { r ^= (r >> 2); r ^= (r >> 1); return (int)(r & (un >> 1)); }
        if (un <= 0x4u) { r ^= (r >> 2); return (int)(((r & 0x3u) * un) >> 2); }
        return (int)(((r & 0xFu) * un) >> 4);
    }
    if (un <= 0x100u) { r ^= (r >> 16); r ^= (r >> 8); return (int)(((r & 0xFFu) * un) >> 8); }
    if (un <= 0x10000u) { r ^= (r >> 16); return (int)(((r & 0xFFFFu) * un) >> 16); }
    return (int)(((uint64_t)r * un) >> 32);
}
void dRSetIdentity(dMatrix3 R) {
    memset(R, 0, sizeof(dMatrix3));
    R[0] = R[5] = R[10] = 1;
}
void dRfromQ(dMatrix3 R, const dQuaternion q) { r_from_q(R, q); }
// rotation.cpp:160-175 dQFromAxisAndAngle
void dQFromAxisAndAngle(dQuaternion q, dReal ax, dReal ay, dReal az, dReal angle) {
    float l = ax * ax + ay * ay + az * az;
    if (l > 0) {
        angle *= 0.5f;
        q[0] = cosf(angle);
        l = sinf(angle) * (1.0f / sqrtf(l));
        q[1] = ax * l; q[2] = ay * l; q[3] = az * l;
    } else {
        q[0] = 1; q[1] = q[2] = q[3] = 0;
    }
}
void dRFromAxisAndAngle(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal angle) {
    dQuaternion q;
    dQFromAxisAndAngle(q, ax, ay, az, angle);
    r_from_q(R, q);
}

// ------------------------------------------------------------------ mass
void dMassSetZero(dMass *m) { memset(m, 0, sizeof(dMass)); }
void dMassSetParameters(dMass *m, dReal themass, dReal cgx, dReal cgy, dReal cgz, dReal I11, dReal I22, dReal I33,
                        dReal I12, dReal I13, dReal I23) {
    dMassSetZero(m);
    m->mass = themass;
    m->c[0] = cgx; m->c[1] = cgy; m->c[2] = cgz;
    m->I[0] = I11; m->I[5] = I22; m->I[10] = I33;
    m->I[1] = I12; m->I[2] = I13; m->I[6] = I23;
    m->I[4] = I12; m->I[8] = I13; m->I[9] = I23;
}
// mass.cpp:118-210
void dMassSetSphereTotal(dMass *m, dReal total_mass, dReal radius) {
    dMassSetZero(m);
    m->mass = total_mass;
    float II = 0.4f * total_mass * radius * radius;
    m->I[0] = II; m->I[5] = II; m->I[10] = II;
}
void dMassSetSphere(dMass *m, dReal density, dReal radius) {
    dMassSetSphereTotal(m, (dReal)((4.0f / 3.0f) * M_PI * radius * radius * radius * density), radius);
}
void dMassSetCapsule(dMass *m, dReal density, int direction, dReal radius, dReal length) {
    dMassSetZero(m);
    float M1 = (float)(M_PI * radius * radius * length * density);
    float M2 = (float)((4.0f / 3.0f) * M_PI * radius * radius * radius * density);
    m->mass = M1 + M2;
    float Ia = M1 * (0.25f * radius * radius + (1.0f / 12.0f) * length * length) +
               M2 * (0.4f * radius * radius + 0.375f * radius * length + 0.25f * length * length);
    float Ib = (M1 * 0.5f + M2 * 0.4f) * radius * radius;
    m->I[0] = Ia; m->I[5] = Ia; m->I[10] = Ia;
    int d = direction - 1;
    if (d >= 0 && d < 3) m->I[5 * d] = Ib;
}
void dMassSetBoxTotal(dMass *m, dReal total_mass, dReal lx, dReal ly, dReal lz) {
    dMassSetZero(m);
    m->mass = total_mass;
    m->I[0] = total_mass / 12.0f * (ly * ly + lz * lz);
    m->I[5] = total_mass / 12.0f * (lx * lx + lz * lz);
    m->I[10] = total_mass / 12.0f * (lx * lx + ly * ly);
}
void dMassSetBox(dMass *m, dReal density, dReal lx, dReal ly, dReal lz) {
    dMassSetBoxTotal(m, lx * ly * lz * density, lx, ly, lz);
}

// ------------------------------------------------------------------ world
dWorldID dWorldCreate(void) {
    dxWorld *w = new dxWorld();
    SolverParams &P = w->P;
    memset(&P, 0, sizeof P);
    P.erp = 0.2f;     // objects.cpp:37
    P.cfm = 1e-5f;    // objects.cpp:40 (single precision)
    P.w = 1.3f;       // objects.cpp:83
    P.iterations = 20;  // objects.h:451
    P.max_vel = INFINITY;
    P.min_depth = 0;
    P.premature_delta = 1e-8f;  // objects.h:473-475
    P.extra_factor = 1.0f;
    P.extra_delta = 1e-2f;
    P.residual_target = 0;
    P.check_every = 10;
    P.max_iterations = 0;
    P.warm_scale = 1.0f;
    P.solver = GBODE_SOLVER_COLOURED;
    g_worlds.push_back(w);
    return w;
}
void dWorldDestroy(dWorldID w) {
    if (!w) return;
    for (dxBody *b : w->bodies) delete b;
    for (dxJoint *j : w->joints) {
        if (j->group) {
            auto &v = j->group->joints;
            for (size_t k = 0; k < v.size(); k++) if (v[k] == j) { v.erase(v.begin() + k); break; }
        }
        delete j;
    }
    if (w->stream) cudaStreamSynchronize(w->stream);
    drop_graph(w);
    if (w->snapshot) { w->snapshot->release(); delete w->snapshot; }
    for (int i = 0; i < 4; i++) if (w->ev[i]) cudaEventDestroy(w->ev[i]);
    if (w->stage_up_done) { cudaEventSynchronize(w->stage_up_done); cudaEventDestroy(w->stage_up_done); }
    if (w->stage_up) cudaFreeHost(w->stage_up);
    if (w->stage_down) cudaFreeHost(w->stage_down);
    w->ws.release();
    if (w->own_stream && w->stream) cudaStreamDestroy(w->stream);
    for (size_t k = 0; k < g_worlds.size(); k++) if (g_worlds[k] == w) { g_worlds.erase(g_worlds.begin() + k); break; }
    if (g_default_world == w) g_default_world = nullptr;
    delete w;
}
void dWorldSetGravity(dWorldID w, dReal x, dReal y, dReal z) { w->P.gravity[0] = x; w->P.gravity[1] = y; w->P.gravity[2] = z; }
void dWorldGetGravity(dWorldID w, dVector3 g) { g[0] = w->P.gravity[0]; g[1] = w->P.gravity[1]; g[2] = w->P.gravity[2]; }
void dWorldSetERP(dWorldID w, dReal erp) { w->P.erp = erp; }
dReal dWorldGetERP(dWorldID w) { return w->P.erp; }
void dWorldSetCFM(dWorldID w, dReal cfm) { w->P.cfm = cfm; }
dReal dWorldGetCFM(dWorldID w) { return w->P.cfm; }
void dWorldSetQuickStepNumIterations(dWorldID w, int num) { w->P.iterations = num > 0 ? num : 1; }
int dWorldGetQuickStepNumIterations(dWorldID w) { return w->P.iterations; }
void dWorldSetQuickStepW(dWorldID w, dReal over_relaxation) { w->P.w = over_relaxation; }
dReal dWorldGetQuickStepW(dWorldID w) { return w->P.w; }
void dWorldSetQuickStepDynamicIterationParameters(dWorldID w, const dReal *pe, const dReal *mf, const dReal *ed) {
    if (pe) w->P.premature_delta = *pe > 0 ? *pe : 0;
    if (ed) w->P.extra_delta = *ed > 0 ? *ed : 0;
    if (mf) w->P.extra_factor = *mf > 0 ? *mf : 0;
}
void dWorldGetQuickStepDynamicIterationParameters(dWorldID w, dReal *pe, dReal *mf, dReal *ed) {
    if (pe) *pe = w->P.premature_delta;
    if (mf) *mf = w->P.extra_factor;
    if (ed) *ed = w->P.extra_delta;
}
void dWorldSetContactMaxCorrectingVel(dWorldID w, dReal vel) { w->P.max_vel = vel; }
dReal dWorldGetContactMaxCorrectingVel(dWorldID w) { return w->P.max_vel; }
void dWorldSetContactSurfaceLayer(dWorldID w, dReal depth) { w->P.min_depth = depth; }
dReal dWorldGetContactSurfaceLayer(dWorldID w) { return w->P.min_depth; }

void gbodeWorldSetSolver(dWorldID w, int solver) { w->P.solver = solver; }
int gbodeWorldGetSolver(dWorldID w) { return w->P.solver; }
void gbodeWorldSetResidualTarget(dWorldID w, dReal target, int check_every, int max_iterations) {
    w->P.residual_target = target > 0 ? target : 0;
    w->P.check_every = check_every > 0 ? check_every : 10;
    w->P.max_iterations = max_iterations;
}
void gbodeWorldSetResidualChecks(dWorldID w, int mode, int reform_every) {
    w->P.fixed_checks = mode == GBODE_CHECKS_FIXED ? 1 : 0;
    w->P.reform_every = reform_every > 0 ? reform_every : 0;
}
void gbodeWorldSetWarmStart(dWorldID w, int mode, dReal scale) { w->P.warm_mode = mode; w->P.warm_scale = scale; }
void gbodeWorldSetSolverBlocks(dWorldID w, int blocks) { w->P.pgs_blocks = blocks > 0 ? blocks : 0; }
void gbodeWorldSetManifoldPasses(dWorldID w, int passes) { w->P.pgs_passes = passes > 1 ? (passes > 16 ? 16 : passes) : 1; }
int gbodeWorldGetManifoldPasses(dWorldID w) { return w->P.pgs_passes > 1 ? w->P.pgs_passes : 1; }
void gbodeWorldSetSolverTiles(dWorldID w, int threads, int chunk_rows) {
    w->P.pgs_threads = threads == 128 ? 128 : 0;
    w->P.pgs_chunk = chunk_rows > 0 ? chunk_rows : 0;
}
void gbodeWorldGetSolverTiles(dWorldID w, int *threads, int *chunk_rows) {
    if (threads) *threads = w->P.pgs_threads == 128 ? 128 : 256;
    if (chunk_rows) *chunk_rows = w->P.pgs_chunk > 0 ? w->P.pgs_chunk : 800;
}
void gbodeWorldSetTwoLevelSweep(dWorldID w, int interior_phases) {
    w->P.pgs_two_level = interior_phases < 0 ? 0 : (interior_phases > 8 ? 8 : interior_phases);
}
int gbodeWorldGetTwoLevelSweep(dWorldID w) { return w->P.pgs_two_level; }
void gbodeWorldSetSweepSync(dWorldID w, int mode) { w->P.pgs_grid_sync = mode == GBODE_SYNC_GRID ? 1 : 0; }
int gbodeWorldGetSweepSync(dWorldID w) { return w->P.pgs_grid_sync ? GBODE_SYNC_GRID : GBODE_SYNC_NEIGHBOURS; }
void gbodeWorldSetCrossClasses(dWorldID w, int classes) {
    w->P.pgs_split = classes < 2 ? 0 : (classes > GBODE_MAX_CROSS_CLASSES ? GBODE_MAX_CROSS_CLASSES : classes);
}
int gbodeWorldGetCrossClasses(dWorldID w) { return w->P.pgs_split; }
void gbodeWorldSetSweepMomentum(dWorldID w, dReal beta) {
    w->P.momentum = beta > 0.f ? (beta < 0.95f ? beta : 0.95f) : 0.f;
}
dReal gbodeWorldGetSweepMomentum(dWorldID w) { return w->P.momentum; }
int gbodeWorldGetSolverBlocks(dWorldID w) { return w->P.pgs_blocks > 0 && w->P.pgs_blocks < num_sms() ? w->P.pgs_blocks : num_sms(); }

int gbodeWorldSetLearnedWarmStart(dWorldID w, const float *params, int enabled) {
    if (!enabled) { w->P.learned = 0; return 1; }
    if (!params) { set_error("gbodeWorldSetLearnedWarmStart: no parameters"); return 0; }
    Workspace &ws = w->ws;
    if (!world_upload(w)) return 0;
    if (!(ws.mlp_P.ensure(GB_MLP_NPARAMS * 4) && ws.mlp_wb.ensure(mlp_wb_bytes()))) {
        set_error("gbodeWorldSetLearnedWarmStart: device allocation");
        return 0;
    }
    cudaMemcpyAsync(ws.mlp_P.p, params, GB_MLP_NPARAMS * 4, cudaMemcpyHostToDevice, w->stream);
    if (!mlp_pack(ws.mlp_P.as<float>(), ws.mlp_wb.as<unsigned char>(), w->stream) ||
        cudaStreamSynchronize(w->stream) != cudaSuccess) {
        set_error("gbodeWorldSetLearnedWarmStart: packing failed");
        return 0;
    }
    w->P.learned = 1;
    return 1;
}
void gbodeWorldSetLearnCapture(dWorldID w, int enabled) { w->P.learn_capture = enabled != 0; }
int gbodeWorldGetLearnSamples(dWorldID w, float *out, int cap) {
    int n = learn_samples(w->ws, out, cap, w->stream);
    if (n < 0) { set_error("gbodeWorldGetLearnSamples", cudaGetLastError()); return 0; }
    return n;
}
void gbodeWorldGetLearnedStats(dWorldID w, float *out3) {
    float v[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(v, w->ws.dc->learn_stats, sizeof v, cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    out3[0] = v[0]; out3[1] = v[1]; out3[2] = v[2];
}
void gbodeWorldSetStream(dWorldID w, void *stream) {
    if (w->own_stream && w->stream) { cudaStreamSynchronize(w->stream); cudaStreamDestroy(w->stream); }
    w->stream = (cudaStream_t)stream;
    w->own_stream = false;
    if (!w->stream) {
        cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
        w->own_stream = true;
    }
}
void *gbodeWorldGetStream(dWorldID w) {
    world_init_device(w);
    return (void *)w->stream;
}
int gbodeWorldSynchronize(dWorldID w) {
    if (!world_init_device(w)) return 0;
    cudaError_t e = cudaStreamSynchronize(w->stream);
    if (e != cudaSuccess) { set_error("stream", e); return 0; }
    unsigned err = 0;
    cudaMemcpy(&err, &w->ws.dc->err, 4, cudaMemcpyDeviceToHost);
    if (err) {
        char buf[96];
        snprintf(buf, sizeof buf, "device error bits 0x%x", err);
        set_error(buf);
        cudaMemset(&w->ws.dc->err, 0, 4);
        return 0;
    }
    return 1;
}
void gbodeWorldSetTiming(dWorldID w, int enabled) { w->timing = enabled != 0; }

// ------------------------------------------------------------------ bodies
dBodyID dBodyCreate(dWorldID w) {
    world_download(w);
    dxBody *b = new dxBody();
    b->world = w;
    b->index = (int)w->bodies.size();
    dMassSetParameters(&b->mass, 1, 0, 0, 0, 1, 1, 1, 0, 0, 0);  // ode.cpp:249-254
    memset(b->invI, 0, sizeof b->invI);
    b->invI[0] = b->invI[5] = b->invI[10] = 1;
    memcpy(b->damp, w->damp, sizeof b->damp);  // dBodySetDampingDefaults
    b->max_w = w->max_w;
    w->bodies.push_back(b);
    dBodySetAutoDisableDefaults(b);  // ode.cpp:268-274
    b->adis_steps_left = b->adis_idle_steps;
    b->adis_time_left = b->adis_idle_time;
    b->adis_counter = 0;
    b->adis_flags &= ~GB_ADIS_READY;
    dBodySetAutoDisableAverageSamplesCount(b, b->adis_samples);
    w->dev_dirty = true;
    return b;
}
// ---- auto-disable: ode.cpp:850-870 (enable), :887-1020 (bodies), :1880-1965 (world)
void dBodyEnable(dBodyID b) {
    mark_host_changed(b);
    b->adis_flags &= ~GB_ADIS_DISABLED;
    b->adis_steps_left = b->adis_idle_steps;
    b->adis_time_left = b->adis_idle_time;
}
void dBodyDisable(dBodyID b) { mark_host_changed(b); b->adis_flags |= GB_ADIS_DISABLED; }
int dBodyIsEnabled(dBodyID b) { world_download(b->world); return (b->adis_flags & GB_ADIS_DISABLED) == 0; }
dReal dBodyGetAutoDisableLinearThreshold(dBodyID b) { return sqrtf(b->adis_lin); }
void dBodySetAutoDisableLinearThreshold(dBodyID b, dReal t) { mark_host_changed(b); b->adis_lin = t * t; }
dReal dBodyGetAutoDisableAngularThreshold(dBodyID b) { return sqrtf(b->adis_ang); }
void dBodySetAutoDisableAngularThreshold(dBodyID b, dReal t) { mark_host_changed(b); b->adis_ang = t * t; }
int dBodyGetAutoDisableAverageSamplesCount(dBodyID b) { return b->adis_samples; }
void dBodySetAutoDisableAverageSamplesCount(dBodyID b, unsigned int n) {
    mark_host_changed(b);
    if (n > 0xffff) n = 0xffff;  // the device keeps the ring position in 16 bits
    b->adis_samples = (int)n;
    b->adis_buf.assign((size_t)n * 8, 0.f);  // the new buffer is empty
    b->adis_counter = 0;
    b->adis_flags &= ~GB_ADIS_READY;
}
int dBodyGetAutoDisableSteps(dBodyID b) { return b->adis_idle_steps; }
void dBodySetAutoDisableSteps(dBodyID b, int steps) { mark_host_changed(b); b->adis_idle_steps = steps; }
dReal dBodyGetAutoDisableTime(dBodyID b) { return b->adis_idle_time; }
void dBodySetAutoDisableTime(dBodyID b, dReal t) { mark_host_changed(b); b->adis_idle_time = t; }
int dBodyGetAutoDisableFlag(dBodyID b) { return (b->adis_flags & GB_ADIS_ON) != 0; }
void dBodySetAutoDisableFlag(dBodyID b, int do_auto_disable) {
    mark_host_changed(b);
    if (!do_auto_disable) {
        dxWorld *w = b->world;
        b->adis_flags &= ~(GB_ADIS_ON | GB_ADIS_DISABLED);
        b->adis_idle_steps = w->adis_idle_steps;
        b->adis_idle_time = w->adis_idle_time;
        dBodySetAutoDisableAverageSamplesCount(b, (unsigned)w->adis_samples);
    } else {
        b->adis_flags |= GB_ADIS_ON;
    }
}
void dBodySetAutoDisableDefaults(dBodyID b) {
    dxWorld *w = b->world;
    mark_host_changed(b);
    b->adis_idle_steps = w->adis_idle_steps;
    b->adis_idle_time = w->adis_idle_time;
    b->adis_samples = w->adis_samples;
    b->adis_lin = w->adis_lin;
    b->adis_ang = w->adis_ang;
    dBodySetAutoDisableFlag(b, w->adis_on);
}
dReal dWorldGetAutoDisableLinearThreshold(dWorldID w) { return sqrtf(w->adis_lin); }
void dWorldSetAutoDisableLinearThreshold(dWorldID w, dReal t) { w->adis_lin = t * t; }
dReal dWorldGetAutoDisableAngularThreshold(dWorldID w) { return sqrtf(w->adis_ang); }
void dWorldSetAutoDisableAngularThreshold(dWorldID w, dReal t) { w->adis_ang = t * t; }
int dWorldGetAutoDisableAverageSamplesCount(dWorldID w) { return w->adis_samples; }
void dWorldSetAutoDisableAverageSamplesCount(dWorldID w, unsigned int n) { w->adis_samples = n > 0xffff ? 0xffff : (int)n; }
int dWorldGetAutoDisableSteps(dWorldID w) { return w->adis_idle_steps; }
void dWorldSetAutoDisableSteps(dWorldID w, int steps) { w->adis_idle_steps = steps; }
dReal dWorldGetAutoDisableTime(dWorldID w) { return w->adis_idle_time; }
void dWorldSetAutoDisableTime(dWorldID w, dReal t) { w->adis_idle_time = t; }
// the reference returns its flag bit (dxBodyAutoDisable, 16), not 1
int dWorldGetAutoDisableFlag(dWorldID w) { return w->adis_on ? 16 : 0; }
void dWorldSetAutoDisableFlag(dWorldID w, int do_auto_disable) { w->adis_on = do_auto_disable != 0; }
// ---- damping and angular speed cap: ode.cpp:1025-1113 (bodies), :1970-2048 (world)
void dWorldSetLinearDamping(dWorldID w, dReal scale) { w->damp[0] = scale; }
void dWorldSetAngularDamping(dWorldID w, dReal scale) { w->damp[1] = scale; }
void dWorldSetDamping(dWorldID w, dReal linear_scale, dReal angular_scale) {
    w->damp[0] = linear_scale;
    w->damp[1] = angular_scale;
}
void dWorldSetLinearDampingThreshold(dWorldID w, dReal threshold) { w->damp[2] = threshold * threshold; }
void dWorldSetAngularDampingThreshold(dWorldID w, dReal threshold) { w->damp[3] = threshold * threshold; }
dReal dWorldGetLinearDamping(dWorldID w) { return w->damp[0]; }
dReal dWorldGetAngularDamping(dWorldID w) { return w->damp[1]; }
dReal dWorldGetLinearDampingThreshold(dWorldID w) { return sqrtf(w->damp[2]); }
dReal dWorldGetAngularDampingThreshold(dWorldID w) { return sqrtf(w->damp[3]); }
void dWorldSetMaxAngularSpeed(dWorldID w, dReal max_speed) { w->max_w = max_speed; }
dReal dWorldGetMaxAngularSpeed(dWorldID w) { return w->max_w; }
void dBodySetLinearDamping(dBodyID b, dReal scale) { mark_host_changed(b); b->damp[0] = scale; }
void dBodySetAngularDamping(dBodyID b, dReal scale) { mark_host_changed(b); b->damp[1] = scale; }
void dBodySetDamping(dBodyID b, dReal linear_scale, dReal angular_scale) {
    mark_host_changed(b);
    b->damp[0] = linear_scale;
    b->damp[1] = angular_scale;
}
void dBodySetLinearDampingThreshold(dBodyID b, dReal threshold) { mark_host_changed(b); b->damp[2] = threshold * threshold; }
void dBodySetAngularDampingThreshold(dBodyID b, dReal threshold) { mark_host_changed(b); b->damp[3] = threshold * threshold; }
void dBodySetDampingDefaults(dBodyID b) { mark_host_changed(b); memcpy(b->damp, b->world->damp, sizeof b->damp); }
dReal dBodyGetLinearDamping(dBodyID b) { return b->damp[0]; }
dReal dBodyGetAngularDamping(dBodyID b) { return b->damp[1]; }
dReal dBodyGetLinearDampingThreshold(dBodyID b) { return sqrtf(b->damp[2]); }
dReal dBodyGetAngularDampingThreshold(dBodyID b) { return sqrtf(b->damp[3]); }
void dBodySetMaxAngularSpeed(dBodyID b, dReal max_speed) { mark_host_changed(b); b->max_w = max_speed; }
dReal dBodyGetMaxAngularSpeed(dBodyID b) { return b->max_w; }
void dBodyDestroy(dBodyID b) {
    dxWorld *w = b->world;
    world_download(w);
    for (dxJoint *j : w->joints) {
        if (j->b1 == b) j->b1 = nullptr;
        if (j->b2 == b) j->b2 = nullptr;
    }
    w->joints_dirty = true;
    for (dxWorld *ww : g_worlds) (void)ww;
    auto &v = w->bodies;
    for (size_t k = 0; k < v.size(); k++) if (v[k] == b) { v.erase(v.begin() + k); break; }
    for (size_t k = 0; k < v.size(); k++) v[k]->index = (int)k;
    w->dev_dirty = true;
    w->uploaded_space = nullptr;  // geoms refer to body indices
    delete b;
}
void dBodySetData(dBodyID b, void *data) { b->data = data; }
void *dBodyGetData(dBodyID b) { return b->data; }
void dBodySetPosition(dBodyID b, dReal x, dReal y, dReal z) {
    mark_host_changed(b);
    b->pos[0] = x; b->pos[1] = y; b->pos[2] = z;
}
void dBodySetRotation(dBodyID b, const dMatrix3 R) {
    mark_host_changed(b);
    memcpy(b->R, R, sizeof(dMatrix3));
    q_from_r(b->q, R);
    normalize4(b->q);
}
void dBodySetQuaternion(dBodyID b, const dQuaternion q) {
    mark_host_changed(b);
    for (int i = 0; i < 4; i++) b->q[i] = q[i];
    normalize4(b->q);
    r_from_q(b->R, b->q);
}
void dBodySetLinearVel(dBodyID b, dReal x, dReal y, dReal z) {
    mark_host_changed(b);
    b->lvel[0] = x; b->lvel[1] = y; b->lvel[2] = z;
}
void dBodySetAngularVel(dBodyID b, dReal x, dReal y, dReal z) {
    mark_host_changed(b);
    b->avel[0] = x; b->avel[1] = y; b->avel[2] = z;
}
const dReal *dBodyGetPosition(dBodyID b) { world_download(b->world); return b->pos; }
const dReal *dBodyGetRotation(dBodyID b) { world_download(b->world); return b->R; }
const dReal *dBodyGetQuaternion(dBodyID b) { world_download(b->world); return b->q; }
const dReal *dBodyGetLinearVel(dBodyID b) { world_download(b->world); return b->lvel; }
const dReal *dBodyGetAngularVel(dBodyID b) { world_download(b->world); return b->avel; }
void dBodySetMass(dBodyID b, const dMass *mass) {
    mark_host_changed(b);
    b->mass = *mass;
    if (!invert_pd3(b->mass.I, b->invI)) {
        memset(b->invI, 0, sizeof b->invI);
        b->invI[0] = b->invI[5] = b->invI[10] = 1;
    }
    b->invMass = 1.0f / b->mass.mass;
}
void dBodyGetMass(dBodyID b, dMass *mass) { *mass = b->mass; }
void dBodyAddForce(dBodyID b, dReal fx, dReal fy, dReal fz) {
    mark_host_changed(b);
    b->facc[0] += fx; b->facc[1] += fy; b->facc[2] += fz;
}
void dBodyAddTorque(dBodyID b, dReal fx, dReal fy, dReal fz) {
    mark_host_changed(b);
    b->tacc[0] += fx; b->tacc[1] += fy; b->tacc[2] += fz;
}
const dReal *dBodyGetForce(dBodyID b) { world_download(b->world); return b->facc; }
const dReal *dBodyGetTorque(dBodyID b) { world_download(b->world); return b->tacc; }
void dBodySetGyroscopicMode(dBodyID b, int enabled) { mark_host_changed(b); b->gyro = enabled != 0; }
int dBodyGetGyroscopicMode(dBodyID b) { return b->gyro; }
int dBodyGetNumJoints(dBodyID b) {
    int n = 0;
    for (dxJoint *j : b->world->joints) if (j->attached && (j->b1 == b || j->b2 == b)) n++;
    return n;
}

int gbodeWorldGetBodyCount(dWorldID w) { return (int)w->bodies.size(); }
// Bulk state.  While the device holds the state (after a step), Get copies
// pos, q, R, lvel and avel straight from the device into the caller's array
// through a pinned staging buffer and leaves the body records alone; Set packs
// the caller's array into pinned staging and copies it to the device
// asynchronously, the body records then read from the device when next
// needed.  Where staging cannot be allocated, both go through the records.
void gbodeWorldGetState(dWorldID w, float *out) {
    const size_t nb = w->bodies.size();
    if (!w->host_valid && nb > 0 && stage_ensure(w->stage_down, w->stage_down_n, nb, nullptr)) {
        float4 *pos = w->stage_down, *q = pos + nb, *R = q + nb, *lv = R + 3 * nb, *av = lv + nb;
        cudaStream_t s = w->stream;
        cudaMemcpyAsync(pos, w->ws.b_pos.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(q, w->ws.b_q.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(R, w->ws.b_R.p, 48 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(lv, w->ws.b_lvel.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(av, w->ws.b_avel.p, 16 * nb, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { set_error("gbodeWorldGetState", e); return; }
        for (size_t i = 0; i < nb; i++) {
            float *o = out + 25 * i;
            o[0] = pos[i].x; o[1] = pos[i].y; o[2] = pos[i].z;
            o[3] = q[i].x; o[4] = q[i].y; o[5] = q[i].z; o[6] = q[i].w;
            for (int r = 0; r < 3; r++) {
                const float4 v = R[3 * i + r];
                o[7 + 4 * r] = v.x; o[8 + 4 * r] = v.y; o[9 + 4 * r] = v.z; o[10 + 4 * r] = 0.f;
            }
            o[19] = lv[i].x; o[20] = lv[i].y; o[21] = lv[i].z;
            o[22] = av[i].x; o[23] = av[i].y; o[24] = av[i].z;
        }
        return;
    }
    world_download(w);
    for (size_t i = 0; i < w->bodies.size(); i++) {
        dxBody *b = w->bodies[i];
        float *o = out + 25 * i;
        memcpy(o, b->pos, 12); memcpy(o + 3, b->q, 16); memcpy(o + 7, b->R, 48);
        memcpy(o + 19, b->lvel, 12); memcpy(o + 22, b->avel, 12);
    }
}
void gbodeWorldSetState(dWorldID w, const float *in) {
    const size_t nb = w->bodies.size();
    // the direct path: every other host change is on the device first
    if (nb > 0 && world_upload(w)) {
        if (!w->stage_up_done && cudaEventCreateWithFlags(&w->stage_up_done, cudaEventDisableTiming) != cudaSuccess)
            w->stage_up_done = nullptr;
        if (w->stage_up_done && stage_ensure(w->stage_up, w->stage_up_n, nb, w->stage_up_done)) {
            cudaEventSynchronize(w->stage_up_done);  // the previous upload has left the staging buffer
            float4 *pos = w->stage_up, *q = pos + nb, *R = q + nb, *lv = R + 3 * nb, *av = lv + nb;
            for (size_t i = 0; i < nb; i++) {
                const dxBody *b = w->bodies[i];
                const float *o = in + 25 * i;
                pos[i] = make_float4(o[0], o[1], o[2], b->invMass);
                q[i] = make_float4(o[3], o[4], o[5], o[6]);
                for (int r = 0; r < 3; r++) R[3 * i + r] = make_float4(o[7 + 4 * r], o[8 + 4 * r], o[9 + 4 * r], 0.f);
                lv[i] = make_float4(o[19], o[20], o[21], b->mass.mass);
                const int flags = b->gyro ? 1 : 0;
                float ff;
                memcpy(&ff, &flags, 4);
                av[i] = make_float4(o[22], o[23], o[24], ff);
            }
            cudaStream_t s = w->stream;
            cudaMemcpyAsync(w->ws.b_pos.p, pos, 16 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_q.p, q, 16 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_R.p, R, 48 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_lvel.p, lv, 16 * nb, cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(w->ws.b_avel.p, av, 16 * nb, cudaMemcpyHostToDevice, s);
            cudaEventRecord(w->stage_up_done, s);
            w->host_valid = false;  // the records read the new state from the device when next needed
            return;
        }
    }
    world_download(w);
    for (size_t i = 0; i < w->bodies.size(); i++) {
        dxBody *b = w->bodies[i];
        const float *o = in + 25 * i;
        memcpy(b->pos, o, 12); memcpy(b->q, o + 3, 16); memcpy(b->R, o + 7, 48);
        memcpy(b->lvel, o + 19, 12); memcpy(b->avel, o + 22, 12);
    }
    w->dev_dirty = true;
}

// ------------------------------------------------------------------ spaces and geoms
dSpaceID dHashSpaceCreate(dSpaceID parent) {
    (void)parent;  // nested spaces are outside the supported subset
    return new dxSpace();
}
void dHashSpaceSetLevels(dSpaceID s, int minlevel, int maxlevel) { s->minlevel = minlevel; s->maxlevel = maxlevel; s->dirty = true; }
void dHashSpaceGetLevels(dSpaceID s, int *minlevel, int *maxlevel) {
    if (minlevel) *minlevel = s->minlevel;
    if (maxlevel) *maxlevel = s->maxlevel;
}
void dSpaceSetCleanup(dSpaceID s, int mode) { s->cleanup = mode; }
void gbodeHashSpaceSetExactPairs(dSpaceID s, int exact) { s->exact_pairs = exact != 0; }
int dSpaceGetNumGeoms(dSpaceID s) { return (int)s->geoms.size(); }
void dSpaceDestroy(dSpaceID s) {
    for (dxGeom *g : s->geoms) {
        g->space = nullptr;
        if (s->cleanup) delete g;
    }
    for (dxWorld *w : g_worlds) if (w->uploaded_space == s) w->uploaded_space = nullptr;
    delete s;
}
static dxGeom *geom_new(dSpaceID space, int cls) {
    dxGeom *g = new dxGeom();
    g->cls = cls;
    g->uid = g_geom_uid++;
    if (space) {
        g->space = space;
        // dSpaceAdd puts new geoms at the head of the space list (collision_space.cpp:160-176)
        space->geoms.insert(space->geoms.begin(), g);
        space->dirty = true;
    }
    return g;
}
dGeomID dCreateSphere(dSpaceID space, dReal radius) {
    dxGeom *g = geom_new(space, dSphereClass);
    g->dims[0] = radius;
    return g;
}
dGeomID dCreateBox(dSpaceID space, dReal lx, dReal ly, dReal lz) {
    dxGeom *g = geom_new(space, dBoxClass);
    g->dims[0] = lx; g->dims[1] = ly; g->dims[2] = lz;
    return g;
}
dGeomID dCreateCapsule(dSpaceID space, dReal radius, dReal length) {
    dxGeom *g = geom_new(space, dCapsuleClass);
    g->dims[0] = radius; g->dims[1] = length;
    return g;
}
// plane.cpp:48-66 normalises the plane equation on creation
dGeomID dCreatePlane(dSpaceID space, dReal a, dReal b, dReal c, dReal d) {
    dxGeom *g = geom_new(space, dPlaneClass);
    float l = a * a + b * b + c * c;
    if (l > 0) {
        l = 1.0f / sqrtf(l);
        g->dims[0] = a * l; g->dims[1] = b * l; g->dims[2] = c * l; g->dims[3] = d * l;
    } else {
        g->dims[0] = 1; g->dims[1] = 0; g->dims[2] = 0; g->dims[3] = 0;
    }
    return g;
}
void dGeomDestroy(dGeomID g) {
    if (g->space) {
        auto &v = g->space->geoms;
        for (size_t k = 0; k < v.size(); k++) if (v[k] == g) { v.erase(v.begin() + k); break; }
        g->space->dirty = true;
    }
    delete g;
}
void dGeomSetData(dGeomID g, void *data) { g->data = data; }
void *dGeomGetData(dGeomID g) { return g->data; }
void dGeomSetBody(dGeomID g, dBodyID b) {
    g->body = b;
    if (g->space) g->space->dirty = true;
}
dBodyID dGeomGetBody(dGeomID g) { return g->body; }
void dGeomSetPosition(dGeomID g, dReal x, dReal y, dReal z) {
    if (g->body) { dBodySetPosition(g->body, x, y, z); return; }
    g->pos[0] = x; g->pos[1] = y; g->pos[2] = z;
    if (g->space) g->space->dirty = true;
}
void dGeomSetRotation(dGeomID g, const dMatrix3 R) {
    if (g->body) { dBodySetRotation(g->body, R); return; }
    memcpy(g->R, R, sizeof(dMatrix3));
    if (g->space) g->space->dirty = true;
}
const dReal *dGeomGetPosition(dGeomID g) { return g->body ? dBodyGetPosition(g->body) : g->pos; }
const dReal *dGeomGetRotation(dGeomID g) { return g->body ? dBodyGetRotation(g->body) : g->R; }
int dGeomGetClass(dGeomID g) { return g->cls; }
void dGeomGetAABB(dGeomID g, dReal aabb[6]) {
    const float *p = dGeomGetPosition(g), *R = dGeomGetRotation(g), *d = g->dims;
    float r[3];
    if (g->cls == dSphereClass) { r[0] = r[1] = r[2] = d[0]; }
    else if (g->cls == dBoxClass) {
        for (int i = 0; i < 3; i++) r[i] = 0.5f * (fabsf(R[4 * i] * d[0]) + fabsf(R[4 * i + 1] * d[1]) + fabsf(R[4 * i + 2] * d[2]));
    } else if (g->cls == dCapsuleClass) {
        for (int i = 0; i < 3; i++) r[i] = fabsf(R[4 * i + 2] * d[1]) * 0.5f + d[0];
    } else {
        // plane.cpp:80-107: unbounded, or the half space below an axis-aligned plane
        for (int i = 0; i < 6; i++) aabb[i] = (i & 1) ? INFINITY : -INFINITY;
        const int ax = (d[1] == 0.0f && d[2] == 0.0f) ? 0 : (d[0] == 0.0f && d[2] == 0.0f) ? 1
                     : (d[0] == 0.0f && d[1] == 0.0f) ? 2 : -1;
        if (ax >= 0) {
            aabb[2 * ax] = d[ax] > 0 ? -INFINITY : -d[3];
            aabb[2 * ax + 1] = d[ax] > 0 ? d[3] : INFINITY;
        }
        return;
    }
    for (int i = 0; i < 3; i++) { aabb[2 * i] = p[i] - r[i]; aabb[2 * i + 1] = p[i] + r[i]; }
}

// ------------------------------------------------------------------ collide
struct CollideBatch {
    dxSpace *space = nullptr;
    dxWorld *world = nullptr;
    std::vector<int> pairs;  // 2 per pair
    std::unordered_map<long long, int> index;  // (a,b) -> pair
    int maxc = -1;
    std::vector<float> out;
    std::vector<int> counts;
};
static thread_local CollideBatch *g_batch = nullptr;

static void fill_contact_geoms(const float *src, int n, dGeomID o1, dGeomID o2, dContactGeom *contact, int skip, bool negate) {
    for (int i = 0; i < n; i++) {
        dContactGeom *c = (dContactGeom *)((char *)contact + (size_t)i * skip);
        const float *o = src + 8 * i;
        c->pos[0] = o[0]; c->pos[1] = o[1]; c->pos[2] = o[2]; c->pos[3] = 0;
        float sg = negate ? -1.f : 1.f;
        c->normal[0] = sg * o[3]; c->normal[1] = sg * o[4]; c->normal[2] = sg * o[5]; c->normal[3] = 0;
        c->depth = o[6];
        c->g1 = o1; c->g2 = o2;
        c->side1 = -1; c->side2 = -1;
    }
}

// A one-off pair outside a dSpaceCollide batch: both geoms are posed on the
// host from their current state and collided on the device.
static int collide_single(dxGeom *o1, dxGeom *o2, int flags, dContactGeom *contact, int skip) {
    if (!g_default_world) g_default_world = dWorldCreate();
    dxWorld *w = g_default_world;
    if (!world_init_device(w)) return 0;
    std::vector<GeomHost> gh(2);
    dxGeom *gg[2] = {o1, o2};
    for (int k = 0; k < 2; k++) {
        gh[k].cls = gg[k]->cls;
        gh[k].body = -1;
        memcpy(gh[k].dims, gg[k]->dims, sizeof gh[k].dims);
        const float *p = dGeomGetPosition(gg[k]), *R = dGeomGetRotation(gg[k]);
        memcpy(gh[k].pos, p, 16);
        memcpy(gh[k].R, R, 48);
    }
    if (!ensure_bodies(w->ws, 1) || !upload_geoms(w->ws, gh, w->stream)) { set_error("dCollide upload"); return 0; }
    w->uploaded_space = nullptr;
    launch_pose_aabb(w->ws, bodies_view(w->ws, 0), 2, -1000, 1000, w->stream);
    int pr[2] = {0, 1};
    std::vector<float> out;
    std::vector<int> counts;
    if (narrow_pairs_host(w->ws, pr, 1, flags & 0xffff, out, counts, w->stream) < 0) { set_error("dCollide"); return 0; }
    int n = counts.empty() ? 0 : counts[0];
    fill_contact_geoms(out.data(), n, o1, o2, contact, skip, false);
    return n;
}

// collision_kernel.cpp:292-338 dCollide
int dCollide(dGeomID o1, dGeomID o2, int flags, dContactGeom *contact, int skip) {
    if ((flags & 0xffff) == 0) return 0;
    if (o1 == o2) return 0;
    if (o1->body == o2->body && o1->body) return 0;
    CollideBatch *B = g_batch;
    if (B && o1->space == B->space && o2->space == B->space) {
        auto it = B->index.find(((long long)o1->index << 32) | (unsigned)o2->index);
        if (it != B->index.end()) {
            int maxc = flags & 0xffff;
            if (maxc > 8) maxc = 8;
            if (B->maxc != maxc) {
                // one device launch serves every pair of this dSpaceCollide
                int np = (int)B->pairs.size() / 2;
                if (narrow_pairs_host(B->world->ws, B->pairs.data(), np, maxc, B->out, B->counts, B->world->stream) < 0) {
                    set_error("dCollide batch");
                    return 0;
                }
                B->maxc = maxc;
            }
            int p = it->second;
            int n = B->counts[p];
            fill_contact_geoms(&B->out[(size_t)p * 64], n, o1, o2, contact, skip, false);
            return n;
        }
    }
    return collide_single(o1, o2, flags, contact, skip);
}

// box.cpp:356-737 dBoxBox as a public function: evaluated on the device.
int dBoxBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2, const dMatrix3 R2,
            const dVector3 side2, dVector3 normal, dReal *depth, int *return_code, int flags, dContactGeom *contact,
            int skip);

void dSpaceCollide(dSpaceID space, void *data, dNearCallback *callback) {
    if (!space || !callback || space->geoms.size() < 2) return;
    dxWorld *w = space_world(space);
    if (!space_upload(space, w)) return;
    int ng = (int)space->geoms.size();
    cudaStream_t s = w->stream;
    launch_pose_aabb(w->ws, bodies_view(w->ws, (int)w->bodies.size()), ng, space->minlevel, space->maxlevel, s);
    if (!launch_broadphase(w->ws, ng, space->exact_pairs, s)) { set_error("broad phase"); return; }
    int np = 0;
    cudaMemcpyAsync(&np, &w->ws.dc->npairs, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { set_error("broad phase", e); return; }
    CollideBatch batch;
    batch.space = space;
    batch.world = w;
    batch.pairs.resize((size_t)np * 2);
    if (np > 0) {
        cudaMemcpyAsync(batch.pairs.data(), w->ws.pairs.p, (size_t)np * 8, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    batch.index.reserve((size_t)np * 2);
    for (int p = 0; p < np; p++) batch.index[((long long)batch.pairs[2 * p] << 32) | (unsigned)batch.pairs[2 * p + 1]] = p;
    w->stats.pairs = np;
    CollideBatch *prev = g_batch;
    g_batch = &batch;
    for (int p = 0; p < np; p++) callback(data, space->geoms[batch.pairs[2 * p]], space->geoms[batch.pairs[2 * p + 1]]);
    g_batch = prev;
}

int gbodeSpaceCollideContacts(dSpaceID space, dWorldID w, dJointGroupID group, const dSurfaceParameters *sp, int maxc) {
    if (!space || !w || !group || !sp || maxc < 1) { set_error("gbodeSpaceCollideContacts: bad argument"); return 0; }
    if (!space_upload(space, w)) return 0;
    int ng = (int)space->geoms.size();
    cudaStream_t s = w->stream;
    Surface surf;
    memset(&surf, 0, sizeof surf);
    surf.mode = sp->mode; surf.mu = sp->mu; surf.mu2 = sp->mu2; surf.rho = sp->rho; surf.rho2 = sp->rho2; surf.rhoN = sp->rhoN;
    surf.bounce = sp->bounce; surf.bounce_vel = sp->bounce_vel; surf.soft_erp = sp->soft_erp; surf.soft_cfm = sp->soft_cfm;
    surf.motion1 = sp->motion1; surf.motion2 = sp->motion2; surf.motionN = sp->motionN; surf.slip1 = sp->slip1; surf.slip2 = sp->slip2;
    if (!w->ws.surfaces.ensure(sizeof(Surface))) { set_error("device allocation (surfaces)"); return 0; }
    launch_set_surface(w->ws, surf, s);  // by value: no host buffer outlives the call
    w->ws.rows_per_contact = (sp->mode & dContactRolling) ? 6 : 3;
    launch_pose_aabb(w->ws, bodies_view(w->ws, (int)w->bodies.size()), ng, space->minlevel, space->maxlevel, s);
    if (!launch_broadphase(w->ws, ng, space->exact_pairs, s)) { set_error("broad phase"); return 0; }
    if (!launch_narrowphase(w->ws, maxc, 0, false, s)) { set_error("narrow phase"); return 0; }
    w->device_contacts = true;
    w->device_surfaces = 1;
    group->device_world = w;
    return 1;
}

// ------------------------------------------------------------------ joints
dJointGroupID dJointGroupCreate(int) { return new dxJointGroup(); }
void dJointGroupEmpty(dJointGroupID g) {
    for (dxJoint *j : g->joints) {
        dxWorld *w = j->world;
        if (j->type != dJointTypeContact) w->joints_dirty = true;
        auto &v = w->joints;
        for (size_t k = v.size(); k-- > 0;) if (v[k] == j) { v.erase(v.begin() + k); break; }
        delete j;
    }
    g->joints.clear();
    if (g->device_world) {
        dxWorld *w = g->device_world;
        w->device_contacts = false;
        cudaMemsetAsync(&w->ws.dc->ncontacts, 0, 4, w->stream);
        g->device_world = nullptr;
    }
}
void dJointGroupDestroy(dJointGroupID g) {
    dJointGroupEmpty(g);
    delete g;
}
dJointID dJointCreateContact(dWorldID w, dJointGroupID group, const dContact *c) {
    dxJoint *j = new dxJoint();
    j->world = w;
    j->group = group;
    j->contact = *c;  // ode.cpp:1198 copies the contact
    w->joints.push_back(j);
    if (group) group->joints.push_back(j);
    return j;
}
static void set_relative_values(dxJoint *j);
void dJointAttach(dJointID j, dBodyID body1, dBodyID body2) {
    j->b1 = body1;
    j->b2 = body2;
    j->attached = body1 || body2;
    if (j->type != dJointTypeContact) {
        j->world->joints_dirty = true;
        if (j->attached) set_relative_values(j);  // ode.cpp:1434-1438
    }
}
void dJointDestroy(dJointID j) {
    dxWorld *w = j->world;
    if (j->type != dJointTypeContact) w->joints_dirty = true;
    auto &v = w->joints;
    for (size_t k = 0; k < v.size(); k++) if (v[k] == j) { v.erase(v.begin() + k); break; }
    if (j->group) {
        auto &gv = j->group->joints;
        for (size_t k = 0; k < gv.size(); k++) if (gv[k] == j) { gv.erase(gv.begin() + k); break; }
    }
    delete j;
}
void dJointSetFeedback(dJointID j, dJointFeedback *fb) { j->feedback = fb; }
dJointFeedback *dJointGetFeedback(dJointID j) { return j->feedback; }
dBodyID dJointGetBody(dJointID j, int index) {
    // a joint attached with a null first body reports its only body as body 0 (ode.cpp:1403-1411)
    dxBody *n0 = j->b1 ? j->b1 : j->b2, *n1 = j->b1 ? j->b2 : nullptr;
    return index == 0 ? n0 : (index == 1 ? n1 : nullptr);
}
// ode.cpp dAreConnectedExcluding: a joint of another type than joint_type
// connects the two bodies
int dAreConnectedExcluding(dBodyID b1, dBodyID b2, int joint_type) {
    if (!b1 || !b2) return 0;
    for (dxJoint *j : b1->world->joints)
        if (j->attached && j->type != joint_type && ((j->b1 == b1 && j->b2 == b2) || (j->b1 == b2 && j->b2 == b1)))
            return 1;
    return 0;
}
int dAreConnected(dBodyID b1, dBodyID b2) { return dAreConnectedExcluding(b1, b2, -1); }

// ---- ball and hinge joints (joints/ball.cpp, joints/hinge.cpp, joints/joint.cpp)
static dxJoint *joint_new(dWorldID w, dJointGroupID group, int type) {
    dxJoint *j = new dxJoint();
    j->world = w;
    j->group = group;
    j->type = type;
    j->erp = w->P.erp;  // ball.cpp:40-41
    j->cfm = w->P.cfm;
    j->limot.normal_cfm = w->P.cfm;  // joint.cpp:495-509
    j->limot.stop_erp = w->P.erp;
    j->limot.stop_cfm = w->P.cfm;
    j->limot2 = j->limot;
    if (type == dJointTypeHinge2) {  // hinge2.cpp:74-98
        j->axis2[0] = 0; j->axis2[1] = 1;
        j->susp_erp = w->P.erp;
        j->susp_cfm = w->P.cfm;
    }
    w->joints.push_back(j);
    if (group) group->joints.push_back(j);
    w->joints_dirty = true;
    return j;
}
dJointID dJointCreateBall(dWorldID w, dJointGroupID group) { return joint_new(w, group, dJointTypeBall); }
dJointID dJointCreateHinge(dWorldID w, dJointGroupID group) { return joint_new(w, group, dJointTypeHinge); }
dJointID dJointCreateHinge2(dWorldID w, dJointGroupID group) { return joint_new(w, group, dJointTypeHinge2); }
int dJointGetType(dJointID j) { return j->type; }

static void mul1_331(float *r, const float *R, const float *q) {  // R^T q (dMultiply1_331)
    const float r0 = R[0] * q[0] + R[4] * q[1] + R[8] * q[2];
    const float r1 = R[1] * q[0] + R[5] * q[1] + R[9] * q[2];
    const float r2 = R[2] * q[0] + R[6] * q[1] + R[10] * q[2];
    r[0] = r0; r[1] = r1; r[2] = r2;
}
static void mul0_331h(float *r, const float *R, const float *v) {  // R v (dMultiply0_331)
    const float r0 = R[0] * v[0] + R[1] * v[1] + R[2] * v[2];
    const float r1 = R[4] * v[0] + R[5] * v[1] + R[6] * v[2];
    const float r2 = R[8] * v[0] + R[9] * v[1] + R[10] * v[2];
    r[0] = r0; r[1] = r1; r[2] = r2;
}
// joint.cpp:289-322 setAnchors
static void set_anchors(dxJoint *j, float x, float y, float z, float *a1, float *a2) {
    world_download(j->world);
    dxBody *b0 = j->node0(), *b1 = j->node1();
    if (b0) {
        float q[4] = {x - b0->pos[0], y - b0->pos[1], z - b0->pos[2], 0};
        mul1_331(a1, b0->R, q);
        if (b1) {
            q[0] = x - b1->pos[0]; q[1] = y - b1->pos[1]; q[2] = z - b1->pos[2];
            mul1_331(a2, b1->R, q);
        } else {
            a2[0] = x; a2[1] = y; a2[2] = z;
        }
    }
    a1[3] = 0;
    a2[3] = 0;
    j->world->joints_dirty = true;
}
// odemath.cpp:95-151 dxSafeNormalize3: scale by the largest component first
static bool safe_normalize3(float *a) {
    const float a0 = fabsf(a[0]), a1 = fabsf(a[1]), a2 = fabsf(a[2]);
    int idx;
    if (a1 > a0) idx = a2 > a1 ? 2 : 1;
    else if (a2 > a0) idx = 2;
    else {
        if (!(a0 > 0.0f)) return false;
        idx = 0;
    }
    const int i1 = idx == 0 ? 1 : 0, i2 = idx == 2 ? 1 : 2;
    const float r = 1.0f / fabsf(a[idx]);
    const float b1 = a[i1] * r, b2 = a[i2] * r;
    const float l = 1.0f / sqrtf(1.0f + b1 * b1 + b2 * b2);
    a[i1] = b1 * l;
    a[i2] = b2 * l;
    a[idx] = copysignf(l, a[idx]);
    return true;
}
// odemath.cpp:37-50: dSafeNormalize3 / dNormalize3 (the reference's dNormalize3
// asserts on a zero vector; here it is left unchanged)
int dSafeNormalize3(dVector3 a) {
    float v[3] = {(float)a[0], (float)a[1], (float)a[2]};
    const bool ok = safe_normalize3(v);
    a[0] = v[0]; a[1] = v[1]; a[2] = v[2];
    return ok ? 1 : 0;
}
void dNormalize3(dVector3 a) { dSafeNormalize3(a); }
// joint.cpp:325-360 setAxes: either target may be null
static void set_axes(dxJoint *j, float x, float y, float z, float *ax1, float *ax2) {
    world_download(j->world);
    dxBody *b0 = j->node0(), *b1 = j->node1();
    if (b0) {
        float q[4] = {x, y, z, 0};
        safe_normalize3(q);  // dNormalize3
        if (ax1) {
            mul1_331(ax1, b0->R, q);
            ax1[3] = 0;
        }
        if (ax2) {
            if (b1) mul1_331(ax2, b1->R, q);
            else { ax2[0] = x; ax2[1] = y; ax2[2] = z; }
            ax2[3] = 0;
        }
    }
    j->world->joints_dirty = true;
}
static void cross3h(float *r, const float *a, const float *b) {
    const float r0 = a[1] * b[2] - a[2] * b[1], r1 = a[2] * b[0] - a[0] * b[2], r2 = a[0] * b[1] - a[1] * b[0];
    r[0] = r0; r[1] = r1; r[2] = r2;
}
static float dot3h(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
// hinge2.cpp:135-144 getAxisInfo (sin and cos of the angle between the axes)
static void hinge2_axis_info(const dxJoint *j, float *ax1, float *ax2, float *q, float &sa, float &ca) {
    mul0_331h(ax1, j->node0()->R, j->axis1);
    mul0_331h(ax2, j->node1()->R, j->axis2);
    cross3h(q, ax1, ax2);
    sa = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    ca = dot3h(ax1, ax2);
}
// hinge2.cpp:215-240 makeV1andV2
static void hinge2_make_v(dxJoint *j) {
    if (!j->node0() || !j->node1()) return;
    float ax1[3], ax2[3], v[3];
    mul0_331h(ax1, j->node0()->R, j->axis1);
    mul0_331h(ax2, j->node1()->R, j->axis2);
    const float k = dot3h(ax1, ax2);
    ax2[0] = ax2[0] + ax1[0] * -k; ax2[1] = ax2[1] + ax1[1] * -k; ax2[2] = ax2[2] + ax1[2] * -k;
    if (safe_normalize3(ax2)) {
        cross3h(v, ax1, ax2);
        mul1_331(j->v1, j->node0()->R, ax2);
        mul1_331(j->v2, j->node0()->R, v);
    }
}
// hinge.cpp:376-393 computeInitialRelativeRotation
static void hinge_qrel(dxJoint *j) {
    dxBody *b0 = j->node0(), *b1 = j->node1();
    if (!b0) return;
    if (b1) {
        const float *qb = b0->q, *qc = b1->q;  // dQMultiply1 (rotation.cpp:201-208)
        j->qrel[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
        j->qrel[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
        j->qrel[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
        j->qrel[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
    } else {
        j->qrel[0] = b0->q[0]; j->qrel[1] = -b0->q[1]; j->qrel[2] = -b0->q[2]; j->qrel[3] = -b0->q[3];
    }
}
void dJointSetBallAnchor(dJointID j, dReal x, dReal y, dReal z) { set_anchors(j, x, y, z, j->anchor1, j->anchor2); }
void dJointSetHingeAnchor(dJointID j, dReal x, dReal y, dReal z) {
    set_anchors(j, x, y, z, j->anchor1, j->anchor2);
    hinge_qrel(j);
}
void dJointSetHingeAxis(dJointID j, dReal x, dReal y, dReal z) {
    set_axes(j, x, y, z, j->axis1, j->axis2);
    hinge_qrel(j);
}
// hinge.cpp:211-228: the axis, then the initial relative rotation turned by
// the angle about it (dQMultiply3(qrel, q_angle, qrel), rotation.cpp:221-228)
void dJointSetHingeAxisOffset(dJointID j, dReal x, dReal y, dReal z, dReal dangle) {
    set_axes(j, x, y, z, j->axis1, j->axis2);
    hinge_qrel(j);
    if (!j->b1 && j->b2) dangle = -dangle;  // dJOINT_REVERSE
    dQuaternion qa;
    dQFromAxisAndAngle(qa, x, y, z, dangle);
    const float *qc = j->qrel;
    const float q0 = qa[0] * qc[0] - qa[1] * qc[1] - qa[2] * qc[2] - qa[3] * qc[3];
    const float q1 = -qa[0] * qc[1] - qa[1] * qc[0] + qa[2] * qc[3] - qa[3] * qc[2];
    const float q2 = -qa[0] * qc[2] - qa[2] * qc[0] + qa[3] * qc[1] - qa[1] * qc[3];
    const float q3 = -qa[0] * qc[3] - qa[3] * qc[0] + qa[1] * qc[2] - qa[2] * qc[1];
    j->qrel[0] = q0; j->qrel[1] = q1; j->qrel[2] = q2; j->qrel[3] = q3;
    j->world->joints_dirty = true;
}
// joint.cpp:363-393 getAnchor: anchor1 in world coordinates (reverse: anchor2 from node 1)
static void anchor_world(dxJoint *j, dVector3 out, const float *a, bool second) {
    world_download(j->world);
    dxBody *b = second ? j->node1() : j->node0();
    if (!b) { out[0] = a[0]; out[1] = a[1]; out[2] = a[2]; return; }
    mul0_331h(out, b->R, a);
    out[0] += b->pos[0]; out[1] += b->pos[1]; out[2] += b->pos[2];
}
void dJointGetBallAnchor(dJointID j, dVector3 out) {
    bool rev = !j->b1 && j->b2;
    anchor_world(j, out, rev ? j->anchor2 : j->anchor1, rev);
}
void dJointGetHingeAnchor(dJointID j, dVector3 out) {
    bool rev = !j->b1 && j->b2;
    anchor_world(j, out, rev ? j->anchor2 : j->anchor1, rev);
}
void dJointGetHingeAxis(dJointID j, dVector3 out) {
    world_download(j->world);
    dxBody *b0 = j->node0();
    if (b0) mul0_331h(out, b0->R, j->axis1);
}
// joint.cpp:511-544 dxJointLimitMotor::set
static void limot_set(Limot &l, int num, float v) {
    switch (num) {
    case dParamLoStop: l.lostop = v; break;
    case dParamHiStop: l.histop = v; break;
    case dParamVel: l.vel = v; break;
    case dParamFMax: if (v >= 0) l.fmax = v; break;
    case dParamFudgeFactor: if (v >= 0 && v <= 1) l.fudge_factor = v; break;
    case dParamBounce: l.bounce = v; break;
    case dParamCFM: l.normal_cfm = v; break;
    case dParamStopERP: l.stop_erp = v; break;
    case dParamStopCFM: l.stop_cfm = v; break;
    }
}
static float limot_get(const Limot &l, int num) {
    switch (num) {
    case dParamLoStop: return l.lostop;
    case dParamHiStop: return l.histop;
    case dParamVel: return l.vel;
    case dParamFMax: return l.fmax;
    case dParamFudgeFactor: return l.fudge_factor;
    case dParamBounce: return l.bounce;
    case dParamCFM: return l.normal_cfm;
    case dParamStopERP: return l.stop_erp;
    case dParamStopCFM: return l.stop_cfm;
    default: return 0;
    }
}
void dJointSetHingeParam(dJointID j, int parameter, dReal value) {
    limot_set(j->limot, parameter, value);  // hinge.cpp: all parameters go to the limit/motor
    j->world->joints_dirty = true;
}
dReal dJointGetHingeParam(dJointID j, int parameter) { return limot_get(j->limot, parameter); }
void dJointSetBallParam(dJointID j, int parameter, dReal value) {  // ball.cpp:150-160
    if (parameter == dParamCFM) j->cfm = value;
    else if (parameter == dParamERP) j->erp = value;
    j->world->joints_dirty = true;
}
dReal dJointGetBallParam(dJointID j, int parameter) {
    return parameter == dParamCFM ? j->cfm : (parameter == dParamERP ? j->erp : 0);
}
// joint.cpp:421-492 getHingeAngle
static float hinge_angle_host(const dxJoint *j) {
    dxBody *b0 = j->node0(), *b1 = j->node1();
    if (!b0) return 0;
    float qrel[4];
    const float *qb = b0->q, *qi = j->qrel;
    if (b1) {
        const float *qc = b1->q;
        float qq[4];  // dQMultiply1(qq, q0, q1), then dQMultiply2(qrel, qq, q_initial)
        qq[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
        qq[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
        qq[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
        qq[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
        qrel[0] = qq[0] * qi[0] + qq[1] * qi[1] + qq[2] * qi[2] + qq[3] * qi[3];
        qrel[1] = -qq[0] * qi[1] + qq[1] * qi[0] - qq[2] * qi[3] + qq[3] * qi[2];
        qrel[2] = -qq[0] * qi[2] + qq[2] * qi[0] - qq[3] * qi[1] + qq[1] * qi[3];
        qrel[3] = -qq[0] * qi[3] + qq[3] * qi[0] - qq[1] * qi[2] + qq[2] * qi[1];
    } else {  // dQMultiply3(qrel, q0, q_initial)
        qrel[0] = qb[0] * qi[0] - qb[1] * qi[1] - qb[2] * qi[2] - qb[3] * qi[3];
        qrel[1] = -qb[0] * qi[1] - qb[1] * qi[0] + qb[2] * qi[3] - qb[3] * qi[2];
        qrel[2] = -qb[0] * qi[2] - qb[2] * qi[0] + qb[3] * qi[1] - qb[1] * qi[3];
        qrel[3] = -qb[0] * qi[3] - qb[3] * qi[0] + qb[1] * qi[2] - qb[2] * qi[1];
    }
    const float cost2 = qrel[0];
    const float sint2 = sqrtf(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
    const float d = qrel[1] * j->axis1[0] + qrel[2] * j->axis1[1] + qrel[3] * j->axis1[2];
    float theta = d >= 0 ? 2 * atan2f(sint2, cost2) : 2 * atan2f(sint2, -cost2);
    if (theta > (float)M_PI) theta -= (float)(2 * M_PI);
    return -theta;
}
dReal dJointGetHingeAngle(dJointID j) {
    world_download(j->world);
    const float a = hinge_angle_host(j);
    return (!j->b1 && j->b2) ? -a : a;
}

// hinge2.cpp:272-330
void dJointSetHinge2Anchor(dJointID j, dReal x, dReal y, dReal z) {
    set_anchors(j, x, y, z, j->anchor1, j->anchor2);
    hinge2_make_v(j);
}
void dJointSetHinge2Axes(dJointID j, const dReal *axis1, const dReal *axis2) {
    if (axis1) set_axes(j, axis1[0], axis1[1], axis1[2], j->axis1, nullptr);
    if (axis2) set_axes(j, axis2[0], axis2[1], axis2[2], nullptr, j->axis2);
    if (j->node0() && j->node1()) {
        float ax1[3], ax2[3], q[3];
        hinge2_axis_info(j, ax1, ax2, q, j->s0, j->c0);
    }
    hinge2_make_v(j);
}
void dJointSetHinge2Axis1(dJointID j, dReal x, dReal y, dReal z) {
    const dReal a[3] = {x, y, z};
    dJointSetHinge2Axes(j, a, nullptr);
}
void dJointSetHinge2Axis2(dJointID j, dReal x, dReal y, dReal z) {
    const dReal a[3] = {x, y, z};
    dJointSetHinge2Axes(j, nullptr, a);
}
void dJointSetHinge2Param(dJointID j, int parameter, dReal value) {  // hinge2.cpp:333-347
    if ((parameter & 0xff00) == 0x100) limot_set(j->limot2, parameter & 0xff, value);
    else if (parameter == dParamSuspensionERP) j->susp_erp = value;
    else if (parameter == dParamSuspensionCFM) j->susp_cfm = value;
    else limot_set(j->limot, parameter, value);
    j->world->joints_dirty = true;
}
dReal dJointGetHinge2Param(dJointID j, int parameter) {
    if ((parameter & 0xff00) == 0x100) return limot_get(j->limot2, parameter & 0xff);
    if (parameter == dParamSuspensionERP) return j->susp_erp;
    if (parameter == dParamSuspensionCFM) return j->susp_cfm;
    return limot_get(j->limot, parameter);
}
void dJointGetHinge2Anchor(dJointID j, dVector3 out) {
    bool rev = !j->b1 && j->b2;
    anchor_world(j, out, rev ? j->anchor2 : j->anchor1, rev);
}
// hinge2.cpp:377-411: the axes in world coordinates from the first and the
// second attached body (zero without that body)
void dJointGetHinge2Axis1(dJointID j, dVector3 out) {
    world_download(j->world);
    if (j->node0()) mul0_331h(out, j->node0()->R, j->axis1);
    else out[0] = out[1] = out[2] = 0;
}
void dJointGetHinge2Axis2(dJointID j, dVector3 out) {
    world_download(j->world);
    if (j->node1()) mul0_331h(out, j->node1()->R, j->axis2);
    else out[0] = out[1] = out[2] = 0;
}
// setRelativeValues, run by dJointAttach: the anchor and the axes as they read
// in world coordinates with the new bodies, set again, so that the body-frame
// values follow the bodies just attached (ball.cpp:178-183, hinge.cpp:362-372,
// hinge2.cpp:521-545; a hinge2 needs both bodies for its axis information)
static void set_relative_values(dxJoint *j) {
    dVector3 a, x1, x2;
    if (j->type == dJointTypeBall) {
        dJointGetBallAnchor(j, a);
        dJointSetBallAnchor(j, a[0], a[1], a[2]);
    } else if (j->type == dJointTypeHinge) {
        dJointGetHingeAnchor(j, a);
        set_anchors(j, a[0], a[1], a[2], j->anchor1, j->anchor2);
        x1[0] = x1[1] = x1[2] = 0;
        dJointGetHingeAxis(j, x1);
        dJointSetHingeAxis(j, x1[0], x1[1], x1[2]);
    } else if (j->type == dJointTypeHinge2) {
        dJointGetHinge2Anchor(j, a);
        set_anchors(j, a[0], a[1], a[2], j->anchor1, j->anchor2);
        dJointGetHinge2Axis1(j, x1);
        dJointGetHinge2Axis2(j, x2);
        dJointSetHinge2Axes(j, x1, j->node1() ? x2 : nullptr);
    }
}
// hinge2.cpp:33-51 measureAngle1
dReal dJointGetHinge2Angle1(dJointID j) {
    world_download(j->world);
    float p[3], q[3];
    if (j->node1()) mul0_331h(p, j->node1()->R, j->axis2);
    else { p[0] = j->axis2[0]; p[1] = j->axis2[1]; p[2] = j->axis2[2]; }
    if (j->node0()) mul1_331(q, j->node0()->R, p);
    else { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    return -atan2f(dot3h(j->v2, q), dot3h(j->v1, q));
}

// ---- bulk builders for large batched scenes (extensions): the same calls an
// ODE program makes per object, looped on the host side of the library
int gbodeCreateBodies(dWorldID w, int n, const float *rows, dBodyID *out) {
    if (!w || n < 0 || (n > 0 && (!rows || !out))) { set_error("gbodeCreateBodies: bad argument"); return 0; }
    dMass m;
    for (int i = 0; i < n; i++) {
        const float *r = rows + 20 * (size_t)i;
        dBodyID b = dBodyCreate(w);
        dBodySetPosition(b, r[0], r[1], r[2]);
        const dReal q[4] = {r[3], r[4], r[5], r[6]};
        dBodySetQuaternion(b, q);
        dBodySetLinearVel(b, r[7], r[8], r[9]);
        dBodySetAngularVel(b, r[10], r[11], r[12]);
        dMassSetParameters(&m, r[13], 0, 0, 0, r[14], r[15], r[16], r[17], r[18], r[19]);
        dBodySetMass(b, &m);
        out[i] = b;
    }
    return 1;
}
int gbodeCreateGeoms(dSpaceID space, int n, const int *cls, const float *dims, const float *pos, const float *R,
                     const dBodyID *body, dGeomID *out) {
    if (!space || n < 0 || (n > 0 && (!cls || !dims || !out))) { set_error("gbodeCreateGeoms: bad argument"); return 0; }
    for (int i = 0; i < n; i++) {
        const float *d = dims + 4 * (size_t)i;
        dGeomID g;
        switch (cls[i]) {
        case dSphereClass: g = dCreateSphere(space, d[0]); break;
        case dBoxClass: g = dCreateBox(space, d[0], d[1], d[2]); break;
        case dCapsuleClass: g = dCreateCapsule(space, d[0], d[1]); break;
        case dPlaneClass: g = dCreatePlane(space, d[0], d[1], d[2], d[3]); break;
        default: set_error("gbodeCreateGeoms: unsupported class"); return 0;
        }
        if (body && body[i]) dGeomSetBody(g, body[i]);
        else if (cls[i] != dPlaneClass) {
            if (pos) dGeomSetPosition(g, pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]);
            if (R) dGeomSetRotation(g, R + 12 * (size_t)i);
        }
        out[i] = g;
    }
    return 1;
}
int gbodeCreateJoints(dWorldID w, int n, const float *rows, const dBodyID *bodies, dJointID *out) {
    if (!w || n < 0 || (n > 0 && (!rows || !bodies || !out))) { set_error("gbodeCreateJoints: bad argument"); return 0; }
    for (int i = 0; i < n; i++) {
        const float *r = rows + GBODE_JOINT_COLS * (size_t)i;
        const int t = (int)r[0], b1 = (int)r[1], b2 = (int)r[2];
        dJointID j;
        if (t == dJointTypeBall) j = dJointCreateBall(w, nullptr);
        else if (t == dJointTypeHinge) j = dJointCreateHinge(w, nullptr);
        else if (t == dJointTypeHinge2) j = dJointCreateHinge2(w, nullptr);
        else { set_error("gbodeCreateJoints: unsupported joint type"); return 0; }
        dJointAttach(j, b1 >= 0 ? bodies[b1] : nullptr, b2 >= 0 ? bodies[b2] : nullptr);
        if (t == dJointTypeBall) {
            dJointSetBallAnchor(j, r[3], r[4], r[5]);
        } else if (t == dJointTypeHinge) {
            dJointSetHingeAnchor(j, r[3], r[4], r[5]);
            dJointSetHingeAxis(j, r[6], r[7], r[8]);
            dJointSetHingeParam(j, dParamLoStop, r[9]);
            dJointSetHingeParam(j, dParamHiStop, r[10]);
            if (r[19] > 0) { dJointSetHingeParam(j, dParamVel, r[18]); dJointSetHingeParam(j, dParamFMax, r[19]); }
        } else {
            dJointSetHinge2Anchor(j, r[3], r[4], r[5]);
            const dReal a1[3] = {r[6], r[7], r[8]}, a2[3] = {r[11], r[12], r[13]};
            dJointSetHinge2Axes(j, a1, a2);
            dJointSetHinge2Param(j, dParamLoStop, r[9]);
            dJointSetHinge2Param(j, dParamHiStop, r[10]);
            dJointSetHinge2Param(j, dParamVel2, r[14]);
            dJointSetHinge2Param(j, dParamFMax2, r[15]);
            dJointSetHinge2Param(j, dParamSuspensionERP, r[16]);
            dJointSetHinge2Param(j, dParamSuspensionCFM, r[17]);
        }
        out[i] = j;
    }
    return 1;
}

// Upload the ball and hinge joints (attached, in world order) when they changed.
static bool upload_joint_table(dxWorld *w) {
    if (!w->joints_dirty) return true;
    std::vector<dxJoint *> jt;
    for (dxJoint *j : w->joints)
        if (j->attached && j->type != dJointTypeContact && j->node0()) jt.push_back(j);
    const int n = (int)jt.size();
    std::vector<int4> info(n);
    std::vector<float4> a1(n), a2(n), x1(n), x2(n), qr(n), l0(n), l1(n), l2(n), hv1(n), hv2(n), m0(n), m1(n), m2(n);
    for (int k = 0; k < n; k++) {
        const dxJoint *j = jt[k];
        info[k] = make_int4(j->type, j->node0()->index, j->node1() ? j->node1()->index : -1, (!j->b1 && j->b2) ? 1 : 0);
        a1[k] = make_float4(j->anchor1[0], j->anchor1[1], j->anchor1[2], 0.f);
        a2[k] = make_float4(j->anchor2[0], j->anchor2[1], j->anchor2[2], 0.f);
        x1[k] = make_float4(j->axis1[0], j->axis1[1], j->axis1[2], 0.f);
        x2[k] = make_float4(j->axis2[0], j->axis2[1], j->axis2[2], 0.f);
        qr[k] = make_float4(j->qrel[0], j->qrel[1], j->qrel[2], j->qrel[3]);
        const Limot &L = j->limot;
        l0[k] = make_float4(L.lostop, L.histop, L.vel, L.fmax);
        l1[k] = make_float4(L.fudge_factor, L.bounce, L.normal_cfm, L.stop_erp);
        l2[k] = make_float4(L.stop_cfm, j->erp, j->cfm, 0.f);
        hv1[k] = make_float4(j->v1[0], j->v1[1], j->v1[2], j->s0);
        hv2[k] = make_float4(j->v2[0], j->v2[1], j->v2[2], j->c0);
        const Limot &M = j->limot2;
        m0[k] = make_float4(M.lostop, M.histop, M.vel, M.fmax);
        m1[k] = make_float4(M.fudge_factor, M.bounce, M.normal_cfm, M.stop_erp);
        m2[k] = make_float4(M.stop_cfm, j->susp_erp, j->susp_cfm, 0.f);
    }
    std::vector<const void *> src = {info.data(), a1.data(), a2.data(), x1.data(), x2.data(), qr.data(),
                                     l0.data(), l1.data(), l2.data(), hv1.data(), hv2.data(), m0.data(),
                                     m1.data(), m2.data()};
    if (!joint_table_upload(w->ws, n, src, w->stream)) return false;
    w->table_joints = jt;
    w->joints_dirty = false;
    return true;
}

// Joint feedback of the last step (quickstep.cpp:3108-3181, the same for
// dWorldStep): F = J^T lambda for every contact joint in `cj` (the step's
// solved contact joints, in row order) and every ball/hinge/hinge2 joint
// with a dJointFeedback; a joint that was not solved (its component sleeps)
// keeps what it had.
static void write_feedback(dxWorld *w, const std::vector<dxJoint *> &cj) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(w->stream, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
        return;  // a step being recorded into a graph: the launch that runs it reads the feedback
    bool any = false;
    for (dxJoint *j : cj) if (j->feedback) { any = true; break; }
    for (dxJoint *j : w->table_joints) if (j->feedback) { any = true; break; }
    if (!any) return;
    std::vector<float> fb;
    const int nc = (int)cj.size(), nj = (int)w->table_joints.size();
    joint_feedback(w->ws, nc, nj, fb, w->stream);
    for (int k = 0; k < nc + nj; k++) {
        dJointFeedback *f = k < nc ? cj[k]->feedback : w->table_joints[k - nc]->feedback;
        if (!f) continue;
        const float *o = &fb[16 * (size_t)k];
        if (o[3] == 0.f) continue;
        for (int q = 0; q < 3; q++) { f->f1[q] = o[q]; f->t1[q] = o[4 + q]; f->f2[q] = o[8 + q]; f->t2[q] = o[12 + q]; }
        f->f1[3] = f->t1[3] = f->f2[3] = f->t2[3] = 0;
    }
}

// ------------------------------------------------------------------ stepping
// joints/contact.cpp:49-122 getInfo1 on the host, for the island schedule
static int host_contact_m(const dSurfaceParameters &s) {
    int m = 1;
    if (s.mode & dContactAxisDep) {
        if (s.mu > 0) m++;
        if (s.mu2 > 0) m++;
        if (s.mode & dContactRolling) { if (!(s.rho < 0)) m++; if (!(s.rho2 < 0)) m++; if (!(s.rhoN < 0)) m++; }
    } else {
        if (s.mu > 0) m += 2;
        if (s.mode & dContactRolling) { if (!(s.rho < 0)) m += 3; }
    }
    return m;
}

// util.cpp:724-860: islands by depth-first search from the newest body over
// each body's joint list (newest attached first), as the reference orders
// them, giving the row order of the reference-order solver.
static void build_islands(dxWorld *w, const std::vector<dxJoint *> &js, const std::vector<int> &rstart,
                          const std::vector<int> &mrows, IslandSchedule &sch) {
    int nb = (int)w->bodies.size(), nj = (int)js.size();
    std::vector<int> cnt(nb + 1, 0);
    std::vector<int> n0(nj), n1(nj);
    for (int k = 0; k < nj; k++) {
        dxJoint *j = js[k];
        int a = j->b1 ? j->b1->index : (j->b2 ? j->b2->index : -1);
        int b = j->b1 ? (j->b2 ? j->b2->index : -1) : -1;
        n0[k] = a; n1[k] = b;
        if (a >= 0) cnt[a]++;
        if (b >= 0) cnt[b]++;
    }
    std::vector<int> start(nb + 1, 0);
    for (int i = 0; i < nb; i++) start[i + 1] = start[i] + cnt[i];
    std::vector<int> lj(start[nb] + 1), lb(start[nb] + 1), fill(nb, 0);
    for (int k = nj - 1; k >= 0; k--) {
        int a = n0[k], b = n1[k];
        if (a >= 0) { int p = start[a] + fill[a]++; lj[p] = k; lb[p] = b; }
        if (b >= 0) { int p = start[b] + fill[b]++; lj[p] = k; lb[p] = a; }
    }
    std::vector<char> btag(nb, 0), jtag(nj, 0);
    std::vector<int> stack, ib, ij;
    sch.start.assign(1, 0);
    sch.bstart.assign(1, 0);
    for (int bb = nb - 1; bb >= 0; bb--) {
        if (btag[bb]) continue;
        btag[bb] = 1;
        ib.assign(1, bb);
        ij.clear();
        stack.clear();
        int b = bb;
        for (;;) {
            for (int p = start[b]; p < start[b + 1]; p++) {
                int k = lj[p];
                if (!jtag[k]) {
                    jtag[k] = 1;
                    ij.push_back(k);
                    int nbody = lb[p];
                    if (nbody >= 0 && !btag[nbody]) { btag[nbody] = 1; stack.push_back(nbody); }
                }
            }
            if (stack.empty()) break;
            b = stack.back();
            stack.pop_back();
            ib.push_back(b);
        }
        if (ij.empty()) continue;  // a lone body has no rows; it is integrated by the body pass
        // ReorderPrep (quickstep.cpp:2329-2355): findex<0 rows first, each group in row order
        std::vector<int> normals, frictions;
        for (int k : ij) {
            int r0 = rstart[k];
            const dSurfaceParameters &s = js[k]->contact.surface;
            for (int r = 0; r < mrows[k]; r++) {
                bool fr = false;
                if (r >= 1) {
                    // friction rows carry findex under dContactApprox1_1/_2 (contact.cpp:257-293)
                    int row = 1;
                    float mu = s.mu > 0 ? s.mu : 0;
                    float mu2 = (s.mode & dContactMu2) ? (s.mu2 > 0 ? s.mu2 : 0) : mu;
                    int which = -1;
                    if (mu > 0) { if (r == row) which = 1; row++; }
                    if (mu2 > 0) { if (r == row) which = 2; row++; }
                    if (which == 1) fr = (s.mode & dContactApprox1_1) != 0;
                    else if (which == 2) fr = (s.mode & dContactApprox1_2) != 0;
                    else if (s.mode & dContactRolling) {
                        const int bits[3] = {dContactApprox1_1, dContactApprox1_2, dContactApprox1_N};
                        float rho[3] = {s.rho, (s.mode & dContactAxisDep) ? s.rho2 : s.rho, (s.mode & dContactAxisDep) ? s.rhoN : s.rho};
                        for (int q = 0; q < 3; q++)
                            if (rho[q] > 0) { if (r == row) { fr = (s.mode & bits[q]) != 0; } row++; }
                    }
                }
                (fr ? frictions : normals).push_back(r0 + r);
            }
        }
        sch.order.insert(sch.order.end(), normals.begin(), normals.end());
        sch.order.insert(sch.order.end(), frictions.begin(), frictions.end());
        sch.start.push_back((int)sch.order.size());
        sch.bodies.insert(sch.bodies.end(), ib.begin(), ib.end());
        sch.bstart.push_back((int)sch.bodies.size());
    }
}

static bool upload_host_contacts(dxWorld *w, const std::vector<dxJoint *> &js) {
    int nc = (int)js.size();
    Workspace &ws = w->ws;
    if (ws.contact_cap < nc) {
        if (!ws.contacts.ensure((size_t)nc * sizeof(Contact))) return false;
        ws.contact_cap = nc;
    }
    if (!ws.surfaces.ensure((size_t)(nc > 0 ? nc : 1) * sizeof(Surface))) return false;
    std::vector<Contact> C(nc);
    std::vector<Surface> S(nc);
    ws.rows_per_contact = 3;
    for (const dxJoint *j : js)
        if (j->contact.surface.mode & dContactRolling) ws.rows_per_contact = 6;
    for (int k = 0; k < nc; k++) {
        const dContact &c = js[k]->contact;
        Contact &o = C[k];
        o.pos_depth = make_float4(c.geom.pos[0], c.geom.pos[1], c.geom.pos[2], c.geom.depth);
        o.normal = make_float4(c.geom.normal[0], c.geom.normal[1], c.geom.normal[2], 0.f);
        o.b1 = js[k]->b1 ? js[k]->b1->index : -1;
        o.b2 = js[k]->b2 ? js[k]->b2->index : -1;
        o.surf = k;
        o.g1 = c.geom.g1 ? c.geom.g1->uid : -1;
        o.g2 = c.geom.g2 ? c.geom.g2->uid : -1;
        // slot: position among consecutive contacts of the same geom pair
        o.slot = (k > 0 && C[k - 1].g1 == o.g1 && C[k - 1].g2 == o.g2) ? C[k - 1].slot + 1 : 0;
        o.pad0 = o.pad1 = 0;
        Surface &s = S[k];
        memset(&s, 0, sizeof s);
        const dSurfaceParameters &sp = c.surface;
        s.mode = sp.mode; s.mu = sp.mu; s.mu2 = sp.mu2; s.rho = sp.rho; s.rho2 = sp.rho2; s.rhoN = sp.rhoN;
        s.bounce = sp.bounce; s.bounce_vel = sp.bounce_vel; s.soft_erp = sp.soft_erp; s.soft_cfm = sp.soft_cfm;
        s.motion1 = sp.motion1; s.motion2 = sp.motion2; s.motionN = sp.motionN; s.slip1 = sp.slip1; s.slip2 = sp.slip2;
        s.fdir1[0] = c.fdir1[0]; s.fdir1[1] = c.fdir1[1]; s.fdir1[2] = c.fdir1[2];
    }
    cudaStream_t s = w->stream;
    if (nc > 0) {
        cudaMemcpyAsync(ws.contacts.p, C.data(), (size_t)nc * sizeof(Contact), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ws.surfaces.p, S.data(), (size_t)nc * sizeof(Surface), cudaMemcpyHostToDevice, s);
    }
    cudaMemcpyAsync(&ws.dc->ncontacts, &nc, 4, cudaMemcpyHostToDevice, s);
    return cudaStreamSynchronize(s) == cudaSuccess;
}

int dWorldQuickStep(dWorldID w, dReal stepsize) {
    if (!world_upload(w)) return 0;
    Workspace &ws = w->ws;
    SolverParams P = w->P;
    P.dt = stepsize;
    cudaStream_t s = w->stream;
    // host-created contact joints (attached) in creation order
    std::vector<dxJoint *> js;
    js.reserve(w->joints.size());
    for (dxJoint *j : w->joints) if (j->attached && j->type == dJointTypeContact) js.push_back(j);
    if (!upload_joint_table(w)) { set_error("dWorldQuickStep: joint table upload"); return 0; }
    if (w->ws.njoints > 0 && P.solver == GBODE_SOLVER_REFERENCE_ORDER && !w->device_contacts) {
        set_error("dWorldQuickStep: the reference-order solver handles contact joints only");
        return 0;
    }
    int nb = (int)w->bodies.size();
    if (w->timing) cudaEventRecord(w->ev[2], s);
    bool ok;
    if (!js.empty() && w->device_contacts) {
        set_error("dWorldQuickStep: a step mixes dJointCreateContact joints with gbodeSpaceCollideContacts contacts");
        return 0;
    }
    if (!w->device_contacts) {
        if (!upload_host_contacts(w, js)) { set_error("upload contacts"); return 0; }
    } else if (ws.contact_cap <= 0) {
        if (!ws.contacts.ensure(sizeof(Contact))) { set_error("device allocation (contacts)"); return 0; }
        ws.contact_cap = 1;
    }
    if (!ws.surfaces.p && !ws.surfaces.ensure(sizeof(Surface))) { set_error("device allocation (surfaces)"); return 0; }
    // the contact joints whose index the rows carry (feedback below)
    std::vector<dxJoint *> awake_js;
    const std::vector<dxJoint *> *solved = &js;
    if (P.solver == GBODE_SOLVER_REFERENCE_ORDER && !w->device_contacts) {
        if (ws.sleep_on) {
            // the sleep stage sees every contact joint; the host-built islands
            // then hold the contacts of awake components only
            if (!launch_sleep(ws, nb, stepsize, s)) { set_error("dWorldQuickStep: sleep stage", cudaGetLastError()); return 0; }
            std::vector<int> asleep(nb > 0 ? nb : 1);
            if (nb > 0) cudaMemcpyAsync(asleep.data(), ws.b_asleep.p, 4 * (size_t)nb, cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess) { set_error("dWorldQuickStep: sleep stage"); return 0; }
            for (dxJoint *j : js) {
                const dxBody *b = j->b1 ? j->b1 : j->b2;
                if (b && !asleep[b->index]) awake_js.push_back(j);
            }
            if (!upload_host_contacts(w, awake_js)) { set_error("upload contacts"); return 0; }
            ws.sleep_precomputed = true;
            solved = &awake_js;
        }
        const std::vector<dxJoint *> &sj = *solved;
        int nc = (int)sj.size();
        std::vector<int> mrows(nc), rstart(nc + 1, 0);
        for (int k = 0; k < nc; k++) {
            mrows[k] = host_contact_m(sj[k]->contact.surface);
            rstart[k + 1] = rstart[k] + mrows[k];
        }
        IslandSchedule sch;
        build_islands(w, sj, rstart, mrows, sch);
        ok = launch_quickstep_islands(ws, nb, P, sch, s, w->timing ? w->ev[0] : nullptr, w->timing ? w->ev[1] : nullptr);
    } else {
        ok = launch_quickstep(ws, nb, 1, P, s, w->timing ? w->ev[0] : nullptr, w->timing ? w->ev[1] : nullptr);
    }
    if (w->timing) cudaEventRecord(w->ev[3], s);
    if (!ok) { set_error("dWorldQuickStep launch", cudaGetLastError()); return 0; }
    w->host_valid = false;
    w->stats_pending = true;
    w->last_host_contacts = (int)js.size();
    write_feedback(w, *solved);
    return 1;
}

static void drop_graph(dxWorld *w) {
    if (w->gexec) cudaGraphExecDestroy(w->gexec);
    if (w->graph) cudaGraphDestroy(w->graph);
    w->gexec = nullptr;
    w->graph = nullptr;
    w->graph_state = 0;
}

// One fused step: gbodeSpaceCollideContacts + dWorldQuickStep +
// dJointGroupEmpty.  With use_graph, the step's kernels, copies and memsets
// are recorded once into a CUDA graph (on the second call after anything that
// changes them: sizes, parameters, host-side edits of bodies, joints or
// geoms) and replayed by one cudaGraphLaunch afterwards.
int gbodeWorldStepFused(dWorldID w, dSpaceID space, dJointGroupID group, const dSurfaceParameters *sp, int maxc,
                        dReal dt, int use_graph) {
    if (!w || !space || !group || !sp || maxc < 1 || !(dt > 0)) {
        set_error("gbodeWorldStepFused: bad argument");
        return 0;
    }
    auto plain = [&]() -> int {
        if (!gbodeSpaceCollideContacts(space, w, group, sp, maxc)) return 0;
        const int ok = dWorldQuickStep(w, dt);
        dJointGroupEmpty(group);
        return ok;
    };
    if (!use_graph) return plain();
    std::vector<unsigned char> key;
    auto put = [&](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        key.insert(key.end(), c, c + n);
    };
    const int nb = (int)w->bodies.size(), ng = (int)space->geoms.size();
    put(&space, sizeof space); put(&group, sizeof group); put(&maxc, sizeof maxc); put(&dt, sizeof dt);
    put(sp, sizeof *sp); put(&w->P, sizeof w->P); put(&nb, sizeof nb); put(&ng, sizeof ng);
    put(&w->ws.sleep_on, sizeof w->ws.sleep_on); put(&w->ws.adis_S, sizeof w->ws.adis_S);
    const bool clean = !w->dev_dirty && !w->joints_dirty && !space->dirty && w->uploaded_space == space &&
                       !w->timing && w->stream != nullptr && group->joints.empty();
    if (clean && key == w->graph_key && w->graph_state == 2) {
        cudaError_t e = cudaGraphLaunch(w->gexec, w->stream);
        if (e != cudaSuccess) { set_error("gbodeWorldStepFused: graph launch", e); drop_graph(w); return 0; }
        // the host-side effects of a fused step
        w->host_valid = false;
        w->stats_pending = true;
        w->last_host_contacts = 0;
        w->device_contacts = false;
        w->device_surfaces = 1;
        write_feedback(w, {});
        return 1;
    }
    if (clean && key == w->graph_key && w->graph_state == 1) {
        drop_graph(w);
        cudaError_t e = cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { set_error("gbodeWorldStepFused: begin capture", e); return 0; }
        const int ok = plain();  // recorded, not run
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(w->stream, &g);
        if (!ok || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            set_error("gbodeWorldStepFused: capture failed", e);
            return 0;
        }
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        if (e != cudaSuccess) { cudaGraphDestroy(g); set_error("gbodeWorldStepFused: instantiate", e); return 0; }
        w->graph = g;
        w->gexec = ex;
        w->graph_state = 2;
        e = cudaGraphLaunch(ex, w->stream);  // run the step just recorded
        if (e != cudaSuccess) { set_error("gbodeWorldStepFused: graph launch", e); drop_graph(w); return 0; }
        write_feedback(w, {});
        return 1;
    }
    // a plain step settles buffer sizes and uploads; the next call captures
    drop_graph(w);
    const int ok = plain();
    w->graph_key = key;
    w->graph_state = ok ? 1 : 0;
    return ok;
}

// dWorldStep (ode.cpp:1828-1845, step.cpp): the rows of the step as for
// dWorldQuickStep, then one dense LCP per island solved exactly on the device
// (dantzig.cu), then the same integration.  Islands (util.cpp:724-860) are the
// connected components of the bodies through this step's contact joints and
// the ball/hinge/hinge2 joints; the static environment joins nothing.
int dWorldStep(dWorldID w, dReal stepsize) {
    if (!world_upload(w)) return 0;
    Workspace &ws = w->ws;
    SolverParams P = w->P;
    P.dt = stepsize;
    P.warm_mode = 0;
    P.learned = 0;
    P.learn_capture = 0;
    cudaStream_t s = w->stream;
    const bool dev = w->device_contacts;  // contacts from gbodeSpaceCollideContacts, on the device
    std::vector<dxJoint *> js;
    for (dxJoint *j : w->joints) if (j->attached && j->type == dJointTypeContact) js.push_back(j);
    if (dev && !js.empty()) {
        set_error("dWorldStep: a step mixes dJointCreateContact joints with gbodeSpaceCollideContacts contacts");
        return 0;
    }
    if (!upload_joint_table(w)) { set_error("dWorldStep: joint table upload"); return 0; }
    if (!dev && !upload_host_contacts(w, js)) { set_error("upload contacts"); return 0; }
    if (dev && ws.contact_cap <= 0) {
        if (!ws.contacts.ensure(sizeof(Contact))) { set_error("device allocation (contacts)"); return 0; }
        ws.contact_cap = 1;
    }
    if (!ws.surfaces.p && !ws.surfaces.ensure(sizeof(Surface))) { set_error("device allocation (surfaces)"); return 0; }
    const int nb = (int)w->bodies.size();
    std::vector<dxJoint *> awake_js;
    const std::vector<dxJoint *> *solved = &js;
    if (ws.sleep_on && !dev) {
        if (!launch_sleep(ws, nb, stepsize, s)) { set_error("dWorldStep: sleep stage", cudaGetLastError()); return 0; }
        std::vector<int> asleep(nb > 0 ? nb : 1);
        if (nb > 0) cudaMemcpyAsync(asleep.data(), ws.b_asleep.p, 4 * (size_t)nb, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) { set_error("dWorldStep: sleep stage"); return 0; }
        for (dxJoint *j : js) {
            const dxBody *b = j->b1 ? j->b1 : j->b2;
            if (b && !asleep[b->index]) awake_js.push_back(j);
        }
        if (!upload_host_contacts(w, awake_js)) { set_error("upload contacts"); return 0; }
        ws.sleep_precomputed = true;
        solved = &awake_js;
    }
    if (w->timing) cudaEventRecord(w->ev[2], s);
    if (!assemble_step(ws, nb, P, s)) { set_error("dWorldStep: assembly", cudaGetLastError()); return 0; }
    // row ranges: contacts in order (rows per contact from getInfo1), then the
    // joints' rows after all contact rows (row counts from the device)
    const std::vector<dxJoint *> &sj = *solved;
    std::vector<int2> cbody;  // per contact: bodies (static -1)
    std::vector<int> crow, cm;  // per contact: first row, rows
    int nc;
    if (dev) {
        nc = download_solver_contacts(ws, cbody, crow, cm, s);
        if (nc < 0) { set_error("dWorldStep: contacts"); return 0; }
    } else {
        nc = (int)sj.size();
        cbody.resize(nc > 0 ? nc : 1);
        crow.assign(nc > 0 ? nc : 1, 0);
        cm.assign(nc > 0 ? nc : 1, 0);
        int r = 0;
        for (int k = 0; k < nc; k++) {
            cbody[k] = make_int2(sj[k]->b1 ? sj[k]->b1->index : -1, sj[k]->b2 ? sj[k]->b2->index : -1);
            crow[k] = r;
            cm[k] = host_contact_m(sj[k]->contact.surface);
            r += cm[k];
        }
    }
    int ncrows = 0;
    for (int k = 0; k < nc; k++) ncrows = crow[k] + cm[k] > ncrows ? crow[k] + cm[k] : ncrows;
    const int nj = ws.njoints;
    std::vector<int> jm(nj > 0 ? nj : 1), jr(nj > 0 ? nj : 1);
    std::vector<int4> jinfo(nj > 0 ? nj : 1);
    if (nj > 0) {
        cudaMemcpyAsync(jm.data(), ws.j_m.p, 4 * (size_t)nj, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(jr.data(), ws.j_rstart.p, 4 * (size_t)nj, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(jinfo.data(), ws.j_info.p, 16 * (size_t)nj, cudaMemcpyDeviceToHost, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) { set_error("dWorldStep: row counts"); return 0; }
    // components (union-find over bodies)
    std::vector<int> parent(nb > 0 ? nb : 1);
    for (int i = 0; i < nb; i++) parent[i] = i;
    auto find = [&](int x) {
        while (parent[x] != x) { parent[x] = parent[parent[x]]; x = parent[x]; }
        return x;
    };
    auto unite = [&](int a, int b) {
        if (a < 0 || b < 0) return;
        a = find(a); b = find(b);
        if (a != b) parent[a > b ? a : b] = a > b ? b : a;
    };
    for (int k = 0; k < nc; k++) unite(cbody[k].x, cbody[k].y);
    for (int k = 0; k < nj; k++)
        if (jm[k] > 0) unite(jinfo[k].y, jinfo[k].z);
    std::vector<std::vector<int>> rows_of(nb > 0 ? nb : 1);
    for (int k = 0; k < nc; k++) {
        const int b = cbody[k].x >= 0 ? cbody[k].x : cbody[k].y;
        if (b < 0) continue;
        auto &v = rows_of[find(b)];
        for (int r = crow[k]; r < crow[k] + cm[k]; r++) v.push_back(r);
    }
    for (int k = 0; k < nj; k++) {
        if (jm[k] <= 0) continue;
        const int b = jinfo[k].y >= 0 ? jinfo[k].y : jinfo[k].z;
        if (b < 0) continue;
        auto &v = rows_of[find(b)];
        for (int r = 0; r < jm[k]; r++) v.push_back(ncrows + jr[k] + r);
    }
    std::vector<int> order, start(1, 0);
    for (int i = 0; i < nb; i++) {
        if (rows_of[i].empty()) continue;
        order.insert(order.end(), rows_of[i].begin(), rows_of[i].end());
        start.push_back((int)order.size());
    }
    if (w->timing) cudaEventRecord(w->ev[0], s);
    if (!launch_dantzig(ws, order, start, s)) { set_error("dWorldStep: island solve", cudaGetLastError()); return 0; }
    if (w->timing) cudaEventRecord(w->ev[1], s);
    if (!launch_integrate(ws, nb, P, s)) { set_error("dWorldStep: integration", cudaGetLastError()); return 0; }
    if (w->timing) cudaEventRecord(w->ev[3], s);
    w->host_valid = false;
    w->stats_pending = true;
    w->last_host_contacts = (int)js.size();
    write_feedback(w, sj);
    return 1;
}

int gbodeWorldAutotune(dWorldID w, dSpaceID space, dJointGroupID group, const dSurfaceParameters *sp, int maxc,
                       dReal dt, int steps, int use_graph, gbodeTuning *best) {
    if (!w || !space || !group || !sp || maxc < 1 || !(dt > 0) || steps < 1 || !best) {
        set_error("gbodeWorldAutotune: bad argument");
        return 0;
    }
    if (!world_init_device(w)) return 0;
    // candidates: threads a block (the colour-group tile: 128 or 256 slots a
    // wave), staged rows a shared-memory buffer (400 or 800; the two-level
    // sweep stages its crossing rows in 128-row buffers), the two-level sweep
    // (off, or two interior passes), the residual check interval; and, as
    // before, half the blocks and two passes over a group's rows
    // and, with a residual target and momentum set (gbodeWorldSetSweepMomentum),
    // every candidate with and without it
    struct Cand { int blocks, passes, check, threads, chunk, two; float mom; };
    std::vector<Cand> cands;
    const int sms = num_sms();
    const bool resid = w->P.residual_target > 0;
    const float mom_set = w->P.momentum;
    std::vector<float> moms{mom_set};
    if (resid && mom_set > 0.f) moms.push_back(0.f);
    for (float mom : moms) {
        for (int threads : {256, 128})
            for (int two : {0, 2})
                for (int chunk : {800, 400}) {
                    if (two && chunk != 800) continue;
                    for (int check : {5, 10}) {
                        if (!resid && check != 5) continue;
                        cands.push_back({sms, 1, resid ? check : 0, threads, chunk, two, mom});
                    }
                }
        cands.push_back({sms / 2, 1, resid ? 5 : 0, 256, 800, 0, mom});
        cands.push_back({sms, 2, resid ? 5 : 0, 256, 800, 0, mom});
    }
    // every candidate starts from the same state: the device-side simulation
    // state (bodies, warm-start tables, joint multipliers, auto-disable state,
    // counters) is copied aside once and put back before each candidate and
    // at the end, so the world leaves the tuner as it entered it
    if (!world_upload(w)) return 0;
    if (!w->host_valid) world_download(w);
    DevSnapshot snap;
    auto restore = [&]() { snapshot_restore(w, snap); };
    auto release = [&]() { snap.release(); };
    // one plain step settles buffer sizes (a later reallocation would not be restored)
    const SolverParams saved = w->P;
    if (!gbodeWorldStepFused(w, space, group, sp, maxc, dt, 0)) return 0;
    if (cudaStreamSynchronize(w->stream) != cudaSuccess) return 0;
    if (!snapshot_save(w, snap)) { set_error("gbodeWorldAutotune: device allocation"); release(); return 0; }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int timing = w->timing;
    w->timing = false;
    float best_ms = INFINITY;
    int best_i = -1;
    for (size_t i = 0; i < cands.size(); i++) {
        restore();
        w->P.pgs_blocks = cands[i].blocks;
        w->P.pgs_passes = cands[i].passes;
        w->P.pgs_threads = cands[i].threads == 128 ? 128 : 0;
        w->P.pgs_chunk = cands[i].chunk;
        w->P.pgs_two_level = cands[i].two;
        w->P.momentum = cands[i].mom;
        if (resid) w->P.check_every = cands[i].check;
        std::vector<float> t;
        for (int k = 0; k < steps + 2; k++) {
            cudaEventRecord(e0, w->stream);
            if (!gbodeWorldStepFused(w, space, group, sp, maxc, dt, use_graph)) {
                w->P = saved;
                w->timing = timing;
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                restore();
                release();
                return 0;
            }
            cudaEventRecord(e1, w->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (k >= 2) t.push_back(ms);
        }
        std::nth_element(t.begin(), t.begin() + t.size() / 2, t.end());
        const float med = t[t.size() / 2];
        if (med < best_ms) { best_ms = med; best_i = (int)i; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    restore();
    release();
    w->P = saved;
    w->timing = timing;
    const Cand &c = cands[best_i];
    w->P.pgs_blocks = c.blocks >= sms ? 0 : c.blocks;
    w->P.pgs_passes = c.passes;
    w->P.pgs_threads = c.threads == 128 ? 128 : 0;
    w->P.pgs_chunk = c.chunk;
    w->P.pgs_two_level = c.two;
    w->P.momentum = c.mom;
    if (resid) w->P.check_every = c.check;
    best->momentum = c.mom;
    best->blocks = c.blocks;
    best->threads = c.threads;
    best->chunk_rows = c.chunk;
    best->two_level = c.two;
    best->passes = c.passes;
    best->check_every = c.check;
    best->ms_per_step = best_ms;
    best->candidates = (int)cands.size();
    return 1;
}

int gbodeWorldSaveSnapshot(dWorldID w) {
    if (!w) { set_error("gbodeWorldSaveSnapshot: no world"); return 0; }
    if (!world_init_device(w) || !world_upload(w)) return 0;
    if (!w->snapshot) w->snapshot = new DevSnapshot();
    if (!snapshot_save(w, *w->snapshot)) {
        w->snapshot->release();
        set_error("gbodeWorldSaveSnapshot: device allocation", cudaGetLastError());
        return 0;
    }
    return 1;
}

int gbodeWorldRestoreSnapshot(dWorldID w) {
    if (!w || !w->snapshot || !w->snapshot->valid) { set_error("gbodeWorldRestoreSnapshot: no snapshot"); return 0; }
    if (w->dev_dirty) {
        set_error("gbodeWorldRestoreSnapshot: the host changed the world since the snapshot");
        return 0;
    }
    if (!snapshot_restore(w, *w->snapshot)) {
        set_error("gbodeWorldRestoreSnapshot: the world's bodies or device buffers changed since the snapshot");
        return 0;
    }
    return 1;
}

void gbodeWorldDropSnapshot(dWorldID w) {
    if (w && w->snapshot) w->snapshot->release();
}

int gbodeSolveLCPBatch(int count, int n, const double *A, const double *b, const double *lo, const double *hi, int nub,
                       const int *findex, double *x, double *w) {
    if (count < 0 || n < 1 || n > GB_DANTZIG_MAX_ROWS || nub < 0 || nub > n || (count > 0 && (!A || !b || !x || !w)) ||
        (count > 0 && nub < n && (!lo || !hi))) {
        set_error("gbodeSolveLCPBatch: bad argument");
        return 0;
    }
    if (count == 0) return 1;
    std::vector<double> zl, zh;
    if (!lo || !hi) {  // all unbounded
        zl.assign((size_t)count * n, -INFINITY);
        zh.assign((size_t)count * n, INFINITY);
        lo = zl.data();
        hi = zh.data();
    }
    if (!solve_lcp_batch(count, n, A, b, lo, hi, nub, findex, x, w, 0)) {
        set_error("gbodeSolveLCPBatch: a problem did not solve (or device allocation failed)", cudaGetLastError());
        return 0;
    }
    return 1;
}

void gbodeWorldGetStepStats(dWorldID w, gbodeStepStats *out) {
    if (w->stats_pending) {
        cudaMemcpyAsync(w->ws.hc, w->ws.dc, sizeof(DevCounters), cudaMemcpyDeviceToHost, w->stream);
        cudaStreamSynchronize(w->stream);
        const DevCounters &h = *w->ws.hc;
        w->stats.contacts = h.step_contacts;
        w->stats.rows = h.nrows;
        w->stats.colours = h.ncolours;
        w->stats.iterations = h.iterations;
        w->stats.residual = h.resid;
        w->stats.sleeping = w->ws.sleep_on ? h.nasleep : 0;
        w->stats.interior_colours = h.nicolours;
        w->stats.interior_rows = h.slab_rows;
        w->stats.neighbour_waits = h.slab_sync;
        w->stats.cross_classes = h.split_k;
        w->stats.momentum = h.mom_final;
        w->stats.solve_ms = 0;
        w->stats.step_ms = 0;
        if (w->timing) {
            cudaEventElapsedTime(&w->stats.solve_ms, w->ev[0], w->ev[1]);
            cudaEventElapsedTime(&w->stats.step_ms, w->ev[2], w->ev[3]);
        }
        w->stats_pending = false;
    }
    *out = w->stats;
}

double gbodeWorldLastResidual(dWorldID w, double *complementarity, double *max_lambda) {
    return last_residual(w->ws, (int)w->bodies.size(), complementarity, max_lambda, w->stream);
}

int gbodeWorldGetLastRows(dWorldID w, float *rows, int cap) { return copy_last_rows(w->ws, rows, cap, w->stream); }

int gbodeWorldGetResidualHistory(dWorldID w, float *out, int cap) {
    if (!w->ws.dc) return 0;
    cudaMemcpyAsync(w->ws.hc, w->ws.dc, sizeof(DevCounters), cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    int n = w->ws.hc->nhist;
    if (out) for (int i = 0; i < n && i < cap; i++) out[i] = w->ws.hc->rhist[i];
    return n;
}

int gbodeWorldGetResidualSweeps(dWorldID w, int *out, int cap) {
    if (!w->ws.dc) return 0;
    cudaMemcpyAsync(w->ws.hc, w->ws.dc, sizeof(DevCounters), cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    int n = w->ws.hc->nhist;
    if (out) for (int i = 0; i < n && i < cap; i++) out[i] = w->ws.hc->rsweep[i];
    return n;
}

int gbodeWorldGetContacts(dWorldID w, float *out, int cap) {
    if (!w->ws.dc) return 0;
    int n = 0;
    cudaMemcpyAsync(&n, &w->ws.dc->ncontacts, 4, cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    if (!out || cap <= 0 || n <= 0) return n;
    int k = n < cap ? n : cap;
    std::vector<Contact> C(k);
    cudaMemcpyAsync(C.data(), w->ws.contacts.p, (size_t)k * sizeof(Contact), cudaMemcpyDeviceToHost, w->stream);
    cudaStreamSynchronize(w->stream);
    for (int i = 0; i < k; i++) {
        float *o = out + 12 * i;
        o[0] = C[i].pos_depth.x; o[1] = C[i].pos_depth.y; o[2] = C[i].pos_depth.z;
        o[3] = C[i].normal.x; o[4] = C[i].normal.y; o[5] = C[i].normal.z;
        o[6] = C[i].pos_depth.w;
        o[7] = (float)C[i].g1; o[8] = (float)C[i].g2; o[9] = (float)C[i].b1; o[10] = (float)C[i].b2;
        o[11] = (float)C[i].slot;
    }
    return n;
}

}  // extern "C"

// dBoxBox on the device through a one-pair narrow phase of two boxes
extern "C" int dBoxBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2, const dMatrix3 R2,
                       const dVector3 side2, dVector3 normal, dReal *depth, int *return_code, int flags,
                       dContactGeom *contact, int skip) {
    if (!g_default_world) g_default_world = dWorldCreate();
    dxWorld *w = g_default_world;
    if (!world_init_device(w)) return 0;
    std::vector<GeomHost> gh(2);
    const float *pp[2] = {p1, p2}, *RR[2] = {R1, R2}, *ss[2] = {side1, side2};
    for (int k = 0; k < 2; k++) {
        gh[k].cls = dBoxClass;
        gh[k].body = -1;
        gh[k].dims[0] = ss[k][0]; gh[k].dims[1] = ss[k][1]; gh[k].dims[2] = ss[k][2]; gh[k].dims[3] = 0;
        memcpy(gh[k].pos, pp[k], 12);
        gh[k].pos[3] = 0;
        memcpy(gh[k].R, RR[k], 48);
    }
    if (!ensure_bodies(w->ws, 1) || !upload_geoms(w->ws, gh, w->stream)) return 0;
    w->uploaded_space = nullptr;
    launch_pose_aabb(w->ws, bodies_view(w->ws, 0), 2, -1000, 1000, w->stream);
    int pr[2] = {0, 1};
    std::vector<float> out;
    std::vector<int> counts;
    if (narrow_pairs_host(w->ws, pr, 1, flags & 0xffff, out, counts, w->stream) < 0) return 0;
    int n = counts.empty() ? 0 : counts[0];
    int code = 0;
    cudaMemcpy(&code, w->ws.c_code.p, 4, cudaMemcpyDeviceToHost);
    // dCollideBoxBox negates dBoxBox's normal (box.cpp:758-760); undo it here
    for (int i = 0; i < n; i++) {
        dContactGeom *c = (dContactGeom *)((char *)contact + (size_t)i * skip);
        const float *o = &out[8 * i];
        c->pos[0] = o[0]; c->pos[1] = o[1]; c->pos[2] = o[2];
        c->depth = o[6];
    }
    if (n > 0) {
        normal[0] = -out[3]; normal[1] = -out[4]; normal[2] = -out[5];
        *depth = 0;
        for (int i = 0; i < n; i++) if (out[8 * i + 6] > *depth) *depth = out[8 * i + 6];
        *return_code = code;
    }
    return n;
}
