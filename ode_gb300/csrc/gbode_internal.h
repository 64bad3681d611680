// Host-side context shared by the C-ABI layer (api.cpp) and the kernel
// launchers (collide.cu, solve.cu).  Device buffers are owned here and grown
// on demand; every launcher enqueues on the world's stream without host syncs
// unless its comment says otherwise.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "gbode_device.cuh"

namespace gb {

// Grow-only device buffer.
struct DBuf {
    void *p = nullptr;
    size_t bytes = 0;
    bool ensure(size_t want);  // false on allocation failure
    template <class T> T *as() const { return (T *)p; }
    void release();
};

struct SolverParams {
    float dt;
    float gravity[3];
    float erp, cfm, w;
    float max_vel, min_depth;
    int iterations;
    // ODE dynamic iteration parameters (objects.h:451-475)
    float premature_delta, extra_factor, extra_delta;
    // residual-target mode
    float residual_target;
    int check_every, max_iterations;
    int warm_mode;
    float warm_scale;
    int solver;  // GBODE_SOLVER_*
    int learned;        // learned warm start (MLP prediction, residual-judged against the plain start)
    int learn_capture;  // record the per-contact features of each step
    int pgs_blocks;     // thread blocks of the coloured solver (0: one per SM)
    int pgs_passes;     // passes over a manifold's rows per visit (0 or 1: one)
    int pgs_two_level;  // two-level sweep: parts' interior groups in shared memory, cross groups coloured globally
    int pgs_threads;    // threads a block of the sweep kernels: 128 or 256 (0: 256)
    int pgs_chunk;      // staged rows a shared-memory buffer of the one-level sweep (0: GB_CHUNK_ROWS)
    int pgs_grid_sync;  // two-level sweep: 1 every cross colour ends at a grid barrier; 0 a block waits only
                        // for the blocks that touch the same bodies (GBODE_SYNC_*)
    int fixed_checks;   // residual-target mode: 1 a check every check_every sweeps; 0 predicted checks
    int pgs_split;      // two-level sweep: cross colours merged into this many classes, each relaxed as one
                        // step with mass splitting (0: every cross colour its own step)
    int reform_every;   // residual-target mode: sweeps between re-formed accumulators (0: 500)
    float momentum;     // coloured solvers: momentum between sweeps (0: off; see k_pgs)
};

// learned warm start network (parameter layout in mlp.cu)
#define GB_MLP_IN 12
#define GB_MLP_HIDDEN 128
#define GB_MLP_OUT 3
#define GB_MLP_NPARAMS (2 * GB_MLP_IN + GB_MLP_HIDDEN * GB_MLP_IN + GB_MLP_HIDDEN + \
                        2 * (GB_MLP_HIDDEN * GB_MLP_HIDDEN + GB_MLP_HIDDEN) + GB_MLP_OUT * GB_MLP_HIDDEN + GB_MLP_OUT)

// Device-side scalars the kernels read and write (one pinned/device block).
struct DevCounters {
    int npairs;        // candidate pairs of the broad phase
    int ncontacts;     // contacts
    int nrows;         // constraint rows
    int nmanifolds;    // contact groups
    int ncolours;      // colours used
    int iterations;    // sweeps performed
    unsigned err;      // ERR_* bits
    int uncoloured;    // colouring progress
    float resid;       // last FP32 relative residual
    float maxlam;      // last max |lambda|
    int nbig;          // geoms in the big-box list
    int maxlevel;      // coarsest hash level in use
    int narrow_total;  // contacts produced by the last narrow phase
    int cells_total;   // scan scratch (hash cells)
    int colour_total;  // scan scratch (colours)
    float racc[4];     // residual / max|lambda| accumulators, two parities
    int step_contacts; // contacts of the last dWorldQuickStep (survives dJointGroupEmpty)
    int nhist;         // residual checks recorded in rhist by the last solve
    float rhist[256];  // FP32 relative residual at each check of the last solve
    GridSync gsync;    // grid barrier state (zeroed before cooperative launches)
    float learn_stats[4];  // last learned start: MLP start used (1/0), its residual, the plain start's residual
    int ncmanifolds;       // contact manifolds (the first groups; ball/hinge joints follow)
    int nrows_contacts;    // rows of the contacts (joint rows follow)
    int njoint_rows;       // scan scratch (joint rows)
    int warm_parity;       // which warm-start table holds the previous step
    int nawake;            // contacts of awake components (the solver's contacts when sleeping is on)
    int nwaves;            // staging waves of the coloured solver
    int nasleep;           // bodies not stepped (their component sleeps)
    int nicolours;         // two-level sweep: colours of the parts' interior groups
    int slab_box[4];       // two-level sweep: body x / y range (order-preserving ints)
    int slab_rows;         // two-level sweep: interior rows of the last solve
    int slab_nbr_over;     // two-level sweep: a body had more cross accessors than listed (grid barriers used)
    int slab_sync;         // the last solve's two-level sweep waited on neighbour blocks (1) or grid barriers (0)
    int split_off;         // two-level sweep: a cross group cannot be relaxed in a split class (exact colours)
    int split_k;           // two-level sweep: classes of the last solve's cross phase with mass splitting (0: off)
    int mom_off;           // two-level sweep: a group touches a body outside the columns' lists (no momentum)
    float mom_final;       // momentum of the last solve's last sweeps (0: off)
    int rsweep[256];       // sweeps done at each residual check of the last solve (rhist's checks)
};

// auto-disable state per body, int4: x flags, y idle steps, z steps left,
// w average samples; float4: squared linear / angular thresholds, idle time,
// time left.  Flags: bit 0 auto-disable on, bit 1 disabled, bit 2 the
// velocity ring buffer is full, bits 8-23 the ring buffer's next slot.
#define GB_ADIS_ON 1
#define GB_ADIS_DISABLED 2
#define GB_ADIS_READY 4

struct Workspace {
    // geoms
    DBuf g_cls, g_body, g_dims, g_spos, g_sR, g_pos, g_R, g_amin, g_amax, g_level, g_dblo, g_dbhi, g_big;
    // broad phase
    DBuf h_keys, h_count, h_start, h_fill, h_members, h_entry, p_count, p_start, pairs;
    DBuf p_cache;  // broad phase: each geom's first partners, kept by the counting pass
    // narrow phase
    DBuf c_slots, c_count, c_start, contacts, surfaces, c_mcount, c_rstart, c_code;
    DBuf n_perm, n_key;  // narrow phase: pairs grouped by collider class, counts and fills per class
    // bodies
    DBuf b_pos, b_q, b_R, b_lvel, b_avel, b_facc, b_tacc, b_Ib, b_invIb, b_invIw, b_fc, b_rt, b_fa;
    DBuf b_damp, b_maxw;  // damping (scales, squared thresholds), angular speed cap
    // sleeping: auto-disable state and velocity ring buffers (adis_S samples a
    // body), per-step components, and the contacts of awake components
    DBuf b_adis_i, b_adis_f, b_adis_buf, b_touch, b_parent, b_awake, b_asleep, c_keep, c_kpos, c_awake, c_orig;
    int adis_S = 1;
    bool sleep_on = false;  // some body has auto-disable on or is disabled
    bool sleep_precomputed = false;  // the caller ran the sleep stage of this step already
    bool use_awake = false;          // the solver of this step reads c_awake / dc->nawake
    // rows
    DBuf r_J1l, r_J1a, r_J2l, r_J2a, r_M1l, r_M1a, r_M2l, r_M2a, r_lambda, r_Ad, r_findex, r_contact, r_body;
    // colouring / schedule
    DBuf m_head, m_id, m_start, m_colour, m_mask, m_claim, m_tent, col_count, col_start, col_fill, col_list, m_desc, p_rows, chunk_rows, chunk_start;
    DBuf wv_count, wv_base, wv_col, wv_sched;  // staging waves: per (colour, block) count and first; per wave colour, slots
    // two-level sweep: body weights, parts, per-part body lists and counts,
    // group classes and descriptors, per-(part, colour) interior lists, the
    // interior rows packed part by part, partition histograms
    DBuf s_bw, s_part, s_blocal, s_pbcount, s_pbody, s_prow, s_pgrp, s_gpart, s_gdesc;
    DBuf s_pccount, s_pcstart, s_pcfill, s_ilist, s_irown, s_irowoff, s_idesc, s_ipack, s_hist, s_binpart;
    // two-level sweep, neighbour waits: cross groups per (colour, owner block) and their first slot, the
    // owner blocks touching each body, block adjacency bit sets, per-block step counters
    DBuf x_cnt, x_start, x_fill, x_accn, x_acc, x_adj, x_prog;
    // two-level sweep, split classes: groups per (class, body), fixed-point accumulators per (class, body)
    DBuf x_nsplit, x_dacc, x_smask;
    // momentum between sweeps: every row's multiplier after the previous sweep, every body's accumulators
    DBuf m_lprev, b_fcprev;
    // learned warm start
    DBuf l_feat, l_scale, l_pred, l_alt, mlp_P, mlp_wb;
    // ball and hinge joints (uploaded when they change) and per-step joint state
    DBuf j_info, j_a1, j_a2, j_x1, j_x2, j_qrel, j_l0, j_l1, j_l2, j_m, j_rstart, j_limit, j_lerr, j_lam;
    DBuf j_v1, j_v2, j_m0, j_m1, j_m2;  // hinge2: angle vectors (+ s0, c0), axis-2 motor, suspension
    DBuf grp_body;  // body pair of every constraint group (contact manifolds, then joints)
    DBuf j_pairs;   // set of jointed body pairs (fused narrow phase skips them)
    unsigned j_pair_mask = 0;
    int njoints = 0;
    int rows_per_contact = 6;  // row capacity per contact: 3, or 6 when a surface uses rolling friction
    // reference-order schedule
    DBuf i_order, i_start, i_bodies, i_bstart, i_normals;
    // dense island solves (dWorldStep): scratch offsets, FP64 and int scratch, row -> island index
    DBuf d_off, d_scr, d_iscr, d_rloc;
    // warm start cache (previous step)
    DBuf w_keys, w_lambda, w_keys_prev, w_lambda_prev;
    // residual
    DBuf res_f, res_v;
    // scan scratch
    DBuf scan_tmp;
    unsigned warm_mask = 0;      // table size - 1 (power of two)
    bool warm_valid = false;     // the previous-step table was filled
    DevCounters *dc = nullptr;   // device counters
    DevCounters *hc = nullptr;   // pinned host mirror
    int pair_cap = 0, contact_cap = 0, row_cap = 0;
    void release();
};

// ---- fault injection for the error-path tests (gbodeTestInject; host-side
// state, consumed by the next launch it applies to).  Nothing faults: a
// barrier counter starts one arrival short or a staging wait names a copy
// that is never issued (bounded waits run out and report), allocations fail
// as cudaMalloc failing would, and capacities the kernels see are lowered
// below what is allocated (the kernels clamp and report).
struct TestFaults {
    int barrier = 0;      // next solver launch: grid barrier counter one arrival short
    int stage = 0;        // next solver launch: its first staging wait names a copy never issued
    int alloc_skip = -1;  // device allocations that still succeed (-1: injection off)
    int alloc_fail = 0;   // then this many fail
    int contact_cap = 0;  // contact capacity the narrow phase sees (0: the allocated one)
    int row_cap = 0;      // row capacity the contact assembly sees (0: the allocated one; worlds without joints)
    int colour_cap = 0;   // colours the colouring may use (0: all)
};
extern TestFaults g_test;

// ---- scan (scan.cu): exclusive prefix sum of n ints (n read from *n_dev if
// non-null, else n_host), writing the total to *total_dev.
void scan_exclusive(const int *in, int *out, const int *n_dev, int n_cap, int *total_dev, Workspace &ws,
                    cudaStream_t s);

// ---- collide.cu
struct GeomHost {
    int cls, body;
    float dims[4];
    float pos[4];
    float R[12];
};
// upload geoms (class/body/dims/static pose) into the workspace
bool upload_geoms(Workspace &ws, const std::vector<GeomHost> &g, cudaStream_t s);
// pose geoms from bodies, AABBs, levels (one launch)
void launch_pose_aabb(Workspace &ws, const Bodies &b, int ng, int minlevel, int maxlevel, cudaStream_t s);
// hash-space broad phase into ws.pairs (device count in dc->npairs); exact = 1
// reports every AABB-overlapping pair, 0 reproduces the reference's pair set
bool launch_broadphase(Workspace &ws, int ng, int exact, cudaStream_t s);
// narrow phase on the pair list; contacts compacted into ws.contacts with
// surface index `surf`; codes (dBoxBox return_code, -1 n/a) optional per slot
bool launch_narrowphase(Workspace &ws, int maxc, int surf, bool append, cudaStream_t s);
// narrow phase on an explicit host pair list; results copied back (syncs)
int narrow_pairs_host(Workspace &ws, const int *pairs, int np, int maxc, std::vector<float> &out,
                      std::vector<int> &counts, cudaStream_t s);

// ---- solve.cu
Bodies bodies_view(Workspace &ws, int nb);
bool ensure_bodies(Workspace &ws, int nb);
bool ensure_rows(Workspace &ws, int ncontacts_cap, int njoints = 0);
// full quickstep on the device contact list (count in dc->ncontacts)
bool launch_quickstep(Workspace &ws, int nb, int nsurf, const SolverParams &P, cudaStream_t s,
                      cudaEvent_t ev_solve0, cudaEvent_t ev_solve1);
// reference-order quickstep with a host-built island schedule
struct IslandSchedule {
    std::vector<int> order;       // rows in island order, findex<0 rows first per island
    std::vector<int> start;       // island row ranges [nisl+1]
    std::vector<int> bodies;      // bodies per island in DFS order
    std::vector<int> bstart;      // [nisl+1]
    std::vector<int> normals;     // per island: count of findex<0 rows
};
bool launch_quickstep_islands(Workspace &ws, int nb, const SolverParams &P, const IslandSchedule &sch,
                              cudaStream_t s, cudaEvent_t ev_solve0, cudaEvent_t ev_solve1);
// FP64 residual of the last step's rows (syncs)
double last_residual(Workspace &ws, int nb, double *compl_err, double *maxlam, cudaStream_t s);
int copy_last_rows(Workspace &ws, float *rows, int cap, cudaStream_t s);
int learn_samples(Workspace &ws, float *out, int cap, cudaStream_t s);
// ball/hinge/hinge2 joint table: src = info, anchor1, anchor2, axis1, axis2, qrel, limot 0-2,
// hinge2 v1(+s0), v2(+c0), second limot 0-2 (n each)
bool joint_table_upload(Workspace &ws, int n, const std::vector<const void *> &src, cudaStream_t s);
// joint feedback (f1 t1 f2 t2, 16 floats a record; word 3 = 1 when solved) of the
// last step into a host array: the ncontacts contacts, then the njoints
// ball/hinge/hinge2 joints of the joint table (syncs)
void joint_feedback(Workspace &ws, int ncontacts, int njoints, std::vector<float> &out, cudaStream_t s);

// ---- dantzig.cu: dWorldStep's dense LCP per island (rows: island by island
// in `order`, island k = order[start[k] .. start[k+1])), fc accumulated for the
// islands' bodies; syncs
#define GB_DANTZIG_MAX_ROWS 2048
bool launch_dantzig(Workspace &ws, const std::vector<int> &order, const std::vector<int> &start, cudaStream_t s);
// a batch of dense LCPs from host arrays (gbodeSolveLCPBatch; syncs)
bool solve_lcp_batch(int count, int n, const double *A, const double *b, const double *lo, const double *hi,
                     int nub, const int *findex, double *x, double *w, cudaStream_t s);
// solve.cu entry points the step drivers share: the rows of a step (body pass,
// contact and joint rows), the integration, and the rows' view
bool assemble_step(Workspace &ws, int nb, const SolverParams &P, cudaStream_t s);
bool launch_integrate(Workspace &ws, int nb, const SolverParams &P, cudaStream_t s);
Rows rows_view_public(Workspace &ws);
int download_solver_contacts(Workspace &ws, std::vector<int2> &bodies, std::vector<int> &rstart,
                             std::vector<int> &mcount, cudaStream_t s);

// ---- sleep.cu: auto-disable state buffers; the sleep stage of a step
bool ensure_sleep(Workspace &ws, int nb, int samples);
bool launch_sleep(Workspace &ws, int nb, float h, cudaStream_t s);

// launch bookkeeping
void count_launch(int n = 1);
int num_sms();
void launch_set_surface(Workspace &ws, const Surface &v, cudaStream_t s);
// records the message gbodeGetLastError() returns on this thread
void report_error(const char *msg);
// learned warm start network (mlp.cu)
bool mlp_pack(const float *P_dev, unsigned char *wb_dev, cudaStream_t s);
bool mlp_infer(const unsigned char *wb_dev, const float *X, int n_host, const int *n_dev, float *Y, unsigned *err,
               cudaStream_t s);
size_t mlp_wb_bytes();

}  // namespace gb
