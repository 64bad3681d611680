/* CPU restatement of the reference's rigid-body hot path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the GPU path and the
 * CPU baseline that bench.py times beside it; no product code includes,
 * links or calls it.  It restates, in plain C and float arithmetic evaluated
 * in the reference's order (compile with -ffp-contract=off), the algorithms of:
 *   collision_kernel.cpp:292-338   dCollide dispatch and reversal
 *   sphere.cpp, box.cpp, capsule.cpp, collision_util.cpp   the colliders
 *   collision_space.cpp:287-614    dHashSpace broad phase (callback order)
 *   joints/contact.cpp:49-347      contact rows (getInfo1/getInfo2)
 *   util.cpp:583-860               dxStepBody and island construction
 *   quickstep.cpp                  SOR-LCP island solver
 *   misc.cpp:35-135                dRand / dRandInt (row shuffling)
 * Its parity with the reference is pinned by the .npz fixtures in tests/golden, which the
 * reference itself produced (tests/golden/make_golden.py).
 */
#ifndef ODE_PORT_H
#define ODE_PORT_H
#ifdef __cplusplus
extern "C" {
#endif

enum { PORT_SPHERE = 0, PORT_BOX = 1, PORT_CAPSULE = 2, PORT_PLANE = 4 };

/* dCollide: out is [8][8] floats per contact: pos(3) normal(3) depth swap(1: g1 is o2). */
int port_collide(int cls1, const float *pos1, const float *R1, const float *dims1,
                 int cls2, const float *pos2, const float *R2, const float *dims2,
                 int flags, float *out);
/* dBoxBox return_code (0 when no contact). */
int port_boxbox_code(const float *p1, const float *R1, const float *s1,
                     const float *p2, const float *R2, const float *s2, int flags);

/* dHashSpace::collide over static geoms.  order = space list order (geom
 * indices, first = head).  pairs receives (o1,o2) in callback order.
 * Returns the number of pairs (may exceed cap; only cap are written). */
int port_hash_pairs(int n, const int *cls, const int *body, const float *pos, const float *R,
                    const float *dims, const int *order, int minlevel, int maxlevel,
                    int *pairs, int cap);

typedef struct port_world port_world;
/* bodies_in: [nb][20] pos q lvel avel mass I11 I22 I33 I12 I13 I23.
 * params: dt gx gy gz erp cfm w max_vel min_depth. reorder: 0 none, 1 random (dRandInt). */
port_world *port_world_create(int nb, const float *bodies_in, const float *params, int iterations,
                              int dyn_enabled, int reorder);
void port_world_destroy(port_world *w);
void port_world_get(const port_world *w, float *out /* [nb][25] pos q R lvel avel */);
void port_world_set_state(port_world *w, const float *state /* [nb][25] */);
void port_world_set_dyn(port_world *w, float premature_delta, float extra_factor, float extra_delta);
/* SOR sweeps on `threads` host threads for islands of at least `min_rows`
 * rows (the reference's opt-in multi-threaded stepping); the multipliers stay
 * those of the single-threaded sweep, to the bit. */
void port_world_set_threads(port_world *w, int threads, int min_rows);
void port_rand_set_seed(unsigned long s);
unsigned long port_rand_get_seed(void);
/* One dWorldQuickStep with the given contact joints attached in order.
 * cb [nc][2] body indices (-1 = none), mode [nc], cs [nc][16] as tests/golden.
 * lambda [nc][3] receives the per-row multipliers (0 for absent rows).
 * rows_out (optional) receives the constraint rows as formed before Ad
 * scaling, in island order: per row J1(6) J2(6) rhs cfm lo hi b1 b2 findex
 * lambda (20 floats; world body indices, global row index for findex), for
 * the residual evaluator. */
int port_world_quickstep(port_world *w, int nc, const int *cb, const int *mode, const float *cs,
                         float *lambda, float *rows_out, int *nrows_out);

typedef struct port_sim port_sim;
/* Full user loop over a hash space: geoms [ng] cls, body (-1 static), pos, R,
 * dims; surface: mu mu2 bounce bounce_vel soft_erp soft_cfm. */
port_sim *port_sim_create(port_world *w, int ng, const int *cls, const int *body, const float *pos,
                          const float *R, const float *dims, int minlevel, int maxlevel, int maxc,
                          int mode, const float *surface);
void port_sim_destroy(port_sim *s);
/* dSpaceCollide(near callback: dCollide + dJointCreateContact + dJointAttach),
 * dWorldQuickStep, dJointGroupEmpty.  Returns the number of contacts. */
int port_sim_step(port_sim *s);
/* Contacts made in the last step: cb [nc][2], cs [nc][16] (pos normal depth ...). */
int port_sim_last_contacts(const port_sim *s, int *cb, float *cs, int cap);

/* Evaluate each step's FP64 natural-map LCP residual (the definition of
 * port_lcp_residual, over the step's unscaled rows) while stepping. */
void port_world_set_residual(port_world *w, int on);
/* Of the last port_sim_step: seconds of collision (geom poses, hash space,
 * contacts) and of the quickstep, the step's residual (with
 * port_world_set_residual on; else 0) and max |lambda|. */
void port_sim_last_stats(const port_sim *s, double *out4);
/* The residual and max |lambda| of the world's last quickstep (residual on). */
void port_world_last_residual(const port_world *w, double *out2);

/* port_world_quickstep that also writes, for every recorded row (rows_out
 * order: islands in the reference's order), 3 * contact index + the row's
 * place in its contact (0 normal, 1 and 2 friction) to row_slot [m].  Not
 * thread-safe (test use). */
int port_world_quickstep_map(port_world *w, int nc, const int *cb, const int *mode, const float *cs, float *lambda,
                             float *rows_out, int *nrows_out, int *row_slot);

/* FP64 LCP residual of a solution lambda (per row, [m]) for rows in the
 * layout of port_world_quickstep's rows_out, with the body inverse masses / world-frame
 * inverse inertias (invm [nb], invI [nb][9]).  Returns the natural-map
 * residual max_i |lambda_i - proj(lambda_i - (A lambda - b)_i / A_ii)|
 * (unnormalised) and writes the min-map complementarity error
 * max_i max(min(lambda_i - lo_i, w_i+ / A_ii), min(hi_i - lambda_i, w_i- / A_ii)),
 * w = A lambda - b (unnormalised, in the units of lambda). */
double port_lcp_residual(int m, const float *rows, int nb, const double *invm, const double *invI,
                         const float *lambda, double *compl_err);

#ifdef __cplusplus
}
#endif
#endif
