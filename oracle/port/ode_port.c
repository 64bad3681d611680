/* CPU restatement of the reference's rigid-body hot path -- the oracle.
 * TEST INFRASTRUCTURE ONLY (see ode_port.h).  Every function cites the
 * reference file:line it restates.  Float expressions keep the reference's
 * evaluation order; build with -O2 -ffp-contract=off (no fast-math). */
#include "ode_port.h"

#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef float real;
#define R0 0.0f
#define INF ((float)INFINITY)
#define NUMC_MASK 0xffff

/* ------------------------------------------------------------------ math */
/* include/ode/odemath.h:120-420 (dot/cross/multiply helpers) */
static inline real dot3(const real *a, const real *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline real dot3_41(const real *a, const real *b) { return a[0] * b[0] + a[4] * b[1] + a[8] * b[2]; }
static inline real dot3_14(const real *a, const real *b) { return a[0] * b[0] + a[1] * b[4] + a[2] * b[8]; }
static inline real dot3_44(const real *a, const real *b) { return a[0] * b[0] + a[4] * b[4] + a[8] * b[8]; }
static inline void cross3(real *r, const real *a, const real *b) {
    real r0 = a[1] * b[2] - a[2] * b[1];
    real r1 = a[2] * b[0] - a[0] * b[2];
    real r2 = a[0] * b[1] - a[1] * b[0];
    r[0] = r0; r[1] = r1; r[2] = r2;
}
static inline void mul0_331(real *r, const real *a, const real *b) {
    real r0 = dot3(a, b), r1 = dot3(a + 4, b), r2 = dot3(a + 8, b);
    r[0] = r0; r[1] = r1; r[2] = r2;
}
static inline void mul1_331(real *r, const real *a, const real *b) {
    real r0 = dot3_41(a, b), r1 = dot3_41(a + 1, b), r2 = dot3_41(a + 2, b);
    r[0] = r0; r[1] = r1; r[2] = r2;
}
/* dMultiply0_333: res row i = (row i of a) * b */
static inline void mul0_333(real *r, const real *a, const real *b) {
    for (int i = 0; i < 3; i++) {
        real t0 = dot3_41(b, a + 4 * i), t1 = dot3_41(b + 1, a + 4 * i), t2 = dot3_41(b + 2, a + 4 * i);
        r[4 * i] = t0; r[4 * i + 1] = t1; r[4 * i + 2] = t2;
    }
}
/* dMultiply2_333: res = a * b^T */
static inline void mul2_333(real *r, const real *a, const real *b) {
    for (int i = 0; i < 3; i++) {
        real t0 = dot3(b, a + 4 * i), t1 = dot3(b + 4, a + 4 * i), t2 = dot3(b + 8, a + 4 * i);
        r[4 * i] = t0; r[4 * i + 1] = t1; r[4 * i + 2] = t2;
    }
}
static inline real length3(const real *a) { return sqrtf(dot3(a, a)); }
static inline real dist3(const real *a, const real *b) {
    real t[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return length3(t);
}

/* odemath.cpp:95-165 dxSafeNormalize3 and odemath.h:36-46 dxNormalize3 */
static void normalize3(real *a) {
    real a0 = fabsf(a[0]), a1 = fabsf(a[1]), a2 = fabsf(a[2]);
    int idx;
    if (a1 > a0) idx = (a2 > a1) ? 2 : 1;
    else if (a2 > a0) idx = 2;
    else {
        if (!(a0 > R0)) { a[0] = 1.0f; a[1] = a[2] = 0.0f; return; }
        idx = 0;
    }
    if (idx == 0) {
        real rc = 1.0f / a0, x1 = a[1] * rc, x2 = a[2] * rc;
        real l = 1.0f / sqrtf(1.0f + x1 * x1 + x2 * x2);
        a[1] = x1 * l; a[2] = x2 * l; a[0] = copysignf(l, a[0]);
    } else if (idx == 1) {
        real rc = 1.0f / a1, x0 = a[0] * rc, x2 = a[2] * rc;
        real l = 1.0f / sqrtf(1.0f + x0 * x0 + x2 * x2);
        a[0] = x0 * l; a[2] = x2 * l; a[1] = copysignf(l, a[1]);
    } else {
        real rc = 1.0f / a2, x0 = a[0] * rc, x1 = a[1] * rc;
        real l = 1.0f / sqrtf(1.0f + x0 * x0 + x1 * x1);
        a[0] = x0 * l; a[1] = x1 * l; a[2] = copysignf(l, a[2]);
    }
}
/* odemath.cpp:200-218 dxSafeNormalize4 + odemath.h:48-57 */
static void normalize4(real *a) {
    real l = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3];
    if (l > 0) {
        l = 1.0f / sqrtf(l);
        a[0] *= l; a[1] *= l; a[2] *= l; a[3] *= l;
    } else {
        a[0] = 1; a[1] = a[2] = a[3] = 0;
    }
}
/* odemath.cpp:224-251 dxPlaneSpace */
static void plane_space(const real *n, real *p, real *q) {
    if (fabsf(n[2]) > (real)M_SQRT1_2) {
        real a = n[1] * n[1] + n[2] * n[2];
        real k = 1.0f / sqrtf(a);
        p[0] = 0; p[1] = -n[2] * k; p[2] = n[1] * k;
        q[0] = a * k; q[1] = -n[0] * p[2]; q[2] = n[0] * p[1];
    } else {
        real a = n[0] * n[0] + n[1] * n[1];
        real k = 1.0f / sqrtf(a);
        p[0] = -n[1] * k; p[1] = n[0] * k; p[2] = 0;
        q[0] = -n[2] * p[1]; q[1] = n[2] * p[0]; q[2] = a * k;
    }
}
/* rotation.cpp:236-254 dRfromQ */
static void r_from_q(real *R, const real *q) {
    real qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
    R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]); R[3] = 0;
    R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]); R[7] = 0;
    R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2; R[11] = 0;
}
/* include/ode/odemath.h:444-500 dCalcMatrix3Det / dInvertMatrix3 */
static real invert3(real *dst, const real *ma) {
    real det = ma[0] * (ma[5] * ma[10] - ma[9] * ma[6]) - ma[1] * (ma[4] * ma[10] - ma[8] * ma[6]) +
               ma[2] * (ma[4] * ma[9] - ma[8] * ma[5]);
    if (det == 0) return 0;
    real r = 1.0f / det;
    dst[0] = (ma[5] * ma[10] - ma[6] * ma[9]) * r;
    dst[1] = (ma[9] * ma[2] - ma[1] * ma[10]) * r;
    dst[2] = (ma[1] * ma[6] - ma[5] * ma[2]) * r;
    dst[4] = (ma[6] * ma[8] - ma[4] * ma[10]) * r;
    dst[5] = (ma[0] * ma[10] - ma[8] * ma[2]) * r;
    dst[6] = (ma[4] * ma[2] - ma[0] * ma[6]) * r;
    dst[8] = (ma[4] * ma[9] - ma[8] * ma[5]) * r;
    dst[9] = (ma[8] * ma[1] - ma[0] * ma[9]) * r;
    dst[10] = (ma[0] * ma[5] - ma[1] * ma[4]) * r;
    return det;
}

/* ------------------------------------------------------------- random */
/* misc.cpp:35-49 dRand and misc.cpp:78-135 dRandInt */
static uint32_t g_seed = 0;
void port_rand_set_seed(unsigned long s) { g_seed = (uint32_t)s; }
unsigned long port_rand_get_seed(void) { return g_seed; }
static uint32_t port_rand(void) {
    g_seed = (uint32_t)(1664525u * g_seed + 1013904223u);
    return g_seed;
}
static int port_rand_int(int n) {
    uint32_t r = port_rand(), un = (uint32_t)n;
    int result;
    if (un <= 0x10u) {
        r ^= (r >> 16); r ^= (r >> 8); r ^= (r >> 4);
        if (un <= 0x2u) {
            r ^= (r >> 2); r ^= (r >> 1);
            result = (int)(r & (un >> 1));
        } else if (un <= 0x4u) {
            r ^= (r >> 2);
            result = (int)(((r & 0x3u) * un) >> 2);
        } else {
            result = (int)(((r & 0xFu) * un) >> 4);
        }
    } else if (un <= 0x100u) {
        r ^= (r >> 16); r ^= (r >> 8);
        result = (int)(((r & 0xFFu) * un) >> 8);
    } else if (un <= 0x10000u) {
        r ^= (r >> 16);
        result = (int)(((r & 0xFFFFu) * un) >> 16);
    } else {
        result = (int)(((uint64_t)r * un) >> 32);
    }
    return result;
}

/* ------------------------------------------------------------- colliders */
typedef struct { int cls; real pos[4]; real R[12]; real dims[4]; } pgeom;
typedef struct { real pos[4]; real normal[4]; real depth; int swap; } pcontact;

/* collision_util.cpp:38-67 dCollideSpheres */
static int collide_spheres(const real *p1, real r1, const real *p2, real r2, pcontact *c) {
    real d = dist3(p1, p2);
    if (d > (r1 + r2)) return 0;
    if (d <= 0) {
        c->pos[0] = p1[0]; c->pos[1] = p1[1]; c->pos[2] = p1[2];
        c->normal[0] = 1; c->normal[1] = 0; c->normal[2] = 0;
        c->depth = r1 + r2;
    } else {
        real d1 = 1.0f / d;
        c->normal[0] = (p1[0] - p2[0]) * d1;
        c->normal[1] = (p1[1] - p2[1]) * d1;
        c->normal[2] = (p1[2] - p2[2]) * d1;
        real k = 0.5f * (r2 - r1 - d);
        c->pos[0] = p1[0] + c->normal[0] * k;
        c->pos[1] = p1[1] + c->normal[1] * k;
        c->pos[2] = p1[2] + c->normal[2] * k;
        c->depth = r1 + r2 - d;
    }
    return 1;
}

/* collision_util.cpp:70-95 dLineClosestApproach */
static void line_closest_approach(const real *pa, const real *ua, const real *pb, const real *ub,
                                  real *alpha, real *beta) {
    real p[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    real uaub = dot3(ua, ub), q1 = dot3(ua, p), q2 = -dot3(ub, p);
    real d = 1 - uaub * uaub;
    if (d <= 0.0001f) { *alpha = 0; *beta = 0; }
    else {
        d = 1.0f / d;
        *alpha = (q1 + uaub * q2) * d;
        *beta = (uaub * q1 + q2) * d;
    }
}

/* collision_util.cpp:109-215 dClosestLineSegmentPoints */
static void closest_segment_points(const real *a1, const real *a2, const real *b1, const real *b2,
                                   real *cp1, real *cp2) {
    real a1a2[3], b1b2[3], a1b1[3], a1b2[3], a2b1[3], a2b2[3], n[3];
    real la, lb, k, da1, da2, da3, da4, db1, db2, db3, db4, det;
#define SET2(a, b) a[0] = b[0]; a[1] = b[1]; a[2] = b[2];
#define SET3(a, b, op, c) a[0] = b[0] op c[0]; a[1] = b[1] op c[1]; a[2] = b[2] op c[2];
    SET3(a1a2, a2, -, a1); SET3(b1b2, b2, -, b1); SET3(a1b1, b1, -, a1);
    da1 = dot3(a1a2, a1b1); db1 = dot3(b1b2, a1b1);
    if (da1 <= 0 && db1 >= 0) { SET2(cp1, a1); SET2(cp2, b1); return; }
    SET3(a1b2, b2, -, a1);
    da2 = dot3(a1a2, a1b2); db2 = dot3(b1b2, a1b2);
    if (da2 <= 0 && db2 <= 0) { SET2(cp1, a1); SET2(cp2, b2); return; }
    SET3(a2b1, b1, -, a2);
    da3 = dot3(a1a2, a2b1); db3 = dot3(b1b2, a2b1);
    if (da3 >= 0 && db3 >= 0) { SET2(cp1, a2); SET2(cp2, b1); return; }
    SET3(a2b2, b2, -, a2);
    da4 = dot3(a1a2, a2b2); db4 = dot3(b1b2, a2b2);
    if (da4 >= 0 && db4 <= 0) { SET2(cp1, a2); SET2(cp2, b2); return; }
    la = dot3(a1a2, a1a2);
    if (da1 >= 0 && da3 <= 0) {
        k = da1 / la;
        n[0] = a1b1[0] - k * a1a2[0]; n[1] = a1b1[1] - k * a1a2[1]; n[2] = a1b1[2] - k * a1a2[2];
        if (dot3(b1b2, n) >= 0) {
            cp1[0] = a1[0] + k * a1a2[0]; cp1[1] = a1[1] + k * a1a2[1]; cp1[2] = a1[2] + k * a1a2[2];
            SET2(cp2, b1); return;
        }
    }
    if (da2 >= 0 && da4 <= 0) {
        k = da2 / la;
        n[0] = a1b2[0] - k * a1a2[0]; n[1] = a1b2[1] - k * a1a2[1]; n[2] = a1b2[2] - k * a1a2[2];
        if (dot3(b1b2, n) <= 0) {
            cp1[0] = a1[0] + k * a1a2[0]; cp1[1] = a1[1] + k * a1a2[1]; cp1[2] = a1[2] + k * a1a2[2];
            SET2(cp2, b2); return;
        }
    }
    lb = dot3(b1b2, b1b2);
    if (db1 <= 0 && db2 >= 0) {
        k = -db1 / lb;
        n[0] = -a1b1[0] - k * b1b2[0]; n[1] = -a1b1[1] - k * b1b2[1]; n[2] = -a1b1[2] - k * b1b2[2];
        if (dot3(a1a2, n) >= 0) {
            SET2(cp1, a1);
            cp2[0] = b1[0] + k * b1b2[0]; cp2[1] = b1[1] + k * b1b2[1]; cp2[2] = b1[2] + k * b1b2[2];
            return;
        }
    }
    if (db3 <= 0 && db4 >= 0) {
        k = -db3 / lb;
        n[0] = -a2b1[0] - k * b1b2[0]; n[1] = -a2b1[1] - k * b1b2[1]; n[2] = -a2b1[2] - k * b1b2[2];
        if (dot3(a1a2, n) <= 0) {
            SET2(cp1, a2);
            cp2[0] = b1[0] + k * b1b2[0]; cp2[1] = b1[1] + k * b1b2[1]; cp2[2] = b1[2] + k * b1b2[2];
            return;
        }
    }
    k = dot3(a1a2, b1b2);
    det = la * lb - k * k;
    if (det <= 0) { SET2(cp1, a1); SET2(cp2, b1); return; }
    det = 1.0f / det;
    real alpha = (lb * da1 - k * db1) * det;
    real beta = (k * da1 - la * db1) * det;
    cp1[0] = a1[0] + alpha * a1a2[0]; cp1[1] = a1[1] + alpha * a1a2[1]; cp1[2] = a1[2] + alpha * a1a2[2];
    cp2[0] = b1[0] + beta * b1b2[0]; cp2[1] = b1[1] + beta * b1b2[1]; cp2[2] = b1[2] + beta * b1b2[2];
#undef SET2
#undef SET3
}

/* collision_util.cpp:247-385 dClosestLineBoxPoints */
static void closest_line_box_points(const real *p1, const real *p2, const real *c, const real *R,
                                    const real *side, real *lret, real *bret) {
    int i;
    real tmp[3], s[3], v[3];
    tmp[0] = p1[0] - c[0]; tmp[1] = p1[1] - c[1]; tmp[2] = p1[2] - c[2];
    mul1_331(s, R, tmp);
    tmp[0] = p2[0] - p1[0]; tmp[1] = p2[1] - p1[1]; tmp[2] = p2[2] - p1[2];
    mul1_331(v, R, tmp);
    real sign[3];
    for (i = 0; i < 3; i++) {
        if (v[i] < 0) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = -1; }
        else sign[i] = 1;
    }
    real v2[3] = {v[0] * v[0], v[1] * v[1], v[2] * v[2]};
    real h[3] = {0.5f * side[0], 0.5f * side[1], 0.5f * side[2]};
    int region[3];
    real tanchor[3];
    const real tanchor_eps = 1e-19f;
    for (i = 0; i < 3; i++) {
        if (v[i] > tanchor_eps) {
            if (s[i] < -h[i]) { region[i] = -1; tanchor[i] = (-h[i] - s[i]) / v[i]; }
            else { region[i] = (s[i] > h[i]); tanchor[i] = (h[i] - s[i]) / v[i]; }
        } else { region[i] = 0; tanchor[i] = 2; }
    }
    real t = 0, dd2dt = 0;
    for (i = 0; i < 3; i++) dd2dt -= (region[i] ? v2[i] : 0) * tanchor[i];
    if (dd2dt >= 0) goto got_answer;
    do {
        real next_t = 1;
        for (i = 0; i < 3; i++)
            if (tanchor[i] > t && tanchor[i] < 1 && tanchor[i] < next_t) next_t = tanchor[i];
        real next_dd2dt = 0;
        for (i = 0; i < 3; i++) next_dd2dt += (region[i] ? v2[i] : 0) * (next_t - tanchor[i]);
        if (next_dd2dt >= 0) {
            real m = (next_dd2dt - dd2dt) / (next_t - t);
            t -= dd2dt / m;
            goto got_answer;
        }
        for (i = 0; i < 3; i++)
            if (tanchor[i] == next_t) { tanchor[i] = (h[i] - s[i]) / v[i]; region[i]++; }
        t = next_t;
        dd2dt = next_dd2dt;
    } while (t < 1);
    t = 1;
got_answer:
    for (i = 0; i < 3; i++) lret[i] = p1[i] + t * tmp[i];
    for (i = 0; i < 3; i++) {
        tmp[i] = sign[i] * (s[i] + t * v[i]);
        if (tmp[i] < -h[i]) tmp[i] = -h[i];
        else if (tmp[i] > h[i]) tmp[i] = h[i];
    }
    mul0_331(s, R, tmp);
    for (i = 0; i < 3; i++) bret[i] = s[i] + c[i];
}

/* box.cpp:212-263 intersectRectQuad */
static int intersect_rect_quad(const real h[2], real p[8], real ret[16]) {
    int nq = 4, nr = 0;
    real buffer[16];
    real *q = p, *r = ret;
    for (int dir = 0; dir <= 1; dir++) {
        for (int sign = -1; sign <= 1; sign += 2) {
            real *pq = q, *pr = r;
            nr = 0;
            for (int i = nq; i > 0; i--) {
                if (sign * pq[dir] < h[dir]) {
                    pr[0] = pq[0]; pr[1] = pq[1];
                    pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                real *nextq = (i > 1) ? pq + 2 : q;
                if ((sign * pq[dir] < h[dir]) ^ (sign * nextq[dir] < h[dir])) {
                    pr[1 - dir] = pq[1 - dir] + (nextq[1 - dir] - pq[1 - dir]) / (nextq[dir] - pq[dir]) *
                                                    (sign * h[dir] - pq[dir]);
                    pr[dir] = sign * h[dir];
                    pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                pq += 2;
            }
            q = r;
            r = (q == ret) ? buffer : ret;
            nq = nr;
        }
    }
done:
    if (q != ret) memcpy(ret, q, nr * 2 * sizeof(real));
    return nr;
}

/* box.cpp:274-336 cullPoints */
static void cull_points(int n, const real p[], int m, int i0, int iret[]) {
    int i, j;
    real a, cx, cy, q;
    if (n == 1) { cx = p[0]; cy = p[1]; }
    else if (n == 2) { cx = 0.5f * (p[0] + p[2]); cy = 0.5f * (p[1] + p[3]); }
    else {
        a = 0; cx = 0; cy = 0;
        for (i = 0; i < (n - 1); i++) {
            q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
            a += q;
            cx += q * (p[i * 2] + p[i * 2 + 2]);
            cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
        }
        q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
        a = 1.0f / (3.0f * (a + q));
        cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
        cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
    }
    real A[8];
    for (i = 0; i < n; i++) A[i] = atan2f(p[i * 2 + 1] - cy, p[i * 2] - cx);
    int avail[8];
    for (i = 0; i < n; i++) avail[i] = 1;
    avail[i0] = 0;
    iret[0] = i0;
    iret++;
    for (j = 1; j < m; j++) {
        a = (real)((double)(real)j * (2 * M_PI / m) + A[i0]);
        if (a > M_PI) a -= (real)(2 * M_PI);
        real maxdiff = 1e9f, diff;
        for (i = 0; i < n; i++) {
            if (avail[i]) {
                diff = fabsf(A[i] - a);
                if (diff > M_PI) diff = (real)(2 * M_PI - diff);
                if (diff < maxdiff) { maxdiff = diff; *iret = i; }
            }
        }
        avail[*iret] = 0;
        iret++;
    }
}

/* box.cpp:356-737 dBoxBox */
static int box_box(const real *p1, const real *R1, const real *side1, const real *p2, const real *R2,
                   const real *side2, real *normal, real *depth, int *return_code, int flags,
                   pcontact *contact) {
    const real fudge_factor = 1.05f;
    real p[3], pp[3], normalC[3] = {0, 0, 0};
    const real *normalR = 0;
    real A[3], B[3], R11, R12, R13, R21, R22, R23, R31, R32, R33, Q11, Q12, Q13, Q21, Q22, Q23, Q31, Q32,
        Q33, s, s2, l, expr1_val;
    int i, j, invert_normal, code;
    p[0] = p2[0] - p1[0]; p[1] = p2[1] - p1[1]; p[2] = p2[2] - p1[2];
    mul1_331(pp, R1, p);
    A[0] = side1[0] * 0.5f; A[1] = side1[1] * 0.5f; A[2] = side1[2] * 0.5f;
    B[0] = side2[0] * 0.5f; B[1] = side2[1] * 0.5f; B[2] = side2[2] * 0.5f;
    R11 = dot3_44(R1 + 0, R2 + 0); R12 = dot3_44(R1 + 0, R2 + 1); R13 = dot3_44(R1 + 0, R2 + 2);
    R21 = dot3_44(R1 + 1, R2 + 0); R22 = dot3_44(R1 + 1, R2 + 1); R23 = dot3_44(R1 + 1, R2 + 2);
    R31 = dot3_44(R1 + 2, R2 + 0); R32 = dot3_44(R1 + 2, R2 + 1); R33 = dot3_44(R1 + 2, R2 + 2);
    Q11 = fabsf(R11); Q12 = fabsf(R12); Q13 = fabsf(R13);
    Q21 = fabsf(R21); Q22 = fabsf(R22); Q23 = fabsf(R23);
    Q31 = fabsf(R31); Q32 = fabsf(R32); Q33 = fabsf(R33);

#define TSTF(expr1, expr2, norm, cc)                                      \
    expr1_val = (expr1);                                                  \
    s2 = fabsf(expr1_val) - (expr2);                                      \
    if (s2 > 0) return 0;                                                 \
    if (s2 > s) { s = s2; normalR = norm; invert_normal = ((expr1_val) < 0); code = (cc); }
#define TSTE(expr1, expr2, n1, n2, n3, cc)                                \
    expr1_val = (expr1);                                                  \
    s2 = fabsf(expr1_val) - (expr2);                                      \
    if (s2 > 0) return 0;                                                 \
    l = sqrtf((n1) * (n1) + (n2) * (n2) + (n3) * (n3));                   \
    if (l > 0) {                                                          \
        s2 /= l;                                                          \
        if (s2 * fudge_factor > s) {                                      \
            s = s2; normalR = 0;                                          \
            normalC[0] = (n1) / l; normalC[1] = (n2) / l; normalC[2] = (n3) / l; \
            invert_normal = ((expr1_val) < 0); code = (cc);               \
        }                                                                 \
    }
    s = -INF; invert_normal = 0; code = 0;
    TSTF(pp[0], (A[0] + B[0] * Q11 + B[1] * Q12 + B[2] * Q13), R1 + 0, 1);
    TSTF(pp[1], (A[1] + B[0] * Q21 + B[1] * Q22 + B[2] * Q23), R1 + 1, 2);
    TSTF(pp[2], (A[2] + B[0] * Q31 + B[1] * Q32 + B[2] * Q33), R1 + 2, 3);
    TSTF(dot3_41(R2 + 0, p), (A[0] * Q11 + A[1] * Q21 + A[2] * Q31 + B[0]), R2 + 0, 4);
    TSTF(dot3_41(R2 + 1, p), (A[0] * Q12 + A[1] * Q22 + A[2] * Q32 + B[1]), R2 + 1, 5);
    TSTF(dot3_41(R2 + 2, p), (A[0] * Q13 + A[1] * Q23 + A[2] * Q33 + B[2]), R2 + 2, 6);
    TSTE(pp[2] * R21 - pp[1] * R31, (A[1] * Q31 + A[2] * Q21 + B[1] * Q13 + B[2] * Q12), 0, -R31, R21, 7);
    TSTE(pp[2] * R22 - pp[1] * R32, (A[1] * Q32 + A[2] * Q22 + B[0] * Q13 + B[2] * Q11), 0, -R32, R22, 8);
    TSTE(pp[2] * R23 - pp[1] * R33, (A[1] * Q33 + A[2] * Q23 + B[0] * Q12 + B[1] * Q11), 0, -R33, R23, 9);
    TSTE(pp[0] * R31 - pp[2] * R11, (A[0] * Q31 + A[2] * Q11 + B[1] * Q23 + B[2] * Q22), R31, 0, -R11, 10);
    TSTE(pp[0] * R32 - pp[2] * R12, (A[0] * Q32 + A[2] * Q12 + B[0] * Q23 + B[2] * Q21), R32, 0, -R12, 11);
    TSTE(pp[0] * R33 - pp[2] * R13, (A[0] * Q33 + A[2] * Q13 + B[0] * Q22 + B[1] * Q21), R33, 0, -R13, 12);
    TSTE(pp[1] * R11 - pp[0] * R21, (A[0] * Q21 + A[1] * Q11 + B[1] * Q33 + B[2] * Q32), -R21, R11, 0, 13);
    TSTE(pp[1] * R12 - pp[0] * R22, (A[0] * Q22 + A[1] * Q12 + B[0] * Q33 + B[2] * Q31), -R22, R12, 0, 14);
    TSTE(pp[1] * R13 - pp[0] * R23, (A[0] * Q23 + A[1] * Q13 + B[0] * Q32 + B[1] * Q31), -R23, R13, 0, 15);
#undef TSTF
#undef TSTE
    if (!code) return 0;
    if (normalR) { normal[0] = normalR[0]; normal[1] = normalR[4]; normal[2] = normalR[8]; }
    else mul0_331(normal, R1, normalC);
    if (invert_normal) { normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2]; }
    *depth = -s;

    if (code > 6) {
        real pa[3], pb[3], sign, alpha, beta, ua[3], ub[3];
        for (i = 0; i < 3; i++) pa[i] = p1[i];
        for (j = 0; j < 3; j++) {
            sign = (dot3_14(normal, R1 + j) > 0) ? 1.0f : -1.0f;
            for (i = 0; i < 3; i++) pa[i] += sign * A[j] * R1[i * 4 + j];
        }
        for (i = 0; i < 3; i++) pb[i] = p2[i];
        for (j = 0; j < 3; j++) {
            sign = (dot3_14(normal, R2 + j) > 0) ? -1.0f : 1.0f;
            for (i = 0; i < 3; i++) pb[i] += sign * B[j] * R2[i * 4 + j];
        }
        for (i = 0; i < 3; i++) ua[i] = R1[((code)-7) / 3 + i * 4];
        for (i = 0; i < 3; i++) ub[i] = R2[((code)-7) % 3 + i * 4];
        line_closest_approach(pa, ua, pb, ub, &alpha, &beta);
        for (i = 0; i < 3; i++) pa[i] += ua[i] * alpha;
        for (i = 0; i < 3; i++) pb[i] += ub[i] * beta;
        for (i = 0; i < 3; i++) contact[0].pos[i] = 0.5f * (pa[i] + pb[i]);
        contact[0].depth = *depth;
        *return_code = code;
        return 1;
    }

    const real *Ra, *Rb, *pa, *pb, *Sa, *Sb;
    if (code <= 3) { Ra = R1; Rb = R2; pa = p1; pb = p2; Sa = A; Sb = B; }
    else { Ra = R2; Rb = R1; pa = p2; pb = p1; Sa = B; Sb = A; }
    real normal2[3], nr[3], anr[3];
    if (code <= 3) { normal2[0] = normal[0]; normal2[1] = normal[1]; normal2[2] = normal[2]; }
    else { normal2[0] = -normal[0]; normal2[1] = -normal[1]; normal2[2] = -normal[2]; }
    mul1_331(nr, Rb, normal2);
    anr[0] = fabsf(nr[0]); anr[1] = fabsf(nr[1]); anr[2] = fabsf(nr[2]);
    int lanr, a1, a2;
    if (anr[1] > anr[0]) {
        if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    real center[3];
    if (nr[lanr] < 0) { for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] + Sb[lanr] * Rb[i * 4 + lanr]; }
    else { for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] - Sb[lanr] * Rb[i * 4 + lanr]; }
    int codeN, code1, code2;
    if (code <= 3) codeN = code - 1; else codeN = code - 4;
    if (codeN == 0) { code1 = 1; code2 = 2; }
    else if (codeN == 1) { code1 = 0; code2 = 2; }
    else { code1 = 0; code2 = 1; }
    real quad[8], c1, c2, m11, m12, m21, m22;
    c1 = dot3_14(center, Ra + code1);
    c2 = dot3_14(center, Ra + code2);
    m11 = dot3_44(Ra + code1, Rb + a1);
    m12 = dot3_44(Ra + code1, Rb + a2);
    m21 = dot3_44(Ra + code2, Rb + a1);
    m22 = dot3_44(Ra + code2, Rb + a2);
    {
        real k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
        quad[0] = c1 - k1 - k3; quad[1] = c2 - k2 - k4;
        quad[2] = c1 - k1 + k3; quad[3] = c2 - k2 + k4;
        quad[4] = c1 + k1 + k3; quad[5] = c2 + k2 + k4;
        quad[6] = c1 + k1 - k3; quad[7] = c2 + k2 - k4;
    }
    real rect[2] = {Sa[code1], Sa[code2]};
    real ret[16];
    int n = intersect_rect_quad(rect, quad, ret);
    if (n < 1) return 0;
    real point[3 * 8], dep[8];
    real det1 = 1.0f / (m11 * m22 - m12 * m21);
    m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
    int cnum = 0;
    for (j = 0; j < n; j++) {
        real k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        real k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb[i * 4 + a1] + k2 * Rb[i * 4 + a2];
        dep[cnum] = Sa[codeN] - dot3(normal2, point + cnum * 3);
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return 0;
    int maxc = flags & NUMC_MASK;
    if (maxc > cnum) maxc = cnum;
    if (maxc < 1) maxc = 1;
    if (cnum <= maxc) {
        for (j = 0; j < cnum; j++) {
            for (i = 0; i < 3; i++) contact[j].pos[i] = point[j * 3 + i] + pa[i];
            contact[j].depth = dep[j];
        }
    } else {
        int i1 = 0;
        real maxdepth = dep[0];
        for (i = 1; i < cnum; i++)
            if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
        int iret[8];
        cull_points(cnum, ret, maxc, i1, iret);
        for (j = 0; j < maxc; j++) {
            for (i = 0; i < 3; i++) contact[j].pos[i] = point[iret[j] * 3 + i] + pa[i];
            contact[j].depth = dep[iret[j]];
        }
        cnum = maxc;
    }
    *return_code = code;
    return cnum;
}

/* box.cpp:741-767 dCollideBoxBox */
static int collide_box_box(const pgeom *o1, const pgeom *o2, int flags, pcontact *c) {
    real normal[3], depth;
    int code;
    int num = box_box(o1->pos, o1->R, o1->dims, o2->pos, o2->R, o2->dims, normal, &depth, &code, flags, c);
    for (int i = 0; i < num; i++) { c[i].normal[0] = -normal[0]; c[i].normal[1] = -normal[1]; c[i].normal[2] = -normal[2]; }
    return num;
}

/* box.cpp:770-903 dCollideBoxPlane */
static int collide_box_plane(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    const real *R = o1->R, *n = o2->dims, *side = o1->dims;
    int ret = 0;
    real Q1 = dot3_14(n, R + 0), Q2 = dot3_14(n, R + 1), Q3 = dot3_14(n, R + 2);
    real A1 = side[0] * Q1, A2 = side[1] * Q2, A3 = side[2] * Q3;
    real B1 = fabsf(A1), B2 = fabsf(A2), B3 = fabsf(A3);
    real depth = n[3] + 0.5f * (B1 + B2 + B3) - dot3(n, o1->pos);
    if (depth < 0) return 0;
    int maxc = flags & NUMC_MASK;
    if (maxc > 4) maxc = 4;
    real p[3] = {o1->pos[0], o1->pos[1], o1->pos[2]};
#define FOO(i, op) p[0] op 0.5f * side[i] * R[0 + i]; p[1] op 0.5f * side[i] * R[4 + i]; p[2] op 0.5f * side[i] * R[8 + i];
#define BAR(i, iinc) if (A##iinc > 0) { FOO(i, -=) } else { FOO(i, +=) }
    BAR(0, 1);
    BAR(1, 2);
    BAR(2, 3);
#undef FOO
#undef BAR
    contact[0].pos[0] = p[0]; contact[0].pos[1] = p[1]; contact[0].pos[2] = p[2];
    contact[0].depth = depth;
    ret = 1;
    if (maxc == 1) goto done;
#define FOO(i, j, op) contact[i].pos[0] = p[0] op side[j] * R[0 + j]; contact[i].pos[1] = p[1] op side[j] * R[4 + j]; contact[i].pos[2] = p[2] op side[j] * R[8 + j];
#define BAR(ctact, side_, sideinc)                                   \
    if (depth - B##sideinc < 0) goto done;                           \
    if (A##sideinc > 0) { FOO(ctact, side_, +); } else { FOO(ctact, side_, -); } \
    contact[ctact].depth = depth - B##sideinc;                       \
    ret++;
    if (B1 < B2) {
        if (B3 < B1) goto use_side_3;
        else {
            BAR(1, 0, 1);
            if (maxc == 2) goto done;
            if (B2 < B3) goto contact2_2; else goto contact2_3;
        }
    } else {
        if (B3 < B2) {
        use_side_3:
            BAR(1, 2, 3);
            if (maxc == 2) goto done;
            if (B1 < B2) goto contact2_1; else goto contact2_2;
        } else {
            BAR(1, 1, 2);
            if (maxc == 2) goto done;
            if (B1 < B3) goto contact2_1; else goto contact2_3;
        }
    }
contact2_1: BAR(2, 0, 1); goto done;
contact2_2: BAR(2, 1, 2); goto done;
contact2_3: BAR(2, 2, 3); goto done;
#undef FOO
#undef BAR
done:
    if (maxc == 4 && ret == 3) {
        real d4 = contact[1].depth + contact[2].depth - depth;
        if (d4 > 0) {
            contact[3].pos[0] = contact[1].pos[0] + contact[2].pos[0] - p[0];
            contact[3].pos[1] = contact[1].pos[1] + contact[2].pos[1] - p[1];
            contact[3].pos[2] = contact[1].pos[2] + contact[2].pos[2] - p[2];
            contact[3].depth = d4;
            ret++;
        }
    }
    for (int i = 0; i < ret; i++) { contact[i].normal[0] = n[0]; contact[i].normal[1] = n[1]; contact[i].normal[2] = n[2]; }
    return ret;
}

/* sphere.cpp:110-128 */
static int collide_sphere_sphere(const pgeom *o1, const pgeom *o2, int flags, pcontact *c) {
    (void)flags;
    return collide_spheres(o1->pos, o1->dims[0], o2->pos, o2->dims[0], c);
}

/* sphere.cpp:131-219 dCollideSphereBox */
static int collide_sphere_box(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    (void)flags;
    real l[3], t[4], p[3], q[3], r[3], depth;
    int onborder = 0;
    const real *R = o2->R;
    p[0] = o1->pos[0] - o2->pos[0]; p[1] = o1->pos[1] - o2->pos[1]; p[2] = o1->pos[2] - o2->pos[2];
    l[0] = o2->dims[0] * 0.5f;
    t[0] = dot3_14(p, R);
    if (t[0] < -l[0]) { t[0] = -l[0]; onborder = 1; }
    if (t[0] > l[0]) { t[0] = l[0]; onborder = 1; }
    l[1] = o2->dims[1] * 0.5f;
    t[1] = dot3_14(p, R + 1);
    if (t[1] < -l[1]) { t[1] = -l[1]; onborder = 1; }
    if (t[1] > l[1]) { t[1] = l[1]; onborder = 1; }
    t[2] = dot3_14(p, R + 2);
    l[2] = o2->dims[2] * 0.5f;
    if (t[2] < -l[2]) { t[2] = -l[2]; onborder = 1; }
    if (t[2] > l[2]) { t[2] = l[2]; onborder = 1; }
    if (!onborder) {
        real min_distance = l[0] - fabsf(t[0]);
        int mini = 0;
        for (int i = 1; i < 3; i++) {
            real face_distance = l[i] - fabsf(t[i]);
            if (face_distance < min_distance) { min_distance = face_distance; mini = i; }
        }
        contact->pos[0] = o1->pos[0]; contact->pos[1] = o1->pos[1]; contact->pos[2] = o1->pos[2];
        real tmp[3] = {0, 0, 0};
        tmp[mini] = (t[mini] > 0) ? 1.0f : -1.0f;
        mul0_331(contact->normal, R, tmp);
        contact->depth = min_distance + o1->dims[0];
        return 1;
    }
    t[3] = 0;
    mul0_331(q, R, t);
    r[0] = p[0] - q[0]; r[1] = p[1] - q[1]; r[2] = p[2] - q[2];
    depth = o1->dims[0] - sqrtf(dot3(r, r));
    if (depth < 0) return 0;
    contact->pos[0] = q[0] + o2->pos[0]; contact->pos[1] = q[1] + o2->pos[1]; contact->pos[2] = q[2] + o2->pos[2];
    contact->normal[0] = r[0]; contact->normal[1] = r[1]; contact->normal[2] = r[2];
    normalize3(contact->normal);
    contact->depth = depth;
    return 1;
}

/* sphere.cpp:222-251 dCollideSpherePlane */
static int collide_sphere_plane(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    (void)flags;
    const real *pl = o2->dims;
    real k = dot3(o1->pos, pl);
    real depth = pl[3] - k + o1->dims[0];
    if (depth >= 0) {
        contact->normal[0] = pl[0]; contact->normal[1] = pl[1]; contact->normal[2] = pl[2];
        contact->pos[0] = o1->pos[0] - pl[0] * o1->dims[0];
        contact->pos[1] = o1->pos[1] - pl[1] * o1->dims[0];
        contact->pos[2] = o1->pos[2] - pl[2] * o1->dims[0];
        contact->depth = depth;
        return 1;
    }
    return 0;
}

/* capsule.cpp:130-161 dCollideCapsuleSphere */
static int collide_capsule_sphere(const pgeom *o1, const pgeom *o2, int flags, pcontact *c) {
    (void)flags;
    const real *R = o1->R;
    real alpha = R[2] * (o2->pos[0] - o1->pos[0]) + R[6] * (o2->pos[1] - o1->pos[1]) + R[10] * (o2->pos[2] - o1->pos[2]);
    real lz2 = o1->dims[1] * 0.5f;
    if (alpha > lz2) alpha = lz2;
    if (alpha < -lz2) alpha = -lz2;
    real p[3] = {o1->pos[0] + alpha * R[2], o1->pos[1] + alpha * R[6], o1->pos[2] + alpha * R[10]};
    return collide_spheres(p, o1->dims[0], o2->pos, o2->dims[0], c);
}

/* capsule.cpp:164-235 dCollideCapsuleBox */
static int collide_capsule_box(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    const real *R1 = o1->R;
    real clen = o1->dims[1] * 0.5f;
    real p1[3] = {o1->pos[0] + clen * R1[2], o1->pos[1] + clen * R1[6], o1->pos[2] + clen * R1[10]};
    real p2[3] = {o1->pos[0] - clen * R1[2], o1->pos[1] - clen * R1[6], o1->pos[2] - clen * R1[10]};
    real radius = o1->dims[0];
    const real *c = o2->pos, *R = o2->R, *side = o2->dims;
    real pl[3], pb[3];
    closest_line_box_points(p1, p2, c, R, side, pl, pb);
    real mindist = 1e-6f;
    if (dist3(pl, pb) < mindist) {
        real normal[3], depth;
        int code;
        real radiusMul2 = radius * 2.0f;
        real capboxside[4] = {radiusMul2, radiusMul2, o1->dims[1] + radiusMul2, 0};
        int num = box_box(c, R, side, o1->pos, o1->R, capboxside, normal, &depth, &code, flags, contact);
        for (int i = 0; i < num; i++) {
            contact[i].normal[0] = normal[0]; contact[i].normal[1] = normal[1]; contact[i].normal[2] = normal[2];
        }
        return num;
    }
    return collide_spheres(pl, radius, pb, 0, contact);
}

/* capsule.cpp:238-353 dCollideCapsuleCapsule */
static int collide_capsule_capsule(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    int i;
    const real tolerance = 1e-5f;
    real lz1 = o1->dims[1] * 0.5f, lz2 = o2->dims[1] * 0.5f;
    const real *pos1 = o1->pos, *pos2 = o2->pos;
    real axis1[3] = {o1->R[2], o1->R[6], o1->R[10]};
    real axis2[3] = {o2->R[2], o2->R[6], o2->R[10]};
    real sphere1[3], sphere2[3];
    real a1a2 = dot3(axis1, axis2);
    real det = 1.0f - a1a2 * a1a2;
    if (det < tolerance) {
        if (a1a2 < 0) { axis2[0] = -axis2[0]; axis2[1] = -axis2[1]; axis2[2] = -axis2[2]; }
        real q[3];
        for (i = 0; i < 3; i++) q[i] = pos1[i] - pos2[i];
        real k = dot3(axis1, q);
        real a1lo = -lz1, a1hi = lz1, a2lo = -lz2 - k, a2hi = lz2 - k;
        real lo = (a1lo > a2lo) ? a1lo : a2lo;
        real hi = (a1hi < a2hi) ? a1hi : a2hi;
        if (lo <= hi) {
            int num_contacts = flags & NUMC_MASK;
            if (num_contacts >= 2 && lo < hi) {
                for (i = 0; i < 3; i++) sphere1[i] = pos1[i] + lo * axis1[i];
                for (i = 0; i < 3; i++) sphere2[i] = pos2[i] + (lo + k) * axis2[i];
                int n1 = collide_spheres(sphere1, o1->dims[0], sphere2, o2->dims[0], contact);
                if (n1) {
                    for (i = 0; i < 3; i++) sphere1[i] = pos1[i] + hi * axis1[i];
                    for (i = 0; i < 3; i++) sphere2[i] = pos2[i] + (hi + k) * axis2[i];
                    int n2 = collide_spheres(sphere1, o1->dims[0], sphere2, o2->dims[0], contact + 1);
                    if (n2) return 2;
                }
            }
            real alpha1 = (lo + hi) * 0.5f;
            real alpha2 = alpha1 + k;
            for (i = 0; i < 3; i++) sphere1[i] = pos1[i] + alpha1 * axis1[i];
            for (i = 0; i < 3; i++) sphere2[i] = pos2[i] + alpha2 * axis2[i];
            return collide_spheres(sphere1, o1->dims[0], sphere2, o2->dims[0], contact);
        }
    }
    real a1[3], a2[3], b1[3], b2[3];
    a1[0] = pos1[0] + axis1[0] * lz1; a1[1] = pos1[1] + axis1[1] * lz1; a1[2] = pos1[2] + axis1[2] * lz1;
    a2[0] = pos1[0] - axis1[0] * lz1; a2[1] = pos1[1] - axis1[1] * lz1; a2[2] = pos1[2] - axis1[2] * lz1;
    b1[0] = pos2[0] + axis2[0] * lz2; b1[1] = pos2[1] + axis2[1] * lz2; b1[2] = pos2[2] + axis2[2] * lz2;
    b2[0] = pos2[0] - axis2[0] * lz2; b2[1] = pos2[1] - axis2[1] * lz2; b2[2] = pos2[2] - axis2[2] * lz2;
    closest_segment_points(a1, a2, b1, b2, sphere1, sphere2);
    return collide_spheres(sphere1, o1->dims[0], sphere2, o2->dims[0], contact);
}

/* capsule.cpp:356-415 dCollideCapsulePlane */
static int collide_capsule_plane(const pgeom *o1, const pgeom *o2, int flags, pcontact *contact) {
    const real *pl = o2->dims, *R = o1->R;
    real lz = o1->dims[1], rad = o1->dims[0];
    real sign = (dot3_14(pl, R + 2) > 0) ? -1.0f : 1.0f;
    real p[3];
    p[0] = o1->pos[0] + R[2] * lz * 0.5f * sign;
    p[1] = o1->pos[1] + R[6] * lz * 0.5f * sign;
    p[2] = o1->pos[2] + R[10] * lz * 0.5f * sign;
    real k = dot3(p, pl);
    real depth = pl[3] - k + rad;
    if (depth < 0) return 0;
    contact->normal[0] = pl[0]; contact->normal[1] = pl[1]; contact->normal[2] = pl[2];
    contact->pos[0] = p[0] - pl[0] * rad; contact->pos[1] = p[1] - pl[1] * rad; contact->pos[2] = p[2] - pl[2] * rad;
    contact->depth = depth;
    int ncontacts = 1;
    if ((flags & NUMC_MASK) >= 2) {
        p[0] = o1->pos[0] - R[2] * lz * 0.5f * sign;
        p[1] = o1->pos[1] - R[6] * lz * 0.5f * sign;
        p[2] = o1->pos[2] - R[10] * lz * 0.5f * sign;
        k = dot3(p, pl);
        depth = pl[3] - k + rad;
        if (depth >= 0) {
            pcontact *c2 = contact + 1;
            c2->normal[0] = pl[0]; c2->normal[1] = pl[1]; c2->normal[2] = pl[2];
            c2->pos[0] = p[0] - pl[0] * rad; c2->pos[1] = p[1] - pl[1] * rad; c2->pos[2] = p[2] - pl[2] * rad;
            c2->depth = depth;
            ncontacts = 2;
        }
    }
    return ncontacts;
}

typedef int (*collider_fn)(const pgeom *, const pgeom *, int, pcontact *);
/* collision_kernel.cpp:182-190 collider table for the four classes */
static collider_fn table_fn(int a, int b, int *reverse) {
    *reverse = 0;
#define E(x, y, f) if (a == x && b == y) return f; if (a == y && b == x) { *reverse = 1; return f; }
    E(PORT_SPHERE, PORT_SPHERE, collide_sphere_sphere);
    E(PORT_SPHERE, PORT_BOX, collide_sphere_box);
    E(PORT_SPHERE, PORT_PLANE, collide_sphere_plane);
    E(PORT_BOX, PORT_BOX, collide_box_box);
    E(PORT_BOX, PORT_PLANE, collide_box_plane);
    E(PORT_CAPSULE, PORT_SPHERE, collide_capsule_sphere);
    E(PORT_CAPSULE, PORT_BOX, collide_capsule_box);
    E(PORT_CAPSULE, PORT_CAPSULE, collide_capsule_capsule);
    E(PORT_CAPSULE, PORT_PLANE, collide_capsule_plane);
#undef E
    return 0;
}

/* collision_kernel.cpp:292-338 dCollide (geoms already posed; same-geom and
 * same-body rejections are done by the callers that know the bodies). */
static int collide_geoms(const pgeom *o1, const pgeom *o2, int flags, pcontact *c) {
    if ((flags & NUMC_MASK) == 0) return 0;
    int rev;
    collider_fn fn = table_fn(o1->cls, o2->cls, &rev);
    if (!fn) return 0;
    int count;
    if (rev) {
        count = fn(o2, o1, flags, c);
        for (int i = 0; i < count; i++) {
            c[i].normal[0] = -c[i].normal[0]; c[i].normal[1] = -c[i].normal[1]; c[i].normal[2] = -c[i].normal[2];
            c[i].swap = 0; /* dCollide swaps g1/g2 back: g1 is always o1 */
        }
    } else {
        count = fn(o1, o2, flags, c);
        for (int i = 0; i < count; i++) c[i].swap = 0;
    }
    return count;
}

static void make_pgeom(pgeom *g, int cls, const float *pos, const float *R, const float *dims) {
    memset(g, 0, sizeof *g);
    g->cls = cls;
    if (pos) { g->pos[0] = pos[0]; g->pos[1] = pos[1]; g->pos[2] = pos[2]; }
    if (R) memcpy(g->R, R, 12 * sizeof(real));
    memcpy(g->dims, dims, 4 * sizeof(real));
    if (cls == PORT_PLANE) {
        /* plane.cpp:48-66 make_sure_plane_normal_has_unit_length */
        real *p = g->dims;
        real l = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        if (l > 0) {
            l = 1.0f / sqrtf(l);
            p[0] *= l; p[1] *= l; p[2] *= l; p[3] *= l;
        } else {
            p[0] = 1; p[1] = 0; p[2] = 0; p[3] = 0;
        }
    }
}

int port_collide(int cls1, const float *pos1, const float *R1, const float *dims1, int cls2,
                 const float *pos2, const float *R2, const float *dims2, int flags, float *out) {
    pgeom a, b;
    make_pgeom(&a, cls1, pos1, R1, dims1);
    make_pgeom(&b, cls2, pos2, R2, dims2);
    pcontact c[8];
    memset(c, 0, sizeof c);
    int n = collide_geoms(&a, &b, flags, c);
    for (int i = 0; i < n; i++) {
        float *o = out + 8 * i;
        o[0] = c[i].pos[0]; o[1] = c[i].pos[1]; o[2] = c[i].pos[2];
        o[3] = c[i].normal[0]; o[4] = c[i].normal[1]; o[5] = c[i].normal[2];
        o[6] = c[i].depth; o[7] = (float)c[i].swap;
    }
    return n;
}

int port_boxbox_code(const float *p1, const float *R1, const float *s1, const float *p2, const float *R2,
                     const float *s2, int flags) {
    real n[3], d;
    int code = 0;
    pcontact c[8];
    int num = box_box(p1, R1, s1, p2, R2, s2, n, &d, &code, flags, c);
    return num ? code : 0;
}

/* ------------------------------------------------------------- AABBs */
/* box.cpp:60-77, sphere.cpp:59-67, capsule.cpp:60-74, plane.cpp:80-105 */
static void compute_aabb(const pgeom *g, real *aabb) {
    const real *R = g->R, *pos = g->pos, *d = g->dims;
    switch (g->cls) {
    case PORT_SPHERE:
        aabb[0] = pos[0] - d[0]; aabb[1] = pos[0] + d[0];
        aabb[2] = pos[1] - d[0]; aabb[3] = pos[1] + d[0];
        aabb[4] = pos[2] - d[0]; aabb[5] = pos[2] + d[0];
        break;
    case PORT_BOX: {
        real xr = 0.5f * (fabsf(R[0] * d[0]) + fabsf(R[1] * d[1]) + fabsf(R[2] * d[2]));
        real yr = 0.5f * (fabsf(R[4] * d[0]) + fabsf(R[5] * d[1]) + fabsf(R[6] * d[2]));
        real zr = 0.5f * (fabsf(R[8] * d[0]) + fabsf(R[9] * d[1]) + fabsf(R[10] * d[2]));
        aabb[0] = pos[0] - xr; aabb[1] = pos[0] + xr;
        aabb[2] = pos[1] - yr; aabb[3] = pos[1] + yr;
        aabb[4] = pos[2] - zr; aabb[5] = pos[2] + zr;
        break;
    }
    case PORT_CAPSULE: {
        real xr = fabsf(R[2] * d[1]) * 0.5f + d[0];
        real yr = fabsf(R[6] * d[1]) * 0.5f + d[0];
        real zr = fabsf(R[10] * d[1]) * 0.5f + d[0];
        aabb[0] = pos[0] - xr; aabb[1] = pos[0] + xr;
        aabb[2] = pos[1] - yr; aabb[3] = pos[1] + yr;
        aabb[4] = pos[2] - zr; aabb[5] = pos[2] + zr;
        break;
    }
    case PORT_PLANE: {
        const real *p = d;
        for (int i = 0; i < 6; i++) aabb[i] = (i & 1) ? INF : -INF;
        if (p[1] == 0.0f && p[2] == 0.0f) {
            aabb[0] = (p[0] > 0) ? -INF : -p[3];
            aabb[1] = (p[0] > 0) ? p[3] : INF;
        } else if (p[0] == 0.0f && p[2] == 0.0f) {
            aabb[2] = (p[1] > 0) ? -INF : -p[3];
            aabb[3] = (p[1] > 0) ? p[3] : INF;
        } else if (p[0] == 0.0f && p[1] == 0.0f) {
            aabb[4] = (p[2] > 0) ? -INF : -p[3];
            aabb[5] = (p[2] > 0) ? p[3] : INF;
        }
        break;
    }
    }
}

/* ------------------------------------------------------------- hash space */
#define MAXINT_ ((int)((((unsigned int)(-1)) << 1) >> 1))
static const unsigned long primes[31] = {1L, 2L, 3L, 7L, 13L, 31L, 61L, 127L, 251L, 509L, 1021L, 2039L, 4093L,
                                         8191L, 16381L, 32749L, 65521L, 131071L, 262139L, 524287L, 1048573L,
                                         2097143L, 4194301L, 8388593L, 16777213L, 33554393L, 67108859L,
                                         134217689L, 268435399L, 536870909L, 1073741789L};
/* collision_space.cpp:329-349 findLevel */
static int find_level(const real *b) {
    if (b[0] <= -INF || b[1] >= INF || b[2] <= -INF || b[3] >= INF || b[4] <= -INF || b[5] >= INF) return MAXINT_;
    real q = b[1] - b[0], q2 = b[3] - b[2];
    if (q2 > q) q = q2;
    q2 = b[5] - b[4];
    if (q2 > q) q = q2;
    int level;
    frexp(q, &level);
    return level;
}
typedef struct { int level; int db[6]; int geom; size_t index; } hbox;
typedef struct { int next; int x, y, z; int box; } hnode;

typedef void (*pair_cb)(void *ctx, int g1, int g2);

/* collision_space_internal.h:44-80 collideAABBs (category bits all set) */
static void collide_aabbs(int g1, int g2, const int *body, const real *aabbs, void *ctx, pair_cb cb) {
    if (body[g1] == body[g2] && body[g1] >= 0) return;
    const real *b1 = aabbs + 6 * g1, *b2 = aabbs + 6 * g2;
    if (b1[0] > b2[1] || b1[1] < b2[0] || b1[2] > b2[3] || b1[3] < b2[2] || b1[4] > b2[5] || b1[5] < b2[4]) return;
    cb(ctx, g1, g2);
}

/* collision_space.cpp:421-614 dxHashSpace::collide.  order: space list order. */
static void hash_collide(int n, const int *order, const int *body, const real *aabbs, int minlevel, int maxlevel_g,
                         void *ctx, pair_cb cb) {
    if (n < 2) return;
    hbox *hb = (hbox *)malloc(sizeof(hbox) * n);
    int *big = (int *)malloc(sizeof(int) * n);
    int nh = 0, nbig = 0, i;
    int maxlevel = minlevel - 1;
    for (int k = 0; k < n; k++) {
        int g = order[k];
        const real *ab = aabbs + 6 * g;
        int level = find_level(ab);
        if (level < minlevel) level = minlevel;
        if (level <= maxlevel_g) {
            hbox *h = &hb[nh];
            h->geom = g;
            h->level = level;
            if (level > maxlevel) maxlevel = level;
            real csr = (real)(1.0f / ldexp(1.0f, level));
            for (i = 0; i < 6; i++) h->db[i] = (int)floorf(ab[i] * csr);
            h->index = (size_t)nh;
            nh++;
        } else {
            big[nbig++] = g;
        }
    }
    int tested_rowsize = (nh + 7) >> 3;
    unsigned char *tested = (unsigned char *)calloc((size_t)nh * tested_rowsize + 1, 1);
    for (i = 0; i < 31; i++) if ((size_t)primes[i] >= (size_t)(8 * nh)) break;
    if (i >= 31) i = 30;
    const unsigned long sz = primes[i];
    int *table = (int *)malloc(sizeof(int) * sz);
    for (unsigned long t = 0; t < sz; t++) table[t] = -1;
    size_t ncap = 16, nn = 0;
    hnode *nodes = (hnode *)malloc(sizeof(hnode) * ncap);
    for (int b = 0; b < nh; b++) {
        const int *db = hb[b].db;
        for (int xi = db[0]; xi <= db[1]; xi++) {
            for (int yi = db[2]; yi <= db[3]; yi++) {
                int zbegin = db[4];
                unsigned long hi = ((unsigned long)(unsigned)hb[b].level * 1000UL + (unsigned long)(unsigned)xi * 100UL +
                                    (unsigned long)(unsigned)yi * 10UL + (unsigned long)(long)zbegin) % sz;
                for (int zi = zbegin; zi <= db[5]; (hi = hi + 1U != sz ? hi + 1U : 0UL), zi++) {
                    if (nn == ncap) { ncap *= 2; nodes = (hnode *)realloc(nodes, sizeof(hnode) * ncap); }
                    nodes[nn].x = xi; nodes[nn].y = yi; nodes[nn].z = zi; nodes[nn].box = b;
                    nodes[nn].next = table[hi];
                    table[hi] = (int)nn;
                    nn++;
                }
            }
        }
    }
    int db[6];
    for (int b = 0; b < nh; b++) {
        for (i = 0; i < 6; i++) db[i] = hb[b].db[i];
        for (int level = hb[b].level;;) {
            for (int xi = db[0]; xi <= db[1]; xi++) {
                for (int yi = db[2]; yi <= db[3]; yi++) {
                    int zbegin = db[4];
                    unsigned long hi = ((unsigned long)(unsigned)level * 1000UL + (unsigned long)(unsigned)xi * 100UL +
                                        (unsigned long)(unsigned)yi * 10UL + (unsigned long)(long)zbegin) % sz;
                    for (int zi = zbegin; zi <= db[5]; (hi = hi + 1U != sz ? hi + 1U : 0UL), zi++) {
                        for (int nd = table[hi]; nd >= 0; nd = nodes[nd].next) {
                            int ob = nodes[nd].box;
                            if (ob == b) continue;
                            if (hb[ob].level == level && nodes[nd].x == xi && nodes[nd].y == yi && nodes[nd].z == zi) {
                                size_t idx;
                                unsigned char mask;
                                if (hb[b].index <= hb[ob].index) {
                                    idx = hb[b].index * tested_rowsize + (hb[ob].index >> 3);
                                    mask = (unsigned char)(1 << (hb[ob].index & 7));
                                } else {
                                    idx = hb[ob].index * tested_rowsize + (hb[b].index >> 3);
                                    mask = (unsigned char)(1 << (hb[b].index & 7));
                                }
                                if ((tested[idx] & mask) == 0) {
                                    tested[idx] |= mask;
                                    collide_aabbs(hb[b].geom, hb[ob].geom, body, aabbs, ctx, cb);
                                }
                            }
                        }
                    }
                }
            }
            if (level == maxlevel) break;
            ++level;
            for (i = 0; i < 6; i++) db[i] >>= 1;
        }
    }
    for (int b = 0; b < nh; b++)
        for (int k = 0; k < nbig; k++) collide_aabbs(hb[b].geom, big[k], body, aabbs, ctx, cb);
    for (int a = 0; a < nbig; a++)
        for (int k = a + 1; k < nbig; k++) collide_aabbs(big[a], big[k], body, aabbs, ctx, cb);
    free(nodes); free(table); free(tested); free(big); free(hb);
}

typedef struct { int *pairs; int cap; int n; } pair_sink;
static void sink_cb(void *ctx, int g1, int g2) {
    pair_sink *s = (pair_sink *)ctx;
    if (s->n < s->cap) { s->pairs[2 * s->n] = g1; s->pairs[2 * s->n + 1] = g2; }
    s->n++;
}

int port_hash_pairs(int n, const int *cls, const int *body, const float *pos, const float *R, const float *dims,
                    const int *order, int minlevel, int maxlevel, int *pairs, int cap) {
    real *aabbs = (real *)malloc(sizeof(real) * 6 * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        pgeom g;
        make_pgeom(&g, cls[i], pos + 3 * i, R + 12 * i, dims + 4 * i);
        compute_aabb(&g, aabbs + 6 * i);
    }
    pair_sink s = {pairs, cap, 0};
    hash_collide(n, order, body, aabbs, minlevel, maxlevel, &s, sink_cb);
    free(aabbs);
    return s.n;
}

/* ------------------------------------------------------------- world */
typedef struct {
    real pos[4], q[4], R[12], lvel[4], avel[4], facc[4], tacc[4];
    real mass, invMass;
    real I[12], invI[12];
    int gyro;
} pbody;

struct port_world {
    int nb;
    pbody *b;
    real dt, g[3], erp, cfm, w, max_vel, min_depth;
    int iterations, reorder;
    real premature_delta, extra_delta;
    unsigned max_extra;
    int dyn_enabled;
    int threads;       /* SOR threads (1: the reference's default self-threaded stepping) */
    int mt_min_rows;   /* islands with fewer rows iterate on one thread */
    int resid_on;      /* evaluate each step's FP64 LCP residual (test / benchmark bookkeeping) */
    double res_max, lam_max;  /* of the last step: max natural-map residual, max |lambda| */
};

/* contact joint as dJointCreateContact + dJointAttach leave it (ode.cpp:1192-1200, 1383-1439) */
typedef struct {
    int node0, node1;  /* body indices after attach (node1 may be -1) */
    int reverse;
    int mode;
    real mu, mu2, rho, rho2, rhoN, bounce, bounce_vel, soft_erp, soft_cfm, motion1, motion2, motionN, slip1, slip2;
    real pos[3], normal[3], depth, fdir1[3];
    int m;
} pjoint;

/* matrix.cpp dxFactorCholesky / dxSolveCholesky / dxInvertPDMatrix for n = 3
 * (row stride 4), as dBodySetMass (ode.cpp:488-505) uses them for invI. */
static int invert_pd3(const real *A, real *Ainv) {
    real L[12], recip[3], X[3], y[3];
    memcpy(L, A, sizeof L);
    for (int i = 0; i < 3; i++) {
        real *aa = L + 4 * i;
        for (int j = 0; j < i; j++) {
            real sum = aa[j];
            const real *bb = L + 4 * j;
            for (int k = 0; k < j; k++) sum -= aa[k] * bb[k];
            aa[j] = sum * recip[j];
        }
        real sum = aa[i];
        for (int k = 0; k < i; k++) sum -= aa[k] * aa[k];
        if (sum <= 0.0f) return 0;
        real sq = sqrtf(sum);
        aa[i] = sq;
        recip[i] = 1.0f / sq;
    }
    memset(Ainv, 0, 12 * sizeof(real));
    for (int c = 0; c < 3; c++) {
        X[0] = X[1] = X[2] = 0; X[c] = 1.0f;
        for (int i = 0; i < 3; i++) {
            real sum = 0.0f;
            for (int k = 0; k < i; k++) sum += L[4 * i + k] * y[k];
            y[i] = (X[i] - sum) / L[4 * i + i];
        }
        for (int i = 2; i >= 0; i--) {
            real sum = 0.0f;
            for (int k = i + 1; k < 3; k++) sum += L[4 * k + i] * X[k];
            X[i] = (y[i] - sum) / L[4 * i + i];
        }
        for (int k = 0; k < 3; k++) Ainv[4 * k + c] = X[k];
    }
    return 1;
}

/* mass.cpp dMassSetParameters + ode.cpp:488-505 dBodySetMass */
static void set_mass(pbody *b, real mass, const real *I6) {
    b->mass = mass;
    memset(b->I, 0, sizeof b->I);
    b->I[0] = I6[0]; b->I[5] = I6[1]; b->I[10] = I6[2];
    b->I[1] = b->I[4] = I6[3]; b->I[2] = b->I[8] = I6[4]; b->I[6] = b->I[9] = I6[5];
    if (!invert_pd3(b->I, b->invI)) {
        memset(b->invI, 0, sizeof b->invI);
        b->invI[0] = b->invI[5] = b->invI[10] = 1.0f;
    }
    b->invMass = 1.0f / mass;
}

port_world *port_world_create(int nb, const float *bin, const float *params, int iterations, int dyn, int reorder) {
    port_world *w = (port_world *)calloc(1, sizeof(port_world));
    w->nb = nb;
    w->b = (pbody *)calloc(nb > 0 ? nb : 1, sizeof(pbody));
    w->dt = params[0]; w->g[0] = params[1]; w->g[1] = params[2]; w->g[2] = params[3];
    w->erp = params[4]; w->cfm = params[5]; w->w = params[6]; w->max_vel = params[7]; w->min_depth = params[8];
    w->iterations = iterations;
    w->reorder = reorder;
    w->threads = 1;
    w->mt_min_rows = 4096;
    /* objects.h:451-475 defaults; objects.cpp:78-91 */
    w->premature_delta = dyn ? 1e-8f : 0.0f;
    w->extra_delta = 1e-2f;
    w->max_extra = dyn ? (unsigned)((real)iterations * 1.0f) : 0;
    w->dyn_enabled = w->max_extra != 0 || w->premature_delta != 0;
    for (int i = 0; i < nb; i++) {
        pbody *b = &w->b[i];
        const float *s = bin + 20 * i;
        b->pos[0] = s[0]; b->pos[1] = s[1]; b->pos[2] = s[2];
        b->q[0] = s[3]; b->q[1] = s[4]; b->q[2] = s[5]; b->q[3] = s[6];
        normalize4(b->q);                 /* ode.cpp:379-387 dBodySetQuaternion */
        r_from_q(b->R, b->q);
        b->lvel[0] = s[7]; b->lvel[1] = s[8]; b->lvel[2] = s[9];
        b->avel[0] = s[10]; b->avel[1] = s[11]; b->avel[2] = s[12];
        set_mass(b, s[13], s + 14);
        b->gyro = 1;                      /* ode.cpp:283 */
    }
    return w;
}

void port_world_destroy(port_world *w) { if (w) { free(w->b); free(w); } }

void port_world_set_dyn(port_world *w, float premature, float extra_factor, float extra_delta) {
    w->premature_delta = premature;
    w->extra_delta = extra_delta;
    w->max_extra = (unsigned)((real)w->iterations * extra_factor);
    w->dyn_enabled = w->max_extra != 0 || w->premature_delta != 0;
}

void port_world_set_threads(port_world *w, int threads, int min_rows) {
    w->threads = threads > 1 ? threads : 1;
    w->mt_min_rows = min_rows > 0 ? min_rows : 1;
}

void port_world_get(const port_world *w, float *out) {
    for (int i = 0; i < w->nb; i++) {
        const pbody *b = &w->b[i];
        float *o = out + 25 * i;
        memcpy(o, b->pos, 3 * sizeof(float));
        memcpy(o + 3, b->q, 4 * sizeof(float));
        memcpy(o + 7, b->R, 12 * sizeof(float));
        memcpy(o + 19, b->lvel, 3 * sizeof(float));
        memcpy(o + 22, b->avel, 3 * sizeof(float));
    }
}

void port_world_set_state(port_world *w, const float *st) {
    for (int i = 0; i < w->nb; i++) {
        pbody *b = &w->b[i];
        const float *o = st + 25 * i;
        memcpy(b->pos, o, 3 * sizeof(float));
        memcpy(b->q, o + 3, 4 * sizeof(float));
        memcpy(b->R, o + 7, 12 * sizeof(float));
        memcpy(b->lvel, o + 19, 3 * sizeof(float));
        memcpy(b->avel, o + 22, 3 * sizeof(float));
    }
}

/* util.cpp:583-692 dxStepBody (no finite rotation, no damping, no speed cap) */
static void step_body(pbody *b, real h) {
    for (int j = 0; j < 3; j++) b->pos[j] += h * b->lvel[j];
    real dq[4];
    const real *w = b->avel, *q = b->q;
    dq[0] = 0.5f * (-w[0] * q[1] - w[1] * q[2] - w[2] * q[3]);
    dq[1] = 0.5f * (w[0] * q[0] + w[1] * q[3] - w[2] * q[2]);
    dq[2] = 0.5f * (-w[0] * q[3] + w[1] * q[0] + w[2] * q[1]);
    dq[3] = 0.5f * (w[0] * q[2] - w[1] * q[1] + w[2] * q[0]);
    for (int j = 0; j < 4; j++) b->q[j] += h * dq[j];
    normalize4(b->q);
    r_from_q(b->R, b->q);
}

/* joints/contact.cpp:49-122 getInfo1 (non-AxisDep, no rolling handled as in reference) */
static int contact_info1(pjoint *j) {
    int m = 1;
    if (j->mode & 0x001 /* dContactAxisDep */) {
        if (j->mu < 0) j->mu = 0; else if (j->mu > 0) m++;
        if (j->mu2 < 0) j->mu2 = 0; else if (j->mu2 > 0) m++;
        if (j->mode & 0x400) {
            if (j->rho < 0) j->rho = 0; else m++;
            if (j->rho2 < 0) j->rho2 = 0; else m++;
            if (j->rhoN < 0) j->rhoN = 0; else m++;
        }
    } else {
        if (j->mu < 0) j->mu = 0; else if (j->mu > 0) m += 2;
        if (j->mode & 0x400) {
            if (j->rho < 0) j->rho = 0; else m += 3;
        }
    }
    j->m = m;
    return m;
}

/* joints/contact.cpp:126-347 getInfo2 (rows: J1 6 rhs cfm J2 6 lo hi in a 16-stride) */
static void contact_info2(const port_world *w, pjoint *j, real fps, real erp_world, real *J, int *findex) {
    const pbody *bodies = w->b;
    const int mode = j->mode;
    real erp = (mode & 0x008) ? j->soft_erp : erp_world;
    real k = fps * erp;
    real depth = j->depth - w->min_depth;
    if (depth < 0) depth = 0;
    real motionN = (mode & 0x080) ? j->motionN : 0.0f;
    const real pushout = k * depth + motionN;
    int apply_bounce = (mode & 0x004) != 0 && j->bounce_vel >= 0;
    real outgoing = 0;
    const real maxvel = w->max_vel;
    real c = pushout > maxvel ? maxvel : pushout;
    real c1[3], c2[3] = {0, 0, 0}, normal[3];
    if (j->reverse) { normal[0] = -j->normal[0]; normal[1] = -j->normal[1]; normal[2] = -j->normal[2]; }
    else { normal[0] = j->normal[0]; normal[1] = j->normal[1]; normal[2] = j->normal[2]; }
    real *J1 = J, *J2 = J + 8;
    if (j->node1 >= 0) {
        const pbody *b1 = &bodies[j->node1];
        c2[0] = j->pos[0] - b1->pos[0]; c2[1] = j->pos[1] - b1->pos[1]; c2[2] = j->pos[2] - b1->pos[2];
        J2[0] = -normal[0]; J2[1] = -normal[1]; J2[2] = -normal[2];
        cross3(J2 + 3, normal, c2);
        if (apply_bounce) outgoing = dot3(J2 + 3, b1->avel) - dot3(normal, b1->lvel);
    }
    const pbody *b0 = &bodies[j->node0];
    c1[0] = j->pos[0] - b0->pos[0]; c1[1] = j->pos[1] - b0->pos[1]; c1[2] = j->pos[2] - b0->pos[2];
    J1[0] = normal[0]; J1[1] = normal[1]; J1[2] = normal[2];
    cross3(J1 + 3, c1, normal);
    if (apply_bounce) outgoing += dot3(J1 + 3, b0->avel) + dot3(normal, b0->lvel);
    if (apply_bounce) {
        real negated_outgoing = motionN - outgoing;
        if (negated_outgoing > j->bounce_vel) {
            const real newc = j->bounce * negated_outgoing + motionN;
            if (newc > c) c = newc;
        }
    }
    J[6] = c;
    if (mode & 0x010) J[7] = j->soft_cfm;
    J[14] = 0; J[15] = INF;
    if (j->m > 1) {
        real t1[3], t2[3];
        if (mode & 0x002) {
            t1[0] = j->fdir1[0]; t1[1] = j->fdir1[1]; t1[2] = j->fdir1[2];
            cross3(t2, normal, t1);
        } else {
            plane_space(normal, t1, t2);
        }
        int row = 1;
        const real mu = j->mu;
        if (mu > 0) {
            real *r = J + 16 * row;
            r[0] = t1[0]; r[1] = t1[1]; r[2] = t1[2];
            cross3(r + 3, c1, t1);
            if (j->node1 >= 0) {
                r[8] = -t1[0]; r[9] = -t1[1]; r[10] = -t1[2];
                cross3(r + 11, t1, c2);
            }
            if (mode & 0x020) r[6] = j->motion1;
            if (mode & 0x100) r[7] = j->slip1;
            r[14] = -mu; r[15] = mu;
            if (mode & 0x1000) findex[row] = 0;
            ++row;
        }
        const real mu2 = (mode & 0x001) ? j->mu2 : mu;
        if (mu2 > 0) {
            real *r = J + 16 * row;
            r[0] = t2[0]; r[1] = t2[1]; r[2] = t2[2];
            cross3(r + 3, c1, t2);
            if (j->node1 >= 0) {
                r[8] = -t2[0]; r[9] = -t2[1]; r[10] = -t2[2];
                cross3(r + 11, t2, c2);
            }
            if (mode & 0x040) r[6] = j->motion2;
            if (mode & 0x200) r[7] = j->slip2;
            r[14] = -mu2; r[15] = mu2;
            if (mode & 0x2000) findex[row] = 0;
            ++row;
        }
        if (mode & 0x400) {
            const real *ax[3] = {t1, t2, normal};
            const int approx_bits[3] = {0x1000, 0x2000, 0x4000};
            real rho[3];
            rho[0] = j->rho;
            if (mode & 0x001) { rho[1] = j->rho2; rho[2] = j->rhoN; }
            else { rho[1] = rho[0]; rho[2] = rho[0]; }
            for (int i = 0; i != 3; ++i) {
                if (rho[i] > 0) {
                    real *r = J + 16 * row;
                    r[3] = ax[i][0]; r[4] = ax[i][1]; r[5] = ax[i][2];
                    if (j->node1 >= 0) { r[11] = -ax[i][0]; r[12] = -ax[i][1]; r[13] = -ax[i][2]; }
                    r[14] = -rho[i]; r[15] = rho[i];
                    if (mode & approx_bits[i]) findex[row] = 0;
                    ++row;
                }
            }
        }
    }
}

/* quickstep.cpp:1112-3439 dxQuickStepIsland, single-threaded path.
 * body_ids/joint_ids: the island in DFS order; rows_out/lambda in joint terms. */
/* ------------------------------------------------------------------ SOR */
/* The rows of one island as the SOR sweep reads them. */
typedef struct {
    const real *J, *iMJ;
    const int *jb1, *jb2, *findex;
    real *lambda, *fc, *fa;
} sor_rows;

/* Stage4LCP_IterationStep (quickstep.cpp:2917-3033): one row's projected
 * Gauss-Seidel update of lambda and of its bodies' fc (and the dynamic
 * iteration's per-body maximum adjustments fa). */
static inline void sor_row(const sor_rows *S, int index) {
    const real *Jr = S->J + 16 * index;
    real *lambda = S->lambda;
    real old_lambda = lambda[index];
    real delta = Jr[6] - old_lambda * Jr[7];
    int b1 = S->jb1[index], b2 = S->jb2[index];
    real *f1 = S->fc + 6 * b1, *f2 = NULL;
    delta -= f1[0] * Jr[0] + f1[1] * Jr[1] + f1[2] * Jr[2] + f1[3] * Jr[3] + f1[4] * Jr[4] + f1[5] * Jr[5];
    if (b2 != -1) {
        f2 = S->fc + 6 * b2;
        delta -= f2[0] * Jr[8] + f2[1] * Jr[9] + f2[2] * Jr[10] + f2[3] * Jr[11] + f2[4] * Jr[12] + f2[5] * Jr[13];
    }
    real hi_act, lo_act;
    const int fi = S->findex[index];
    if (fi != -1) { hi_act = fabsf(Jr[15] * lambda[fi]); lo_act = -hi_act; }
    else { hi_act = Jr[15]; lo_act = Jr[14]; }
    real new_lambda = old_lambda + delta;
    if (new_lambda < lo_act) { delta = lo_act - old_lambda; lambda[index] = lo_act; }
    else if (new_lambda > hi_act) { delta = hi_act - old_lambda; lambda[index] = hi_act; }
    else lambda[index] = new_lambda;
    if (delta != 0) {
        const real *o = S->iMJ + 14 * index;
        int pos_ = delta > 0;
        for (int k = 0; k < 6; k++) f1[k] += delta * o[k];
        S->fa[2 * b1 + pos_] += delta * o[6];
        if (f2) {
            S->fa[2 * b2 + pos_] += delta * o[13];
            for (int k = 0; k < 6; k++) f2[k] += delta * o[7 + k];
        }
    }
}

/* IsSORConstraintsReorderRequiredForIteration (quickstep.cpp:1080-1109) and
 * the random shuffle of ConstraintsShuffling (quickstep.cpp:2578-2618). */
static int sor_reorder_due(const port_world *w, unsigned iteration) {
    return w->reorder == 1 && iteration >= 8u && iteration % 8u == 0u;
}
static void sor_shuffle(int *order, int m) {
    for (int idx = 1; idx < m; ++idx) {
        int sw = port_rand_int(idx + 1);
        int t = order[idx]; order[idx] = order[sw]; order[sw] = t;
    }
}

/* The iteration driver's exit rule (quickstep.cpp:1823-1856) and the dynamic
 * iteration check (CheckForMaximumToBeLessThanLimitAndResetMaxAdjustments,
 * quickstep.cpp:3253-3285), after one sweep: 1 when the sweeps end. */
typedef struct { unsigned iteration, extra; real premature; } sor_driver;
static int sor_after_sweep(const port_world *w, sor_driver *d, real *fa, int nb) {
    ++d->iteration;
    if (d->iteration - d->extra == (unsigned)w->iterations) {
        if (d->extra != 0 || w->max_extra == 0) return 1;
        d->extra = w->max_extra;
        d->premature = w->extra_delta;
    }
    if (w->dyn_enabled) {
        int hit = 0;
        if (d->premature == 0) { memset(fa, 0, sizeof(real) * 2 * nb); hit = 1; }
        else {
            for (int i = 0; i < nb; i++) {
                if (!(fa[2 * i + 1] < d->premature) || !(-fa[2 * i] < d->premature)) {
                    memset(fa + 2 * i, 0, sizeof(real) * 2 * (nb - i));
                    hit = 1;
                    break;
                }
                fa[2 * i] = 0; fa[2 * i + 1] = 0;
            }
        }
        if (!hit) return 1;
    }
    return 0;
}

/* Multi-threaded sweeps: the reference's opt-in threaded iteration
 * (dWorldSetStepThreadingImplementation, ode.cpp:1814-1825; the dependency
 * map of quickstep.cpp:2661-2742 and MTIteration, :2807-2890) runs a row once
 * the rows before it in the order that share one of its bodies have run.  This
 * restatement groups the rows of an order into levels -- a row's level is one
 * above the highest level of the earlier rows on its bodies, so the rows of a
 * level share no body -- and runs the levels one after another, each level's
 * rows split over the threads, with a spin barrier between levels.  A
 * friction row's normal row belongs to the same contact, so it is ordered by
 * the shared bodies too.  Every row then reads the body accumulators the
 * sequential order gives it: the multipliers are the sequential ones to the
 * bit (the reference's tree releases a row after the later of its two
 * predecessors only, and waits for fewer).  The level map is rebuilt by one
 * thread after every reorder, as the reference rebuilds its map. */
typedef struct {
    sor_rows S;
    const port_world *w;
    int m, nb, nthreads;
    int *order, *lev_start, *lev_rows, *lev_of, *blev;
    int nlev, serial;
    sor_driver drv;
    int stop;
    atomic_int bar_count, bar_sense, go;
} sor_mt;

typedef struct { sor_mt *C; int tid; } sor_mt_arg;

static void sor_barrier(sor_mt *C, int *sense) {
    const int s = !*sense;
    *sense = s;
    if (atomic_fetch_add(&C->bar_count, 1) == C->nthreads - 1) {
        atomic_store(&C->bar_count, 0);
        atomic_store(&C->bar_sense, s);
    } else {
        /* spin, then give the core away: with more threads than free cores a
         * pure spin would wait for a descheduled thread's whole time slice */
        for (unsigned spins = 0; atomic_load(&C->bar_sense) != s; spins++)
            if (spins >= 2048u) sched_yield();
    }
}

static void sor_levels(sor_mt *C) {
    const int m = C->m;
    memset(C->blev, 0, sizeof(int) * (C->nb > 0 ? C->nb : 1));
    int nlev = 0;
    for (int ii = 0; ii < m; ii++) {
        const int index = C->order[ii];
        const int b1 = C->S.jb1[index], b2 = C->S.jb2[index];
        int l = C->blev[b1];
        if (b2 != -1 && C->blev[b2] > l) l = C->blev[b2];
        C->blev[b1] = l + 1;
        if (b2 != -1) C->blev[b2] = l + 1;
        C->lev_of[index] = l;
        if (l + 1 > nlev) nlev = l + 1;
    }
    memset(C->lev_start, 0, sizeof(int) * (nlev + 1));
    for (int r = 0; r < m; r++) C->lev_start[C->lev_of[r] + 1]++;
    for (int l = 0; l < nlev; l++) C->lev_start[l + 1] += C->lev_start[l];
    /* a level's rows are independent: they are listed by row index (the
     * order of memory), lev_start[l] running to the end of level l */
    for (int r = 0; r < m; r++) C->lev_rows[C->lev_start[C->lev_of[r]]++] = r;
    for (int l = nlev; l > 0; l--) C->lev_start[l] = C->lev_start[l - 1];
    C->lev_start[0] = 0;
    C->nlev = nlev;
    /* an order whose levels hold fewer than 8 rows a thread on average (the
     * initial order: contacts of a body next to each other, chained through
     * their bodies) is swept by one thread in order */
    C->serial = (long long)nlev * 8 * C->nthreads > (long long)m;
}

static void *sor_mt_run(void *argp) {
    sor_mt_arg *a = (sor_mt_arg *)argp;
    sor_mt *C = a->C;
    while (!atomic_load(&C->go)) sched_yield();
    const int tid = a->tid, T = C->nthreads;
    int sense = 0;
    for (;;) {
        if (C->serial) {
            if (tid == 0)
                for (int ii = 0; ii < C->m; ii++) sor_row(&C->S, C->order[ii]);
            sor_barrier(C, &sense);
        } else {
            for (int l = 0; l < C->nlev; l++) {
                const int s0 = C->lev_start[l], n = C->lev_start[l + 1] - s0;
                const int lo = s0 + (int)((long long)n * tid / T), hi = s0 + (int)((long long)n * (tid + 1) / T);
                for (int k = lo; k < hi; k++) sor_row(&C->S, C->lev_rows[k]);
                sor_barrier(C, &sense);
            }
        }
        if (tid == 0) {
            C->stop = sor_after_sweep(C->w, &C->drv, C->S.fa, C->nb);
            if (!C->stop && sor_reorder_due(C->w, C->drv.iteration)) {
                sor_shuffle(C->order, C->m);
                sor_levels(C);
            }
        }
        sor_barrier(C, &sense);
        if (C->stop) break;
    }
    return NULL;
}

static void sor_sweeps_mt(const port_world *w, const sor_rows *S, int *order, int m, int nb) {
    sor_mt C;
    memset(&C, 0, sizeof C);
    C.S = *S;
    C.w = w;
    C.m = m;
    C.nb = nb;
    C.nthreads = w->threads;
    C.order = order;
    C.lev_start = (int *)malloc(sizeof(int) * (m + 2));
    C.lev_rows = (int *)malloc(sizeof(int) * (m + 1));
    C.lev_of = (int *)malloc(sizeof(int) * (m + 1));
    C.blev = (int *)malloc(sizeof(int) * (nb + 1));
    C.drv.premature = w->premature_delta;
    atomic_init(&C.bar_count, 0);
    atomic_init(&C.bar_sense, 0);
    atomic_init(&C.go, 0);
    const int asked = w->threads;
    sor_mt_arg *args = (sor_mt_arg *)malloc(sizeof(sor_mt_arg) * asked);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * asked);
    int started = 1;
    for (int t = 0; t < asked; t++) { args[t].C = &C; args[t].tid = t; }
    for (int t = 1; t < asked; t++) {
        if (pthread_create(&th[t], NULL, sor_mt_run, &args[t]) != 0) break;
        started++;
    }
    /* the threads read the count only after the gate opens: a failed
     * pthread_create leaves fewer threads, with tids 0 .. started-1 */
    C.nthreads = started;
    sor_levels(&C);
    atomic_store(&C.go, 1);
    sor_mt_run(&args[0]);
    for (int t = 1; t < started; t++) pthread_join(th[t], NULL);
    free(th); free(args);
    free(C.blev); free(C.lev_of); free(C.lev_rows); free(C.lev_start);
}

/* FP64 natural-map residual of one island's solution (unscaled rows Ju:
 * J1 0-5, rhs 6, cfm 7, J2 8-13, lo 14, hi 15; findex island-local), the
 * definition of port_lcp_residual, folded into w->res_max / w->lam_max. */
static void island_residual(port_world *w, const real *Ju, int m, const int *jb1, const int *jb2,
                            const int *findex, const real *lambda, const int *body_ids, int nb, const real *invI) {
    double *f = (double *)calloc((size_t)6 * (nb > 0 ? nb : 1), sizeof(double));
    double *v = (double *)calloc((size_t)6 * (nb > 0 ? nb : 1), sizeof(double));
    for (int i = 0; i < m; i++) {
        const real *r = Ju + 16 * i;
        for (int k = 0; k < 6; k++) f[6 * jb1[i] + k] += (double)r[k] * lambda[i];
        if (jb2[i] != -1) for (int k = 0; k < 6; k++) f[6 * jb2[i] + k] += (double)r[8 + k] * lambda[i];
    }
    for (int b = 0; b < nb; b++) {
        const double im = w->b[body_ids[b]].invMass;
        const real *I = invI + 12 * b;
        for (int k = 0; k < 3; k++) v[6 * b + k] = im * f[6 * b + k];
        for (int k = 0; k < 3; k++)
            v[6 * b + 3 + k] = (double)I[4 * k] * f[6 * b + 3] + (double)I[4 * k + 1] * f[6 * b + 4] +
                               (double)I[4 * k + 2] * f[6 * b + 5];
    }
    for (int i = 0; i < m; i++) {
        const real *r = Ju + 16 * i;
        double Av = 0, D = 0;
        const int b1 = jb1[i], b2 = jb2[i];
        for (int k = 0; k < 6; k++) Av += (double)r[k] * v[6 * b1 + k];
        const double im1 = w->b[body_ids[b1]].invMass;
        for (int k = 0; k < 3; k++) D += (double)r[k] * r[k] * im1;
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) D += (double)r[3 + a] * invI[12 * b1 + 4 * a + c] * r[3 + c];
        if (b2 != -1) {
            for (int k = 0; k < 6; k++) Av += (double)r[8 + k] * v[6 * b2 + k];
            const double im2 = w->b[body_ids[b2]].invMass;
            for (int k = 0; k < 3; k++) D += (double)r[8 + k] * r[8 + k] * im2;
            for (int a = 0; a < 3; a++)
                for (int c = 0; c < 3; c++) D += (double)r[11 + a] * invI[12 * b2 + 4 * a + c] * r[11 + c];
        }
        const double cfm = r[7], li = lambda[i];
        const double wi = Av + cfm * li - r[6];
        D += cfm;
        double lo, hi;
        if (findex[i] >= 0) { hi = fabs((double)r[15] * lambda[findex[i]]); lo = -hi; }
        else { lo = r[14]; hi = r[15]; }
        double t = li - wi / D;
        if (t < lo) t = lo;
        if (t > hi) t = hi;
        if (fabs(li - t) > w->res_max) w->res_max = fabs(li - t);
        if (fabs(li) > w->lam_max) w->lam_max = fabs(li);
    }
    free(f); free(v);
}

/* set only while port_world_quickstep_map runs: receives each recorded row's contact slot */
static int *g_row_slot = NULL;

static void quickstep_island(port_world *w, const int *body_ids, int nb, pjoint *joints, const int *joint_ids,
                             int nj_in, const int *joint_cidx, float *lambda_out, float *rows_out, int row_base) {
    const real h = w->dt;
    int *tag = (int *)malloc(sizeof(int) * (w->nb > 0 ? w->nb : 1));
    for (int i = 0; i < nb; i++) tag[body_ids[i]] = i;
    /* Stage0_Bodies :1176-1306 */
    for (int ax = 0; ax < 3; ax++) {
        real g = w->g[ax];
        if (g) for (int i = 0; i < nb; i++) { pbody *b = &w->b[body_ids[i]]; b->facc[ax] += b->mass * g; }
    }
    real *invI = (real *)calloc((size_t)12 * (nb > 0 ? nb : 1), sizeof(real));
    for (int i = 0; i < nb; i++) {
        pbody *b = &w->b[body_ids[i]];
        real tmp[12];
        mul2_333(tmp, b->invI, b->R);
        mul0_333(invI + 12 * i, b->R, tmp);
        if (b->gyro && b->invMass > 0) {
            real I[12];
            mul2_333(tmp, b->I, b->R);
            mul0_333(I, b->R, tmp);
            I[3] = I[7] = I[11] = 0;
            real L[3];
            mul0_331(L, I, b->avel);
            real Itild[12] = {0};
            Itild[1] = +L[2]; Itild[2] = -L[1]; Itild[4] = -L[2]; Itild[6] = +L[0]; Itild[8] = +L[1]; Itild[9] = -L[0];
            for (int ii = 0; ii < 12; ++ii) Itild[ii] = Itild[ii] * h + I[ii];
            real rh = 1.0f / h;
            L[0] *= rh; L[1] *= rh; L[2] *= rh;
            real itInv[12] = {0};
            if (invert3(itInv, Itild) != 0) {
                mul0_333(Itild, I, itInv);
                Itild[0] -= 1; Itild[5] -= 1; Itild[10] -= 1;
                real tau0[3];
                mul0_331(tau0, Itild, L);
                b->tacc[0] = b->tacc[0] + tau0[0]; b->tacc[1] = b->tacc[1] + tau0[1]; b->tacc[2] = b->tacc[2] + tau0[2];
            }
        }
    }
    /* Stage0_Joints / Stage1 :1319-1472 */
    int nj = 0, m = 0;
    int *jl = (int *)malloc(sizeof(int) * (nj_in > 0 ? nj_in : 1));
    int *mindex = (int *)malloc(sizeof(int) * (nj_in + 1));
    for (int k = 0; k < nj_in; k++) {
        pjoint *j = &joints[joint_ids[k]];
        int jm = contact_info1(j);
        if (jm) { jl[nj] = joint_ids[k]; mindex[nj] = m; m += jm; nj++; }
    }
    mindex[nj] = m;
    if (m > 0) {
        real *J = (real *)calloc((size_t)16 * m, sizeof(real));
        int *findex = (int *)malloc(sizeof(int) * m);
        int *jb1 = (int *)malloc(sizeof(int) * m), *jb2 = (int *)malloc(sizeof(int) * m);
        const real rh = 1.0f / h;
        int valid_findices = 0;
        /* Stage2a :1486-1610 */
        for (int ji = 0; ji < nj; ji++) {
            int ofs = mindex[ji], im = mindex[ji + 1] - ofs;
            real *JR = J + 16 * ofs;
            for (int r = 0; r < im; r++) {
                real *Jc = JR + 16 * r;
                memset(Jc, 0, 16 * sizeof(real));
                Jc[7] = w->cfm; Jc[14] = -INF; Jc[15] = INF;
                findex[ofs + r] = -1;
            }
            pjoint *j = &joints[jl[ji]];
            contact_info2(w, j, rh, w->erp, JR, findex + ofs);
            for (int r = 0; r < im; r++)
                if (findex[ofs + r] != -1) { findex[ofs + r] += ofs; valid_findices++; }
            for (int r = 0; r < im; r++) { JR[16 * r + 6] *= rh; JR[16 * r + 7] *= rh; }
            int b1 = tag[j->node0], b2 = j->node1 >= 0 ? tag[j->node1] : -1;
            for (int r = 0; r < im; r++) { jb1[ofs + r] = b1; jb2[ofs + r] = b2; }
        }
        /* Stage2b :1644-1690 */
        real *rhs_tmp = (real *)malloc(sizeof(real) * 6 * nb);
        for (int i = 0; i < nb; i++) {
            pbody *b = &w->b[body_ids[i]];
            real *rc = rhs_tmp + 6 * i;
            for (int k = 0; k < 3; k++) rc[k] = -(b->facc[k] * b->invMass + b->lvel[k] * rh);
            mul0_331(rc + 3, invI + 12 * i, b->tacc);
            for (int k = 0; k < 3; k++) rc[3 + k] = -(b->avel[k] * rh) - rc[3 + k];
        }
        /* Stage2c :1727-1747 multiplyAdd_J */
        for (int i = 0; i < m; i++) {
            real *Jr = J + 16 * i;
            real sum = 0;
            const real *in = rhs_tmp + 6 * jb1[i];
            for (int k = 0; k < 6; k++) sum += Jr[k] * in[k];
            if (jb2[i] != -1) {
                in = rhs_tmp + 6 * jb2[i];
                for (int k = 0; k < 6; k++) sum += Jr[8 + k] * in[k];
            }
            Jr[6] += sum;
        }
        /* the unscaled rows, for the step's FP64 residual after the solve */
        real *Ju = NULL;
        if (w->resid_on) {
            Ju = (real *)malloc(sizeof(real) * 16 * (m > 0 ? m : 1));
            memcpy(Ju, J, sizeof(real) * 16 * m);
        }
        if (rows_out) {
            for (int i = 0; i < m; i++) {
                float *o = rows_out + 20 * i;
                const real *Jr = J + 16 * i;
                for (int k = 0; k < 6; k++) { o[k] = Jr[k]; o[6 + k] = Jr[8 + k]; }
                o[12] = Jr[6]; o[13] = Jr[7]; o[14] = Jr[14]; o[15] = Jr[15];
                o[16] = (float)body_ids[jb1[i]];
                o[17] = jb2[i] >= 0 ? (float)body_ids[jb2[i]] : -1.0f;
                o[18] = findex[i] >= 0 ? (float)(findex[i] + row_base) : -1.0f;
            }
        }
        /* Stage3/4a :1761-1972 lambda = 0 (no warm starting) */
        real *lambda = (real *)calloc(m, sizeof(real));
        real *fc = (real *)calloc((size_t)6 * nb, sizeof(real));
        real *fa = (real *)calloc((size_t)2 * nb, sizeof(real));
        real *iMJ = (real *)calloc((size_t)14 * m, sizeof(real));
        /* compute_invM_JT :858-897 */
        for (int i = 0; i < m; i++) {
            const real *Jr = J + 16 * i;
            real *o = iMJ + 14 * i;
            pbody *b1 = &w->b[body_ids[jb1[i]]];
            real k1 = b1->invMass;
            for (int k = 0; k < 3; k++) o[k] = k1 * Jr[k];
            mul0_331(o + 3, invI + 12 * jb1[i], Jr + 3);
            if (w->dyn_enabled) {
                real mx = fabsf(o[0]);
                for (int k = 1; k < 6; k++) mx = fmaxf(mx, fabsf(o[k]));
                o[6] = mx;
            }
            if (jb2[i] != -1) {
                pbody *b2 = &w->b[body_ids[jb2[i]]];
                real k2 = b2->invMass;
                for (int k = 0; k < 3; k++) o[7 + k] = k2 * Jr[8 + k];
                mul0_331(o + 10, invI + 12 * jb2[i], Jr + 11);
                if (w->dyn_enabled) {
                    real mx = fabsf(o[7]);
                    for (int k = 8; k < 13; k++) mx = fmaxf(mx, fabsf(o[k]));
                    o[13] = mx;
                }
            }
        }
        /* Stage4LCP_AdComputation :2251-2316 */
        for (int i = 0; i < m; i++) {
            real *Jr = J + 16 * i;
            const real *o = iMJ + 14 * i;
            real sum = 0;
            for (int k = 0; k < 6; k++) sum += o[k] * Jr[k];
            if (jb2[i] != -1) for (int k = 0; k < 6; k++) sum += o[7 + k] * Jr[8 + k];
            real cfm_i = Jr[7];
            real Ad = w->w / (sum + cfm_i);
            Jr[7] = cfm_i * Ad;
            Jr[6] *= Ad;
            for (int k = 0; k < 6; k++) Jr[k] *= Ad;
            if (jb2[i] != -1) for (int k = 0; k < 6; k++) Jr[8 + k] *= Ad;
        }
        /* ReorderPrep :2329-2355 */
        int *order = (int *)malloc(sizeof(int) * m);
        {
            int head = 0, tail = m - valid_findices;
            for (int i = 0; i < m; i++) { if (findex[i] == -1) order[head++] = i; else order[tail++] = i; }
        }
        /* iteration driver :1823-1856 */
        sor_rows S = {J, iMJ, jb1, jb2, findex, lambda, fc, fa};
        if (w->threads > 1 && m >= w->mt_min_rows) {
            sor_sweeps_mt(w, &S, order, m, nb);
        } else {
            sor_driver drv = {0u, 0u, w->premature_delta};
            for (;;) {
                if (sor_reorder_due(w, drv.iteration)) sor_shuffle(order, m);
                /* Stage4LCP_IterationStep :2917-3033 */
                for (int ii = 0; ii < m; ii++) sor_row(&S, order[ii]);
                if (sor_after_sweep(w, &drv, fa, nb)) break;
            }
        }
        if (Ju) {
            island_residual(w, Ju, m, jb1, jb2, findex, lambda, body_ids, nb, invI);
            free(Ju);
        }
        /* Stage4b :3082-3182 */
        for (int i = 0; i < nb; i++) {
            pbody *b = &w->b[body_ids[i]];
            for (int k = 0; k < 3; k++) { b->lvel[k] += h * fc[6 * i + k]; b->avel[k] += h * fc[6 * i + 3 + k]; }
        }
        if (rows_out) for (int i = 0; i < m; i++) rows_out[20 * i + 19] = lambda[i];
        if (lambda_out) {
            for (int ji = 0; ji < nj; ji++) {
                int ofs = mindex[ji], im = mindex[ji + 1] - ofs;
                int ci = joint_cidx[jl[ji]];
                for (int r = 0; r < im && r < 3; r++) lambda_out[3 * ci + r] = lambda[ofs + r];
            }
        }
        if (g_row_slot) {  /* row -> 3 * contact + row of the contact (port_world_quickstep_map) */
            for (int ji = 0; ji < nj; ji++) {
                int ofs = mindex[ji], im = mindex[ji + 1] - ofs;
                int ci = joint_cidx[jl[ji]];
                for (int r = 0; r < im; r++) g_row_slot[row_base + ofs + r] = 3 * ci + r;
            }
        }
        free(order); free(iMJ); free(fa); free(fc); free(lambda); free(rhs_tmp);
        free(jb2); free(jb1); free(findex); free(J);
    }
    /* Stage6a :3299-3337 and Stage6b :3409-3439 */
    for (int i = 0; i < nb; i++) {
        pbody *b = &w->b[body_ids[i]];
        real ims = h * b->invMass;
        for (int k = 0; k < 3; k++) { b->lvel[k] += ims * b->facc[k]; b->tacc[k] *= h; }
        real tmp[3];
        mul0_331(tmp, invI + 12 * i, b->tacc);
        b->avel[0] = b->avel[0] + tmp[0]; b->avel[1] = b->avel[1] + tmp[1]; b->avel[2] = b->avel[2] + tmp[2];
    }
    for (int i = 0; i < nb; i++) {
        pbody *b = &w->b[body_ids[i]];
        step_body(b, h);
        b->facc[0] = b->facc[1] = b->facc[2] = 0;
        b->tacc[0] = b->tacc[1] = b->tacc[2] = 0;
    }
    free(mindex); free(jl); free(invI); free(tag);
}

/* util.cpp:724-860 BuildIslands... + util.cpp:886-1071 island processing.
 * stepped (optional) receives the bodies in stepping order (dGeomMoved order). */
static void world_quickstep(port_world *w, pjoint *joints, int nj, const int *joint_cidx, float *lambda_out,
                            float *rows_out, int *nrows, int *stepped) {
    int nb = w->nb;
    /* per-body joint lists, newest attached first (ode.cpp:1417-1431) */
    int *cnt = (int *)calloc(nb + 1, sizeof(int));
    for (int k = 0; k < nj; k++) {
        if (joints[k].node0 >= 0) cnt[joints[k].node0]++;
        if (joints[k].node1 >= 0) cnt[joints[k].node1]++;
    }
    int *start = (int *)malloc(sizeof(int) * (nb + 1));
    start[0] = 0;
    for (int i = 0; i < nb; i++) start[i + 1] = start[i] + cnt[i];
    int *lj = (int *)malloc(sizeof(int) * (start[nb] + 1)), *lb = (int *)malloc(sizeof(int) * (start[nb] + 1));
    int *fill = (int *)calloc(nb + 1, sizeof(int));
    for (int k = nj - 1; k >= 0; k--) {
        int a = joints[k].node0, b = joints[k].node1;
        if (a >= 0) { int p = start[a] + fill[a]++; lj[p] = k; lb[p] = b; }
        if (b >= 0) { int p = start[b] + fill[b]++; lj[p] = k; lb[p] = a; }
    }
    int *btag = (int *)calloc(nb + 1, sizeof(int)), *jtag = (int *)calloc(nj + 1, sizeof(int));
    int *ib = (int *)malloc(sizeof(int) * (nb + 1)), *ij = (int *)malloc(sizeof(int) * (nj + 1));
    int *stack = (int *)malloc(sizeof(int) * (nb + 1));
    int nstep = 0, row_base = 0;
    for (int bb = nb - 1; bb >= 0; bb--) {   /* world->firstbody is the newest body */
        if (btag[bb]) continue;
        btag[bb] = 1;
        int nbi = 0, nji = 0, ss = 0;
        ib[nbi++] = bb;
        int b = bb;
        for (;;) {
            for (int p = start[b]; p < start[b + 1]; p++) {
                int k = lj[p];
                if (!jtag[k]) {
                    jtag[k] = 1;
                    ij[nji++] = k;
                    int nbody = lb[p];
                    if (nbody >= 0 && btag[nbody] <= 0) { btag[nbody] = 1; stack[ss++] = nbody; }
                }
            }
            if (ss == 0) break;
            b = stack[--ss];
            ib[nbi++] = b;
        }
        quickstep_island(w, ib, nbi, joints, ij, nji, joint_cidx, lambda_out, rows_out ? rows_out + 20 * row_base : NULL, row_base);
        for (int k = 0; k < nji; k++) row_base += joints[ij[k]].m;
        if (stepped) for (int i = 0; i < nbi; i++) stepped[nstep++] = ib[i];
    }
    if (nrows) *nrows = row_base;
    free(stack); free(ij); free(ib); free(jtag); free(btag); free(fill); free(lb); free(lj); free(start); free(cnt);
}

static void fill_joint(pjoint *j, int b1, int b2, int mode, const float *s) {
    memset(j, 0, sizeof *j);
    /* dJointAttach: a null first body swaps and sets dJOINT_REVERSE */
    if (b1 < 0) { j->node0 = b2; j->node1 = -1; j->reverse = 1; }
    else { j->node0 = b1; j->node1 = b2; j->reverse = 0; }
    j->mode = mode;
    j->pos[0] = s[0]; j->pos[1] = s[1]; j->pos[2] = s[2];
    j->normal[0] = s[3]; j->normal[1] = s[4]; j->normal[2] = s[5];
    j->depth = s[6]; j->mu = s[7]; j->mu2 = s[8]; j->bounce = s[9]; j->bounce_vel = s[10];
    j->soft_erp = s[11]; j->soft_cfm = s[12]; j->slip1 = s[13]; j->slip2 = s[14];
}

int port_world_quickstep_map(port_world *w, int nc, const int *cb, const int *mode, const float *cs, float *lambda,
                             float *rows_out, int *nrows_out, int *row_slot) {
    g_row_slot = row_slot;
    int r = port_world_quickstep(w, nc, cb, mode, cs, lambda, rows_out, nrows_out);
    g_row_slot = NULL;
    return r;
}

int port_world_quickstep(port_world *w, int nc, const int *cb, const int *mode, const float *cs, float *lambda,
                         float *rows_out, int *nrows_out) {
    pjoint *joints = (pjoint *)calloc(nc > 0 ? nc : 1, sizeof(pjoint));
    int *cidx = (int *)malloc(sizeof(int) * (nc > 0 ? nc : 1));
    for (int k = 0; k < nc; k++) { fill_joint(&joints[k], cb[2 * k], cb[2 * k + 1], mode[k], cs + 16 * k); cidx[k] = k; }
    if (lambda) memset(lambda, 0, sizeof(float) * 3 * nc);
    w->res_max = 0;
    w->lam_max = 0;
    world_quickstep(w, joints, nc, cidx, lambda, rows_out, nrows_out, NULL);
    free(cidx); free(joints);
    return 1;
}

/* ------------------------------------------------------------- sim loop */
struct port_sim {
    port_world *w;
    int ng;
    int *cls, *body;
    real *pos, *R, *dims;     /* static pose for body-less geoms */
    int *list;                /* space list order, head first */
    unsigned char *dirty;
    int minlevel, maxlevel, maxc, mode;
    real surface[8];
    pjoint *joints; int nj, capj;
    int *made_b; float *made_cs;
    pgeom *posed;
    double t_collide, t_step;  /* seconds of the last step: collision (dSpaceCollide + contacts), quickstep */
};

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

port_sim *port_sim_create(port_world *w, int ng, const int *cls, const int *body, const float *pos, const float *R,
                          const float *dims, int minlevel, int maxlevel, int maxc, int mode, const float *surface) {
    port_sim *s = (port_sim *)calloc(1, sizeof(port_sim));
    s->w = w; s->ng = ng;
    s->cls = (int *)malloc(sizeof(int) * ng); memcpy(s->cls, cls, sizeof(int) * ng);
    s->body = (int *)malloc(sizeof(int) * ng); memcpy(s->body, body, sizeof(int) * ng);
    s->pos = (real *)malloc(sizeof(real) * 3 * ng); memcpy(s->pos, pos, sizeof(real) * 3 * ng);
    s->R = (real *)malloc(sizeof(real) * 12 * ng); memcpy(s->R, R, sizeof(real) * 12 * ng);
    s->dims = (real *)malloc(sizeof(real) * 4 * ng); memcpy(s->dims, dims, sizeof(real) * 4 * ng);
    /* dSpaceAdd puts each new geom at the list head (collision_space.cpp:160-176) */
    s->list = (int *)malloc(sizeof(int) * ng);
    for (int i = 0; i < ng; i++) s->list[i] = ng - 1 - i;
    s->dirty = (unsigned char *)malloc(ng); memset(s->dirty, 1, ng);
    s->minlevel = minlevel; s->maxlevel = maxlevel; s->maxc = maxc; s->mode = mode;
    memcpy(s->surface, surface, sizeof(real) * 6);
    s->capj = 1024; s->nj = 0;
    s->joints = (pjoint *)malloc(sizeof(pjoint) * s->capj);
    s->made_b = (int *)malloc(sizeof(int) * 2 * s->capj);
    s->made_cs = (float *)malloc(sizeof(float) * 16 * s->capj);
    s->posed = (pgeom *)malloc(sizeof(pgeom) * ng);
    return s;
}

void port_sim_destroy(port_sim *s) {
    if (!s) return;
    free(s->cls); free(s->body); free(s->pos); free(s->R); free(s->dims); free(s->list); free(s->dirty);
    free(s->joints); free(s->made_b); free(s->made_cs); free(s->posed); free(s);
}

/* demo_boxstack.cpp:130-170 near callback: dCollide then one contact joint per point */
static void sim_cb(void *ctx, int g1, int g2) {
    port_sim *s = (port_sim *)ctx;
    pcontact c[16];
    memset(c, 0, sizeof c);
    int n = collide_geoms(&s->posed[g1], &s->posed[g2], s->maxc, c);
    int b1 = s->body[g1], b2 = s->body[g2];
    for (int i = 0; i < n; i++) {
        if (s->nj == s->capj) {
            s->capj *= 2;
            s->joints = (pjoint *)realloc(s->joints, sizeof(pjoint) * s->capj);
            s->made_b = (int *)realloc(s->made_b, sizeof(int) * 2 * s->capj);
            s->made_cs = (float *)realloc(s->made_cs, sizeof(float) * 16 * s->capj);
        }
        float *cs = s->made_cs + 16 * s->nj;
        memset(cs, 0, 16 * sizeof(float));
        cs[0] = c[i].pos[0]; cs[1] = c[i].pos[1]; cs[2] = c[i].pos[2];
        cs[3] = c[i].normal[0]; cs[4] = c[i].normal[1]; cs[5] = c[i].normal[2];
        cs[6] = c[i].depth;
        memcpy(cs + 7, s->surface, 6 * sizeof(float));
        s->made_b[2 * s->nj] = b1; s->made_b[2 * s->nj + 1] = b2;
        fill_joint(&s->joints[s->nj], b1, b2, s->mode, cs);
        s->nj++;
    }
}

int port_sim_step(port_sim *s) {
    port_world *w = s->w;
    const double t0 = now_s();
    /* geoms take their body's pose (collision_kernel.cpp recomputePosr) */
    real *aabbs = (real *)malloc(sizeof(real) * 6 * (s->ng > 0 ? s->ng : 1));
    for (int i = 0; i < s->ng; i++) {
        pgeom *g = &s->posed[i];
        if (s->body[i] >= 0) {
            const pbody *b = &w->b[s->body[i]];
            make_pgeom(g, s->cls[i], b->pos, b->R, s->dims + 4 * i);
        } else {
            make_pgeom(g, s->cls[i], s->pos + 3 * i, s->R + 12 * i, s->dims + 4 * i);
        }
        compute_aabb(g, aabbs + 6 * i);
    }
    /* cleanGeoms clears the dirty prefix (collision_space.cpp:403-418) */
    for (int k = 0; k < s->ng && s->dirty[s->list[k]]; k++) s->dirty[s->list[k]] = 0;
    s->nj = 0;
    hash_collide(s->ng, s->list, s->body, aabbs, s->minlevel, s->maxlevel, s, sim_cb);
    free(aabbs);
    int *cidx = (int *)malloc(sizeof(int) * (s->nj > 0 ? s->nj : 1));
    for (int k = 0; k < s->nj; k++) cidx[k] = k;
    int *stepped = (int *)malloc(sizeof(int) * (w->nb > 0 ? w->nb : 1));
    const double t1 = now_s();
    w->res_max = 0;
    w->lam_max = 0;
    world_quickstep(w, s->joints, s->nj, cidx, NULL, NULL, NULL, stepped);
    s->t_collide = t1 - t0;
    s->t_step = now_s() - t1;
    /* dGeomMoved for each stepped body's geom: a clean geom is marked dirty
     * and moved to the head of the space's list (collision_space.cpp:49-75,
     * 205-209).  The moves are applied at once: the moved geoms, last moved
     * first, then the others in their previous order -- the list the
     * one-at-a-time moves leave, in O(geoms) instead of O(geoms^2). */
    int *geom_of = (int *)malloc(sizeof(int) * (w->nb > 0 ? w->nb : 1));
    int *moved = (int *)malloc(sizeof(int) * (s->ng > 0 ? s->ng : 1));
    unsigned char *was_moved = (unsigned char *)calloc(s->ng > 0 ? s->ng : 1, 1);
    int *list2 = (int *)malloc(sizeof(int) * (s->ng > 0 ? s->ng : 1));
    for (int i = 0; i < w->nb; i++) geom_of[i] = -1;
    for (int g = 0; g < s->ng; g++) if (s->body[g] >= 0) geom_of[s->body[g]] = g;
    int nmoved = 0;
    for (int k = 0; k < w->nb; k++) {
        int g = geom_of[stepped[k]];
        if (g < 0 || s->dirty[g]) continue;
        s->dirty[g] = 1;
        was_moved[g] = 1;
        moved[nmoved++] = g;
    }
    if (nmoved > 0) {
        int p = 0;
        for (int k = nmoved - 1; k >= 0; k--) list2[p++] = moved[k];
        for (int k = 0; k < s->ng; k++) if (!was_moved[s->list[k]]) list2[p++] = s->list[k];
        memcpy(s->list, list2, sizeof(int) * s->ng);
    }
    free(list2); free(was_moved); free(moved);
    free(geom_of); free(stepped); free(cidx);
    return s->nj;
}

void port_sim_last_stats(const port_sim *s, double *out4) {
    out4[0] = s->t_collide;
    out4[1] = s->t_step;
    out4[2] = s->w->res_max;
    out4[3] = s->w->lam_max;
}

void port_world_set_residual(port_world *w, int on) { w->resid_on = on != 0; }
void port_world_last_residual(const port_world *w, double *out2) { out2[0] = w->res_max; out2[1] = w->lam_max; }

int port_sim_last_contacts(const port_sim *s, int *cb, float *cs, int cap) {
    int n = s->nj < cap ? s->nj : cap;
    if (cb) memcpy(cb, s->made_b, sizeof(int) * 2 * n);
    if (cs) memcpy(cs, s->made_cs, sizeof(float) * 16 * n);
    return s->nj;
}

/* ------------------------------------------------------------- residual */
/* FP64 natural-map residual of the LCP the quickstep rows pose
 * (quickstep.cpp:1555-1561, 1644-1747 form A = J M^-1 J^T + diag(cfm),
 * b = rhs; bounds per quickstep.cpp:2972-2978). */
double port_lcp_residual(int m, const float *rows, int nb, const double *invm, const double *invI,
                         const float *lambda, double *compl_err) {
    double *v = (double *)calloc((size_t)6 * (nb > 0 ? nb : 1), sizeof(double));
    double *f = (double *)calloc((size_t)6 * (nb > 0 ? nb : 1), sizeof(double));
    for (int i = 0; i < m; i++) {
        const float *r = rows + 20 * i;
        int b1 = (int)r[16], b2 = (int)r[17];
        double l = lambda[i];
        for (int k = 0; k < 6; k++) f[6 * b1 + k] += r[k] * l;
        if (b2 >= 0) for (int k = 0; k < 6; k++) f[6 * b2 + k] += r[6 + k] * l;
    }
    for (int b = 0; b < nb; b++) {
        for (int k = 0; k < 3; k++) v[6 * b + k] = invm[b] * f[6 * b + k];
        for (int k = 0; k < 3; k++)
            v[6 * b + 3 + k] = invI[9 * b + 3 * k] * f[6 * b + 3] + invI[9 * b + 3 * k + 1] * f[6 * b + 4] +
                               invI[9 * b + 3 * k + 2] * f[6 * b + 5];
    }
    double res = 0, ce = 0;
    for (int i = 0; i < m; i++) {
        const float *r = rows + 20 * i;
        int b1 = (int)r[16], b2 = (int)r[17], fi = (int)r[18];
        double Av = 0, D = 0;
        for (int k = 0; k < 6; k++) Av += r[k] * v[6 * b1 + k];
        for (int k = 0; k < 3; k++) D += r[k] * r[k] * invm[b1];
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) D += r[3 + a] * invI[9 * b1 + 3 * a + c] * r[3 + c];
        if (b2 >= 0) {
            for (int k = 0; k < 6; k++) Av += r[6 + k] * v[6 * b2 + k];
            for (int k = 0; k < 3; k++) D += r[6 + k] * r[6 + k] * invm[b2];
            for (int a = 0; a < 3; a++)
                for (int c = 0; c < 3; c++) D += r[9 + a] * invI[9 * b2 + 3 * a + c] * r[9 + c];
        }
        double cfm = r[13];
        double w_i = Av + cfm * lambda[i] - r[12];
        D += cfm;
        double lo, hi;
        if (fi >= 0) { hi = fabs((double)r[15] * lambda[fi]); lo = -hi; }
        else { lo = r[14]; hi = r[15]; }
        double li = lambda[i];
        double t = li - w_i / D;
        if (t < lo) t = lo;
        if (t > hi) t = hi;
        double e = fabs(li - t);
        if (e > res) res = e;
        /* complementarity, min-map form in the units of lambda (w / A_ii) */
        double wp = w_i > 0 ? w_i / D : 0, wm = w_i < 0 ? -w_i / D : 0;
        double cc = fmax(fmin(li - lo, wp), fmin(hi - li, wm));
        cc = fabs(cc);
        if (cc > ce) ce = cc;
    }
    if (compl_err) *compl_err = ce;
    free(v); free(f);
    return res;
}
