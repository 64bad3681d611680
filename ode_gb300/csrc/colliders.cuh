// Narrow-phase colliders for sphere, box, capsule and plane, as device code.
//
// Each function restates the reference collider it names (file:line) with the
// same arithmetic in the same order, so that with -fmad=false the contact
// count, positions, normals, depths and dBoxBox's feature code come out as the
// reference's float build computes them.  Differences from the reference are
// structural only: geometry arrives as registers (pos, 3x4 R, dims) instead of
// dxGeom objects and contacts are written to a small local array.
#pragma once
#include <math.h>
#include "gbode_device.cuh"

namespace gb {

#define GB_NUMC_MASK 0xffff

struct GeomView {
    int cls;
    float pos[4];
    float R[12];
    float dims[4];
};

struct CPoint {
    float pos[3];
    float normal[3];
    float depth;
};

__device__ __forceinline__ float d3_41(const float *a, const float *b) { return a[0] * b[0] + a[4] * b[1] + a[8] * b[2]; }
__device__ __forceinline__ float d3_14(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[4] + a[2] * b[8]; }
__device__ __forceinline__ float d3_44(const float *a, const float *b) { return a[0] * b[0] + a[4] * b[4] + a[8] * b[8]; }
__device__ __forceinline__ void m0_331(float *r, const float *a, const float *b) {
    float r0 = dot3(a, b), r1 = dot3(a + 4, b), r2 = dot3(a + 8, b);
    r[0] = r0; r[1] = r1; r[2] = r2;
}
__device__ __forceinline__ void m1_331(float *r, const float *a, const float *b) {
    float r0 = d3_41(a, b), r1 = d3_41(a + 1, b), r2 = d3_41(a + 2, b);
    r[0] = r0; r[1] = r1; r[2] = r2;
}
__device__ __forceinline__ float dist3(const float *a, const float *b) {
    float t[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return sqrtf(dot3(t, t));
}

// odemath.cpp:95-165 dxSafeNormalize3 (+ odemath.h:36-46 fallback)
__device__ inline void normalize3(float *a) {
    float a0 = fabsf(a[0]), a1 = fabsf(a[1]), a2 = fabsf(a[2]);
    int idx;
    if (a1 > a0) idx = (a2 > a1) ? 2 : 1;
    else if (a2 > a0) idx = 2;
    else {
        if (!(a0 > 0.0f)) { a[0] = 1.0f; a[1] = 0.0f; a[2] = 0.0f; return; }
        idx = 0;
    }
    int i1 = idx == 0 ? 1 : 0, i2 = idx == 2 ? 1 : 2;
    float rc = 1.0f / fabsf(a[idx]);
    float x1 = a[i1] * rc, x2 = a[i2] * rc;
    float l = 1.0f / sqrtf(1.0f + x1 * x1 + x2 * x2);
    a[i1] = x1 * l; a[i2] = x2 * l; a[idx] = copysignf(l, a[idx]);
}

// collision_util.cpp:38-67 dCollideSpheres
__device__ inline int collide_spheres(const float *p1, float r1, const float *p2, float r2, CPoint *c) {
    float d = dist3(p1, p2);
    if (d > (r1 + r2)) return 0;
    if (d <= 0) {
        c->pos[0] = p1[0]; c->pos[1] = p1[1]; c->pos[2] = p1[2];
        c->normal[0] = 1; c->normal[1] = 0; c->normal[2] = 0;
        c->depth = r1 + r2;
    } else {
        float d1 = 1.0f / d;
        c->normal[0] = (p1[0] - p2[0]) * d1;
        c->normal[1] = (p1[1] - p2[1]) * d1;
        c->normal[2] = (p1[2] - p2[2]) * d1;
        float k = 0.5f * (r2 - r1 - d);
        c->pos[0] = p1[0] + c->normal[0] * k;
        c->pos[1] = p1[1] + c->normal[1] * k;
        c->pos[2] = p1[2] + c->normal[2] * k;
        c->depth = r1 + r2 - d;
    }
    return 1;
}

// collision_util.cpp:70-95 dLineClosestApproach
__device__ inline void line_closest_approach(const float *pa, const float *ua, const float *pb, const float *ub,
                                             float *alpha, float *beta) {
    float p[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    float uaub = dot3(ua, ub), q1 = dot3(ua, p), q2 = -dot3(ub, p);
    float d = 1 - uaub * uaub;
    if (d <= 0.0001f) { *alpha = 0; *beta = 0; }
    else {
        d = 1.0f / d;
        *alpha = (q1 + uaub * q2) * d;
        *beta = (uaub * q1 + q2) * d;
    }
}

// collision_util.cpp:109-215 dClosestLineSegmentPoints
__device__ inline void closest_segment_points(const float *a1, const float *a2, const float *b1, const float *b2,
                                              float *cp1, float *cp2) {
    float a1a2[3], b1b2[3], a1b1[3], a1b2[3], a2b1[3], a2b2[3], n[3];
    float la, lb, k, da1, da2, da3, da4, db1, db2, db3, db4, det;
#define GB_SET2(a, b) { a[0] = b[0]; a[1] = b[1]; a[2] = b[2]; }
#define GB_SUB(a, b, c) { a[0] = b[0] - c[0]; a[1] = b[1] - c[1]; a[2] = b[2] - c[2]; }
    GB_SUB(a1a2, a2, a1); GB_SUB(b1b2, b2, b1); GB_SUB(a1b1, b1, a1);
    da1 = dot3(a1a2, a1b1); db1 = dot3(b1b2, a1b1);
    if (da1 <= 0 && db1 >= 0) { GB_SET2(cp1, a1); GB_SET2(cp2, b1); return; }
    GB_SUB(a1b2, b2, a1);
    da2 = dot3(a1a2, a1b2); db2 = dot3(b1b2, a1b2);
    if (da2 <= 0 && db2 <= 0) { GB_SET2(cp1, a1); GB_SET2(cp2, b2); return; }
    GB_SUB(a2b1, b1, a2);
    da3 = dot3(a1a2, a2b1); db3 = dot3(b1b2, a2b1);
    if (da3 >= 0 && db3 >= 0) { GB_SET2(cp1, a2); GB_SET2(cp2, b1); return; }
    GB_SUB(a2b2, b2, a2);
    da4 = dot3(a1a2, a2b2); db4 = dot3(b1b2, a2b2);
    if (da4 >= 0 && db4 <= 0) { GB_SET2(cp1, a2); GB_SET2(cp2, b2); return; }
    la = dot3(a1a2, a1a2);
    if (da1 >= 0 && da3 <= 0) {
        k = da1 / la;
        for (int i = 0; i < 3; i++) n[i] = a1b1[i] - k * a1a2[i];
        if (dot3(b1b2, n) >= 0) {
            for (int i = 0; i < 3; i++) cp1[i] = a1[i] + k * a1a2[i];
            GB_SET2(cp2, b1); return;
        }
    }
    if (da2 >= 0 && da4 <= 0) {
        k = da2 / la;
        for (int i = 0; i < 3; i++) n[i] = a1b2[i] - k * a1a2[i];
        if (dot3(b1b2, n) <= 0) {
            for (int i = 0; i < 3; i++) cp1[i] = a1[i] + k * a1a2[i];
            GB_SET2(cp2, b2); return;
        }
    }
    lb = dot3(b1b2, b1b2);
    if (db1 <= 0 && db2 >= 0) {
        k = -db1 / lb;
        for (int i = 0; i < 3; i++) n[i] = -a1b1[i] - k * b1b2[i];
        if (dot3(a1a2, n) >= 0) {
            GB_SET2(cp1, a1);
            for (int i = 0; i < 3; i++) cp2[i] = b1[i] + k * b1b2[i];
            return;
        }
    }
    if (db3 <= 0 && db4 >= 0) {
        k = -db3 / lb;
        for (int i = 0; i < 3; i++) n[i] = -a2b1[i] - k * b1b2[i];
        if (dot3(a1a2, n) <= 0) {
            GB_SET2(cp1, a2);
            for (int i = 0; i < 3; i++) cp2[i] = b1[i] + k * b1b2[i];
            return;
        }
    }
    k = dot3(a1a2, b1b2);
    det = la * lb - k * k;
    if (det <= 0) { GB_SET2(cp1, a1); GB_SET2(cp2, b1); return; }
    det = 1.0f / det;
    float alpha = (lb * da1 - k * db1) * det;
    float beta = (k * da1 - la * db1) * det;
    for (int i = 0; i < 3; i++) { cp1[i] = a1[i] + alpha * a1a2[i]; cp2[i] = b1[i] + beta * b1b2[i]; }
#undef GB_SET2
#undef GB_SUB
}

// collision_util.cpp:247-385 dClosestLineBoxPoints
__device__ inline void closest_line_box_points(const float *p1, const float *p2, const float *c, const float *R,
                                               const float *side, float *lret, float *bret) {
    float tmp[3], s[3], v[3];
    tmp[0] = p1[0] - c[0]; tmp[1] = p1[1] - c[1]; tmp[2] = p1[2] - c[2];
    m1_331(s, R, tmp);
    tmp[0] = p2[0] - p1[0]; tmp[1] = p2[1] - p1[1]; tmp[2] = p2[2] - p1[2];
    m1_331(v, R, tmp);
    float sign[3];
    for (int i = 0; i < 3; i++) {
        if (v[i] < 0) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = -1; }
        else sign[i] = 1;
    }
    float v2[3] = {v[0] * v[0], v[1] * v[1], v[2] * v[2]};
    float h[3] = {0.5f * side[0], 0.5f * side[1], 0.5f * side[2]};
    int region[3];
    float tanchor[3];
    const float tanchor_eps = 1e-19f;
    for (int i = 0; i < 3; i++) {
        if (v[i] > tanchor_eps) {
            if (s[i] < -h[i]) { region[i] = -1; tanchor[i] = (-h[i] - s[i]) / v[i]; }
            else { region[i] = (s[i] > h[i]); tanchor[i] = (h[i] - s[i]) / v[i]; }
        } else { region[i] = 0; tanchor[i] = 2; }
    }
    float t = 0, dd2dt = 0;
    for (int i = 0; i < 3; i++) dd2dt -= (region[i] ? v2[i] : 0) * tanchor[i];
    if (!(dd2dt >= 0)) {
        bool done = false;
        // the reference loops while t < 1; every pass moves t to a new anchor
        // or to 1, so at most four passes occur
        for (int pass = 0; pass < 8 && !done; pass++) {
            float next_t = 1;
            for (int i = 0; i < 3; i++)
                if (tanchor[i] > t && tanchor[i] < 1 && tanchor[i] < next_t) next_t = tanchor[i];
            float next_dd2dt = 0;
            for (int i = 0; i < 3; i++) next_dd2dt += (region[i] ? v2[i] : 0) * (next_t - tanchor[i]);
            if (next_dd2dt >= 0) {
                float m = (next_dd2dt - dd2dt) / (next_t - t);
                t -= dd2dt / m;
                done = true;
                break;
            }
            for (int i = 0; i < 3; i++)
                if (tanchor[i] == next_t) { tanchor[i] = (h[i] - s[i]) / v[i]; region[i]++; }
            t = next_t;
            dd2dt = next_dd2dt;
            if (!(t < 1)) break;
        }
        if (!done) t = 1;
    }
    for (int i = 0; i < 3; i++) lret[i] = p1[i] + t * tmp[i];
    for (int i = 0; i < 3; i++) {
        tmp[i] = sign[i] * (s[i] + t * v[i]);
        if (tmp[i] < -h[i]) tmp[i] = -h[i];
        else if (tmp[i] > h[i]) tmp[i] = h[i];
    }
    m0_331(s, R, tmp);
    for (int i = 0; i < 3; i++) bret[i] = s[i] + c[i];
}

// box.cpp:212-263 intersectRectQuad (ping-pong between two local buffers)
__device__ inline int intersect_rect_quad(const float h[2], const float p[8], float ret[16]) {
    float bufA[16], bufB[16];
    for (int i = 0; i < 8; i++) bufA[i] = p[i];
    float *q = bufA, *r = bufB;
    int nq = 4, nr = 0;
    for (int dir = 0; dir <= 1; dir++) {
        for (int sign = -1; sign <= 1; sign += 2) {
            const float hd = h[dir];
            float *pq = q, *pr = r;
            nr = 0;
            for (int i = nq; i > 0; i--) {
                if (sign * pq[dir] < hd) {
                    pr[0] = pq[0]; pr[1] = pq[1];
                    pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                const float *nextq = (i > 1) ? pq + 2 : q;
                if ((sign * pq[dir] < hd) ^ (sign * nextq[dir] < hd)) {
                    pr[1 - dir] = pq[1 - dir] + (nextq[1 - dir] - pq[1 - dir]) / (nextq[dir] - pq[dir]) * (sign * hd - pq[dir]);
                    pr[dir] = sign * hd;
                    pr += 2; nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                pq += 2;
            }
            float *t = q; q = r; r = t;
            nq = nr;
        }
    }
done:
    for (int i = 0; i < nr * 2; i++) ret[i] = q[i];
    return nr;
}

// box.cpp:274-336 cullPoints
__device__ inline void cull_points(int n, const float *p, int m, int i0, int *iret) {
    float a, cx, cy, q;
    if (n == 1) { cx = p[0]; cy = p[1]; }
    else if (n == 2) { cx = 0.5f * (p[0] + p[2]); cy = 0.5f * (p[1] + p[3]); }
    else {
        a = 0; cx = 0; cy = 0;
        for (int i = 0; i < (n - 1); i++) {
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
    float A[8];
    for (int i = 0; i < n; i++) A[i] = atan2f(p[i * 2 + 1] - cy, p[i * 2] - cx);
    int avail[8];
    for (int i = 0; i < n; i++) avail[i] = 1;
    avail[i0] = 0;
    iret[0] = i0;
    for (int j = 1; j < m; j++) {
        a = (float)((double)(float)j * (2 * M_PI / m) + (double)A[i0]);
        if ((double)a > M_PI) a -= (float)(2 * M_PI);
        float maxdiff = 1e9f, diff;
        int pick = i0;
        for (int i = 0; i < n; i++) {
            if (avail[i]) {
                diff = fabsf(A[i] - a);
                if ((double)diff > M_PI) diff = (float)(2 * M_PI - (double)diff);
                if (diff < maxdiff) { maxdiff = diff; pick = i; }
            }
        }
        iret[j] = pick;
        avail[pick] = 0;
    }
}

// box.cpp:356-737 dBoxBox.  Writes positions and depths; returns the count.
__device__ inline int box_box(const float *p1, const float *R1, const float *side1, const float *p2, const float *R2,
                              const float *side2, float *normal, float *depth, int *return_code, int flags,
                              CPoint *contact) {
    const float fudge_factor = 1.05f;
    float p[3], pp[3], normalC[3] = {0, 0, 0};
    const float *normalR = 0;
    float A[3], B[3], R11, R12, R13, R21, R22, R23, R31, R32, R33, Q11, Q12, Q13, Q21, Q22, Q23, Q31, Q32, Q33, s,
        s2, l, e;
    int invert_normal, code;
    p[0] = p2[0] - p1[0]; p[1] = p2[1] - p1[1]; p[2] = p2[2] - p1[2];
    m1_331(pp, R1, p);
    A[0] = side1[0] * 0.5f; A[1] = side1[1] * 0.5f; A[2] = side1[2] * 0.5f;
    B[0] = side2[0] * 0.5f; B[1] = side2[1] * 0.5f; B[2] = side2[2] * 0.5f;
    R11 = d3_44(R1 + 0, R2 + 0); R12 = d3_44(R1 + 0, R2 + 1); R13 = d3_44(R1 + 0, R2 + 2);
    R21 = d3_44(R1 + 1, R2 + 0); R22 = d3_44(R1 + 1, R2 + 1); R23 = d3_44(R1 + 1, R2 + 2);
    R31 = d3_44(R1 + 2, R2 + 0); R32 = d3_44(R1 + 2, R2 + 1); R33 = d3_44(R1 + 2, R2 + 2);
    Q11 = fabsf(R11); Q12 = fabsf(R12); Q13 = fabsf(R13);
    Q21 = fabsf(R21); Q22 = fabsf(R22); Q23 = fabsf(R23);
    Q31 = fabsf(R31); Q32 = fabsf(R32); Q33 = fabsf(R33);
#define GB_TSTF(expr1, expr2, norm, cc)                                            \
    e = (expr1);                                                                   \
    s2 = fabsf(e) - (expr2);                                                       \
    if (s2 > 0) return 0;                                                          \
    if (s2 > s) { s = s2; normalR = norm; invert_normal = (e < 0); code = (cc); }
#define GB_TSTE(expr1, expr2, n1, n2, n3, cc)                                      \
    e = (expr1);                                                                   \
    s2 = fabsf(e) - (expr2);                                                       \
    if (s2 > 0) return 0;                                                          \
    l = sqrtf((n1) * (n1) + (n2) * (n2) + (n3) * (n3));                            \
    if (l > 0) {                                                                   \
        s2 /= l;                                                                   \
        if (s2 * fudge_factor > s) {                                               \
            s = s2; normalR = 0;                                                   \
            normalC[0] = (n1) / l; normalC[1] = (n2) / l; normalC[2] = (n3) / l;   \
            invert_normal = (e < 0); code = (cc);                                  \
        }                                                                          \
    }
    s = -INFINITY; invert_normal = 0; code = 0;
    GB_TSTF(pp[0], (A[0] + B[0] * Q11 + B[1] * Q12 + B[2] * Q13), R1 + 0, 1);
    GB_TSTF(pp[1], (A[1] + B[0] * Q21 + B[1] * Q22 + B[2] * Q23), R1 + 1, 2);
    GB_TSTF(pp[2], (A[2] + B[0] * Q31 + B[1] * Q32 + B[2] * Q33), R1 + 2, 3);
    GB_TSTF(d3_41(R2 + 0, p), (A[0] * Q11 + A[1] * Q21 + A[2] * Q31 + B[0]), R2 + 0, 4);
    GB_TSTF(d3_41(R2 + 1, p), (A[0] * Q12 + A[1] * Q22 + A[2] * Q32 + B[1]), R2 + 1, 5);
    GB_TSTF(d3_41(R2 + 2, p), (A[0] * Q13 + A[1] * Q23 + A[2] * Q33 + B[2]), R2 + 2, 6);
    GB_TSTE(pp[2] * R21 - pp[1] * R31, (A[1] * Q31 + A[2] * Q21 + B[1] * Q13 + B[2] * Q12), 0, -R31, R21, 7);
    GB_TSTE(pp[2] * R22 - pp[1] * R32, (A[1] * Q32 + A[2] * Q22 + B[0] * Q13 + B[2] * Q11), 0, -R32, R22, 8);
    GB_TSTE(pp[2] * R23 - pp[1] * R33, (A[1] * Q33 + A[2] * Q23 + B[0] * Q12 + B[1] * Q11), 0, -R33, R23, 9);
    GB_TSTE(pp[0] * R31 - pp[2] * R11, (A[0] * Q31 + A[2] * Q11 + B[1] * Q23 + B[2] * Q22), R31, 0, -R11, 10);
    GB_TSTE(pp[0] * R32 - pp[2] * R12, (A[0] * Q32 + A[2] * Q12 + B[0] * Q23 + B[2] * Q21), R32, 0, -R12, 11);
    GB_TSTE(pp[0] * R33 - pp[2] * R13, (A[0] * Q33 + A[2] * Q13 + B[0] * Q22 + B[1] * Q21), R33, 0, -R13, 12);
    GB_TSTE(pp[1] * R11 - pp[0] * R21, (A[0] * Q21 + A[1] * Q11 + B[1] * Q33 + B[2] * Q32), -R21, R11, 0, 13);
    GB_TSTE(pp[1] * R12 - pp[0] * R22, (A[0] * Q22 + A[1] * Q12 + B[0] * Q33 + B[2] * Q31), -R22, R12, 0, 14);
    GB_TSTE(pp[1] * R13 - pp[0] * R23, (A[0] * Q23 + A[1] * Q13 + B[0] * Q32 + B[1] * Q31), -R23, R13, 0, 15);
#undef GB_TSTF
#undef GB_TSTE
    if (!code) return 0;
    if (normalR) { normal[0] = normalR[0]; normal[1] = normalR[4]; normal[2] = normalR[8]; }
    else m0_331(normal, R1, normalC);
    if (invert_normal) { normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2]; }
    *depth = -s;

    if (code > 6) {
        float pa[3], pb[3], sign, alpha, beta, ua[3], ub[3];
        for (int i = 0; i < 3; i++) pa[i] = p1[i];
        for (int j = 0; j < 3; j++) {
            sign = (d3_14(normal, R1 + j) > 0) ? 1.0f : -1.0f;
            for (int i = 0; i < 3; i++) pa[i] += sign * A[j] * R1[i * 4 + j];
        }
        for (int i = 0; i < 3; i++) pb[i] = p2[i];
        for (int j = 0; j < 3; j++) {
            sign = (d3_14(normal, R2 + j) > 0) ? -1.0f : 1.0f;
            for (int i = 0; i < 3; i++) pb[i] += sign * B[j] * R2[i * 4 + j];
        }
        for (int i = 0; i < 3; i++) ua[i] = R1[((code)-7) / 3 + i * 4];
        for (int i = 0; i < 3; i++) ub[i] = R2[((code)-7) % 3 + i * 4];
        line_closest_approach(pa, ua, pb, ub, &alpha, &beta);
        for (int i = 0; i < 3; i++) pa[i] += ua[i] * alpha;
        for (int i = 0; i < 3; i++) pb[i] += ub[i] * beta;
        for (int i = 0; i < 3; i++) contact[0].pos[i] = 0.5f * (pa[i] + pb[i]);
        contact[0].depth = *depth;
        *return_code = code;
        return 1;
    }

    const float *Ra, *Rb, *pa, *pb, *Sa, *Sb;
    if (code <= 3) { Ra = R1; Rb = R2; pa = p1; pb = p2; Sa = A; Sb = B; }
    else { Ra = R2; Rb = R1; pa = p2; pb = p1; Sa = B; Sb = A; }
    float normal2[3], nr[3], anr[3];
    if (code <= 3) { normal2[0] = normal[0]; normal2[1] = normal[1]; normal2[2] = normal[2]; }
    else { normal2[0] = -normal[0]; normal2[1] = -normal[1]; normal2[2] = -normal[2]; }
    m1_331(nr, Rb, normal2);
    anr[0] = fabsf(nr[0]); anr[1] = fabsf(nr[1]); anr[2] = fabsf(nr[2]);
    int lanr, a1, a2;
    if (anr[1] > anr[0]) {
        if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    float center[3];
    if (nr[lanr] < 0) { for (int i = 0; i < 3; i++) center[i] = pb[i] - pa[i] + Sb[lanr] * Rb[i * 4 + lanr]; }
    else { for (int i = 0; i < 3; i++) center[i] = pb[i] - pa[i] - Sb[lanr] * Rb[i * 4 + lanr]; }
    int codeN, code1, code2;
    if (code <= 3) codeN = code - 1; else codeN = code - 4;
    if (codeN == 0) { code1 = 1; code2 = 2; }
    else if (codeN == 1) { code1 = 0; code2 = 2; }
    else { code1 = 0; code2 = 1; }
    float quad[8], c1, c2, m11, m12, m21, m22;
    c1 = d3_14(center, Ra + code1);
    c2 = d3_14(center, Ra + code2);
    m11 = d3_44(Ra + code1, Rb + a1);
    m12 = d3_44(Ra + code1, Rb + a2);
    m21 = d3_44(Ra + code2, Rb + a1);
    m22 = d3_44(Ra + code2, Rb + a2);
    {
        float k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
        quad[0] = c1 - k1 - k3; quad[1] = c2 - k2 - k4;
        quad[2] = c1 - k1 + k3; quad[3] = c2 - k2 + k4;
        quad[4] = c1 + k1 + k3; quad[5] = c2 + k2 + k4;
        quad[6] = c1 + k1 - k3; quad[7] = c2 + k2 - k4;
    }
    float rect[2] = {Sa[code1], Sa[code2]};
    float ret[16];
    int n = intersect_rect_quad(rect, quad, ret);
    if (n < 1) return 0;
    float point[3 * 8], dep[8];
    float det1 = 1.0f / (m11 * m22 - m12 * m21);
    m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
    int cnum = 0;
    for (int j = 0; j < n; j++) {
        float k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        float k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (int i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb[i * 4 + a1] + k2 * Rb[i * 4 + a2];
        dep[cnum] = Sa[codeN] - dot3(normal2, point + cnum * 3);
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return 0;
    int maxc = flags & GB_NUMC_MASK;
    if (maxc > cnum) maxc = cnum;
    if (maxc < 1) maxc = 1;
    if (cnum <= maxc) {
        for (int j = 0; j < cnum; j++) {
            for (int i = 0; i < 3; i++) contact[j].pos[i] = point[j * 3 + i] + pa[i];
            contact[j].depth = dep[j];
        }
    } else {
        int i1 = 0;
        float maxdepth = dep[0];
        for (int i = 1; i < cnum; i++)
            if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
        int iret[8];
        cull_points(cnum, ret, maxc, i1, iret);
        for (int j = 0; j < maxc; j++) {
            for (int i = 0; i < 3; i++) contact[j].pos[i] = point[iret[j] * 3 + i] + pa[i];
            contact[j].depth = dep[iret[j]];
        }
        cnum = maxc;
    }
    *return_code = code;
    return cnum;
}

// box.cpp:741-767 dCollideBoxBox
__device__ inline int collide_box_box(const GeomView &o1, const GeomView &o2, int flags, CPoint *c, int *code_out) {
    float normal[3], depth;
    int code = 0;
    int num = box_box(o1.pos, o1.R, o1.dims, o2.pos, o2.R, o2.dims, normal, &depth, &code, flags, c);
    for (int i = 0; i < num; i++) { c[i].normal[0] = -normal[0]; c[i].normal[1] = -normal[1]; c[i].normal[2] = -normal[2]; }
    if (code_out) *code_out = num ? code : 0;
    return num;
}

// box.cpp:770-903 dCollideBoxPlane
__device__ inline int collide_box_plane(const GeomView &o1, const GeomView &o2, int flags, CPoint *contact) {
    const float *R = o1.R, *n = o2.dims, *side = o1.dims;
    float Q1 = d3_14(n, R + 0), Q2 = d3_14(n, R + 1), Q3 = d3_14(n, R + 2);
    float A_[3] = {side[0] * Q1, side[1] * Q2, side[2] * Q3};
    float B_[3] = {fabsf(A_[0]), fabsf(A_[1]), fabsf(A_[2])};
    float depth = n[3] + 0.5f * (B_[0] + B_[1] + B_[2]) - dot3(n, o1.pos);
    if (depth < 0) return 0;
    int maxc = flags & GB_NUMC_MASK;
    if (maxc > 4) maxc = 4;
    float p[3] = {o1.pos[0], o1.pos[1], o1.pos[2]};
    for (int i = 0; i < 3; i++) {
        if (A_[i] > 0) { p[0] -= 0.5f * side[i] * R[0 + i]; p[1] -= 0.5f * side[i] * R[4 + i]; p[2] -= 0.5f * side[i] * R[8 + i]; }
        else { p[0] += 0.5f * side[i] * R[0 + i]; p[1] += 0.5f * side[i] * R[4 + i]; p[2] += 0.5f * side[i] * R[8 + i]; }
    }
    contact[0].pos[0] = p[0]; contact[0].pos[1] = p[1]; contact[0].pos[2] = p[2];
    contact[0].depth = depth;
    int ret = 1;
    if (maxc > 1) {
        // the reference's goto ladder: second contact along the side with the
        // smallest projected length, third along the next smallest
        int s1, s2;
        const float B1 = B_[0], B2 = B_[1], B3 = B_[2];
        if (B1 < B2) {
            if (B3 < B1) { s1 = 2; s2 = (B1 < B2) ? 0 : 1; }
            else { s1 = 0; s2 = (B2 < B3) ? 1 : 2; }
        } else {
            if (B3 < B2) { s1 = 2; s2 = (B1 < B2) ? 0 : 1; }
            else { s1 = 1; s2 = (B1 < B3) ? 0 : 2; }
        }
        int sides[2] = {s1, s2};
        for (int k = 0; k < 2; k++) {
            int j = sides[k];
            if (depth - B_[j] < 0) break;
            float sg = (A_[j] > 0) ? 1.0f : -1.0f;
            if (sg > 0) { contact[1 + k].pos[0] = p[0] + side[j] * R[0 + j]; contact[1 + k].pos[1] = p[1] + side[j] * R[4 + j]; contact[1 + k].pos[2] = p[2] + side[j] * R[8 + j]; }
            else { contact[1 + k].pos[0] = p[0] - side[j] * R[0 + j]; contact[1 + k].pos[1] = p[1] - side[j] * R[4 + j]; contact[1 + k].pos[2] = p[2] - side[j] * R[8 + j]; }
            contact[1 + k].depth = depth - B_[j];
            ret++;
            if (maxc == 2) break;
        }
        if (maxc == 4 && ret == 3) {
            float d4 = contact[1].depth + contact[2].depth - depth;
            if (d4 > 0) {
                contact[3].pos[0] = contact[1].pos[0] + contact[2].pos[0] - p[0];
                contact[3].pos[1] = contact[1].pos[1] + contact[2].pos[1] - p[1];
                contact[3].pos[2] = contact[1].pos[2] + contact[2].pos[2] - p[2];
                contact[3].depth = d4;
                ret++;
            }
        }
    }
    for (int i = 0; i < ret; i++) { contact[i].normal[0] = n[0]; contact[i].normal[1] = n[1]; contact[i].normal[2] = n[2]; }
    return ret;
}

// sphere.cpp:131-219 dCollideSphereBox
__device__ inline int collide_sphere_box(const GeomView &o1, const GeomView &o2, CPoint *contact) {
    float l[3], t[4], p[3], q[3], r[3];
    int onborder = 0;
    const float *R = o2.R;
    p[0] = o1.pos[0] - o2.pos[0]; p[1] = o1.pos[1] - o2.pos[1]; p[2] = o1.pos[2] - o2.pos[2];
    for (int i = 0; i < 3; i++) {
        l[i] = o2.dims[i] * 0.5f;
        t[i] = d3_14(p, R + i);
        if (t[i] < -l[i]) { t[i] = -l[i]; onborder = 1; }
        if (t[i] > l[i]) { t[i] = l[i]; onborder = 1; }
    }
    if (!onborder) {
        float min_distance = l[0] - fabsf(t[0]);
        int mini = 0;
        for (int i = 1; i < 3; i++) {
            float fd = l[i] - fabsf(t[i]);
            if (fd < min_distance) { min_distance = fd; mini = i; }
        }
        contact->pos[0] = o1.pos[0]; contact->pos[1] = o1.pos[1]; contact->pos[2] = o1.pos[2];
        float tmp[3] = {0, 0, 0};
        tmp[mini] = (t[mini] > 0) ? 1.0f : -1.0f;
        m0_331(contact->normal, R, tmp);
        contact->depth = min_distance + o1.dims[0];
        return 1;
    }
    t[3] = 0;
    m0_331(q, R, t);
    r[0] = p[0] - q[0]; r[1] = p[1] - q[1]; r[2] = p[2] - q[2];
    float depth = o1.dims[0] - sqrtf(dot3(r, r));
    if (depth < 0) return 0;
    contact->pos[0] = q[0] + o2.pos[0]; contact->pos[1] = q[1] + o2.pos[1]; contact->pos[2] = q[2] + o2.pos[2];
    contact->normal[0] = r[0]; contact->normal[1] = r[1]; contact->normal[2] = r[2];
    normalize3(contact->normal);
    contact->depth = depth;
    return 1;
}

// sphere.cpp:222-251 dCollideSpherePlane
__device__ inline int collide_sphere_plane(const GeomView &o1, const GeomView &o2, CPoint *c) {
    const float *pl = o2.dims;
    float k = dot3(o1.pos, pl);
    float depth = pl[3] - k + o1.dims[0];
    if (depth >= 0) {
        c->normal[0] = pl[0]; c->normal[1] = pl[1]; c->normal[2] = pl[2];
        c->pos[0] = o1.pos[0] - pl[0] * o1.dims[0];
        c->pos[1] = o1.pos[1] - pl[1] * o1.dims[0];
        c->pos[2] = o1.pos[2] - pl[2] * o1.dims[0];
        c->depth = depth;
        return 1;
    }
    return 0;
}

// capsule.cpp:130-161 dCollideCapsuleSphere
__device__ inline int collide_capsule_sphere(const GeomView &o1, const GeomView &o2, CPoint *c) {
    const float *R = o1.R;
    float alpha = R[2] * (o2.pos[0] - o1.pos[0]) + R[6] * (o2.pos[1] - o1.pos[1]) + R[10] * (o2.pos[2] - o1.pos[2]);
    float lz2 = o1.dims[1] * 0.5f;
    if (alpha > lz2) alpha = lz2;
    if (alpha < -lz2) alpha = -lz2;
    float p[3] = {o1.pos[0] + alpha * R[2], o1.pos[1] + alpha * R[6], o1.pos[2] + alpha * R[10]};
    return collide_spheres(p, o1.dims[0], o2.pos, o2.dims[0], c);
}

// capsule.cpp:164-235 dCollideCapsuleBox
__device__ inline int collide_capsule_box(const GeomView &o1, const GeomView &o2, int flags, CPoint *contact) {
    const float *R1 = o1.R;
    float clen = o1.dims[1] * 0.5f;
    float p1[3] = {o1.pos[0] + clen * R1[2], o1.pos[1] + clen * R1[6], o1.pos[2] + clen * R1[10]};
    float p2[3] = {o1.pos[0] - clen * R1[2], o1.pos[1] - clen * R1[6], o1.pos[2] - clen * R1[10]};
    float radius = o1.dims[0];
    float pl[3], pb[3];
    closest_line_box_points(p1, p2, o2.pos, o2.R, o2.dims, pl, pb);
    if (dist3(pl, pb) < 1e-6f) {
        float normal[3], depth;
        int code;
        float r2 = radius * 2.0f;
        float capboxside[4] = {r2, r2, o1.dims[1] + r2, 0};
        int num = box_box(o2.pos, o2.R, o2.dims, o1.pos, o1.R, capboxside, normal, &depth, &code, flags, contact);
        for (int i = 0; i < num; i++) { contact[i].normal[0] = normal[0]; contact[i].normal[1] = normal[1]; contact[i].normal[2] = normal[2]; }
        return num;
    }
    float zero3[3] = {pb[0], pb[1], pb[2]};
    return collide_spheres(pl, radius, zero3, 0, contact);
}

// capsule.cpp:238-353 dCollideCapsuleCapsule
__device__ inline int collide_capsule_capsule(const GeomView &o1, const GeomView &o2, int flags, CPoint *contact) {
    const float tolerance = 1e-5f;
    float lz1 = o1.dims[1] * 0.5f, lz2 = o2.dims[1] * 0.5f;
    const float *pos1 = o1.pos, *pos2 = o2.pos;
    float axis1[3] = {o1.R[2], o1.R[6], o1.R[10]};
    float axis2[3] = {o2.R[2], o2.R[6], o2.R[10]};
    float sphere1[3], sphere2[3];
    float a1a2 = dot3(axis1, axis2);
    float det = 1.0f - a1a2 * a1a2;
    if (det < tolerance) {
        if (a1a2 < 0) { axis2[0] = -axis2[0]; axis2[1] = -axis2[1]; axis2[2] = -axis2[2]; }
        float q[3];
        for (int i = 0; i < 3; i++) q[i] = pos1[i] - pos2[i];
        float k = dot3(axis1, q);
        float a1lo = -lz1, a1hi = lz1, a2lo = -lz2 - k, a2hi = lz2 - k;
        float lo = (a1lo > a2lo) ? a1lo : a2lo;
        float hi = (a1hi < a2hi) ? a1hi : a2hi;
        if (lo <= hi) {
            int num_contacts = flags & GB_NUMC_MASK;
            if (num_contacts >= 2 && lo < hi) {
                for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + lo * axis1[i];
                for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (lo + k) * axis2[i];
                int n1 = collide_spheres(sphere1, o1.dims[0], sphere2, o2.dims[0], contact);
                if (n1) {
                    for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + hi * axis1[i];
                    for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (hi + k) * axis2[i];
                    int n2 = collide_spheres(sphere1, o1.dims[0], sphere2, o2.dims[0], contact + 1);
                    if (n2) return 2;
                }
            }
            float alpha1 = (lo + hi) * 0.5f;
            float alpha2 = alpha1 + k;
            for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + alpha1 * axis1[i];
            for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + alpha2 * axis2[i];
            return collide_spheres(sphere1, o1.dims[0], sphere2, o2.dims[0], contact);
        }
    }
    float a1[3], a2[3], b1[3], b2[3];
    for (int i = 0; i < 3; i++) {
        a1[i] = pos1[i] + axis1[i] * lz1; a2[i] = pos1[i] - axis1[i] * lz1;
        b1[i] = pos2[i] + axis2[i] * lz2; b2[i] = pos2[i] - axis2[i] * lz2;
    }
    closest_segment_points(a1, a2, b1, b2, sphere1, sphere2);
    return collide_spheres(sphere1, o1.dims[0], sphere2, o2.dims[0], contact);
}

// capsule.cpp:356-415 dCollideCapsulePlane
__device__ inline int collide_capsule_plane(const GeomView &o1, const GeomView &o2, int flags, CPoint *contact) {
    const float *pl = o2.dims, *R = o1.R;
    float lz = o1.dims[1], rad = o1.dims[0];
    float sign = (d3_14(pl, R + 2) > 0) ? -1.0f : 1.0f;
    float p[3];
    p[0] = o1.pos[0] + R[2] * lz * 0.5f * sign;
    p[1] = o1.pos[1] + R[6] * lz * 0.5f * sign;
    p[2] = o1.pos[2] + R[10] * lz * 0.5f * sign;
    float k = dot3(p, pl);
    float depth = pl[3] - k + rad;
    if (depth < 0) return 0;
    contact[0].normal[0] = pl[0]; contact[0].normal[1] = pl[1]; contact[0].normal[2] = pl[2];
    contact[0].pos[0] = p[0] - pl[0] * rad; contact[0].pos[1] = p[1] - pl[1] * rad; contact[0].pos[2] = p[2] - pl[2] * rad;
    contact[0].depth = depth;
    int nc = 1;
    if ((flags & GB_NUMC_MASK) >= 2) {
        p[0] = o1.pos[0] - R[2] * lz * 0.5f * sign;
        p[1] = o1.pos[1] - R[6] * lz * 0.5f * sign;
        p[2] = o1.pos[2] - R[10] * lz * 0.5f * sign;
        k = dot3(p, pl);
        depth = pl[3] - k + rad;
        if (depth >= 0) {
            contact[1].normal[0] = pl[0]; contact[1].normal[1] = pl[1]; contact[1].normal[2] = pl[2];
            contact[1].pos[0] = p[0] - pl[0] * rad; contact[1].pos[1] = p[1] - pl[1] * rad; contact[1].pos[2] = p[2] - pl[2] * rad;
            contact[1].depth = depth;
            nc = 2;
        }
    }
    return nc;
}

// collision_kernel.cpp:166-190 collider table + :292-338 dCollide reversal,
// for the four classes (0 sphere, 1 box, 2 capsule, 4 plane).
__device__ inline int collide_pair(const GeomView &a, const GeomView &b, int flags, CPoint *c, int *code) {
    if ((flags & GB_NUMC_MASK) == 0) return 0;
    if (code) *code = -1;
    const GeomView *o1 = &a, *o2 = &b;
    int c1 = a.cls, c2 = b.cls;
    bool rev = false;
    // canonical order: sphere < box < capsule-first tables as the reference sets them
    // (sphere,sphere) (sphere,box) (sphere,plane) (box,box) (box,plane)
    // (capsule,sphere) (capsule,box) (capsule,capsule) (capsule,plane)
    auto swap_needed = [](int x, int y) -> bool {
        if (x == 1 && y == 0) return true;   // box,sphere
        if (x == 4 && y != 4) return true;   // plane,*
        if (x == 0 && y == 2) return true;   // sphere,capsule
        if (x == 1 && y == 2) return true;   // box,capsule
        return false;
    };
    if (swap_needed(c1, c2)) { o1 = &b; o2 = &a; rev = true; int t = c1; c1 = c2; c2 = t; }
    int n = 0;
    if (c1 == 0 && c2 == 0) n = collide_spheres(o1->pos, o1->dims[0], o2->pos, o2->dims[0], c);
    else if (c1 == 0 && c2 == 1) n = collide_sphere_box(*o1, *o2, c);
    else if (c1 == 0 && c2 == 4) n = collide_sphere_plane(*o1, *o2, c);
    else if (c1 == 1 && c2 == 1) n = collide_box_box(*o1, *o2, flags, c, code);
    else if (c1 == 1 && c2 == 4) n = collide_box_plane(*o1, *o2, flags, c);
    else if (c1 == 2 && c2 == 0) n = collide_capsule_sphere(*o1, *o2, c);
    else if (c1 == 2 && c2 == 1) n = collide_capsule_box(*o1, *o2, flags, c);
    else if (c1 == 2 && c2 == 2) n = collide_capsule_capsule(*o1, *o2, flags, c);
    else if (c1 == 2 && c2 == 4) n = collide_capsule_plane(*o1, *o2, flags, c);
    if (rev)
        for (int i = 0; i < n; i++) { c[i].normal[0] = -c[i].normal[0]; c[i].normal[1] = -c[i].normal[1]; c[i].normal[2] = -c[i].normal[2]; }
    return n;
}

}  // namespace gb
