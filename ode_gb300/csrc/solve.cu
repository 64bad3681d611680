// dWorldQuickStep on the device.
//
// Pipeline (reference stages in quickstep.cpp in brackets):
//   k_bodies      gravity, world-frame inverse inertia, implicit gyroscopic
//                 torque, rhs_tmp, fc = 0                  [Stage0_Bodies, 2b]
//   k_contact_m   rows per contact                           [Stage0_Joints]
//   k_rows        contact rows J/rhs/cfm/lo/hi/findex, J*rhs_tmp, invM J^T,
//                 Ad scaling, lambda init -- one pass       [2a, 2c, 4a, iMJ, Ad]
//   colouring     manifolds (runs of contacts on one body pair) get colours
//                 such that no two of a colour share a body
//   k_pgs         projected Gauss-Seidel: colours in sequence, the
//                 manifolds of a colour in parallel; one persistent
//                 cooperative launch with bounded grid barriers [4LCP]
//   k_islands     the same relaxation in the reference's own row order, one
//                 island per block (for lambda parity)      [4LCP, serial]
//   k_integrate   v += h fc; v += h invM f_ext; x, q update; AABB-ready pose
//                                                           [4b, 6a, 6b, util.cpp:583-692]
#include <cooperative_groups.h>
#include <math.h>

#include <algorithm>

#include <map>
#include <mutex>

#include "gbode_internal.h"
#include "../../include/gbode.h"

namespace gb {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ void load_rows3(const float4 *R3, float *m) {
    for (int r = 0; r < 3; r++) {
        float4 v = R3[r];
        m[4 * r] = v.x; m[4 * r + 1] = v.y; m[4 * r + 2] = v.z; m[4 * r + 3] = 0;
    }
}
__device__ __forceinline__ void store_rows3(float4 *R3, const float *m) {
    for (int r = 0; r < 3; r++) R3[r] = make_float4(m[4 * r], m[4 * r + 1], m[4 * r + 2], 0.f);
}
__device__ __forceinline__ float d41(const float *a, const float *b) { return a[0] * b[0] + a[4] * b[1] + a[8] * b[2]; }
// dMultiply0_331
__device__ __forceinline__ void mul0_331(float *r, const float *a, const float *b) {
    float r0 = dot3(a, b), r1 = dot3(a + 4, b), r2 = dot3(a + 8, b);
    r[0] = r0; r[1] = r1; r[2] = r2;
}
// dMultiply0_333: row i of a times b
__device__ __forceinline__ void mul0_333(float *r, const float *a, const float *b) {
    for (int i = 0; i < 3; i++) {
        float t0 = d41(b, a + 4 * i), t1 = d41(b + 1, a + 4 * i), t2 = d41(b + 2, a + 4 * i);
        r[4 * i] = t0; r[4 * i + 1] = t1; r[4 * i + 2] = t2; r[4 * i + 3] = 0;
    }
}
// dMultiply2_333: a * b^T
__device__ __forceinline__ void mul2_333(float *r, const float *a, const float *b) {
    for (int i = 0; i < 3; i++) {
        float t0 = dot3(b, a + 4 * i), t1 = dot3(b + 4, a + 4 * i), t2 = dot3(b + 8, a + 4 * i);
        r[4 * i] = t0; r[4 * i + 1] = t1; r[4 * i + 2] = t2; r[4 * i + 3] = 0;
    }
}
__device__ __forceinline__ void cross3(float *r, const float *a, const float *b) {
    float r0 = a[1] * b[2] - a[2] * b[1], r1 = a[2] * b[0] - a[0] * b[2], r2 = a[0] * b[1] - a[1] * b[0];
    r[0] = r0; r[1] = r1; r[2] = r2;
}

// ------------------------------------------------------------------ bodies
// quickstep.cpp:1176-1306 (Stage0_Bodies) and :1644-1690 (Stage2b)
__global__ void k_bodies(Bodies B, SolverParams P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    if (B.asleep && B.asleep[i]) return;  // not in any island this step
    const float h = P.dt;
    float4 lv = B.lvel[i], av = B.avel[i], fa = B.facc[i], ta = B.tacc[i], ps = B.pos[i];
    const float mass = lv.w, invMass = ps.w;
    int flags = __float_as_int(av.w);
    float facc[3] = {fa.x, fa.y, fa.z}, tacc[3] = {ta.x, ta.y, ta.z};
    // gravity: added per axis only when that component is non-zero
    if (P.gravity[0]) facc[0] += mass * P.gravity[0];
    if (P.gravity[1]) facc[1] += mass * P.gravity[1];
    if (P.gravity[2]) facc[2] += mass * P.gravity[2];
    float R[12], invIb[12], tmp[12], invIw[12];
    load_rows3(B.R + 3 * i, R);
    load_rows3(B.invIb + 3 * i, invIb);
    mul2_333(tmp, invIb, R);
    mul0_333(invIw, R, tmp);
    float avel[3] = {av.x, av.y, av.z};
    if ((flags & 1) && invMass > 0) {
        float Ib[12], I[12];
        load_rows3(B.Ib + 3 * i, Ib);
        mul2_333(tmp, Ib, R);
        mul0_333(I, R, tmp);
        float L[3];
        mul0_331(L, I, avel);
        float It[12] = {0, L[2], -L[1], 0, -L[2], 0, L[0], 0, L[1], -L[0], 0, 0};
        for (int k = 0; k < 12; ++k) It[k] = It[k] * h + I[k];
        float rh = 1.0f / h;
        L[0] *= rh; L[1] *= rh; L[2] *= rh;
        // dInvertMatrix3 (odemath.h:463-500)
        float det = It[0] * (It[5] * It[10] - It[9] * It[6]) - It[1] * (It[4] * It[10] - It[8] * It[6]) +
                    It[2] * (It[4] * It[9] - It[8] * It[5]);
        if (det != 0) {
            float r = 1.0f / det, iv[12];
            iv[0] = (It[5] * It[10] - It[6] * It[9]) * r;
            iv[1] = (It[9] * It[2] - It[1] * It[10]) * r;
            iv[2] = (It[1] * It[6] - It[5] * It[2]) * r;
            iv[4] = (It[6] * It[8] - It[4] * It[10]) * r;
            iv[5] = (It[0] * It[10] - It[8] * It[2]) * r;
            iv[6] = (It[4] * It[2] - It[0] * It[6]) * r;
            iv[8] = (It[4] * It[9] - It[8] * It[5]) * r;
            iv[9] = (It[8] * It[1] - It[0] * It[9]) * r;
            iv[10] = (It[0] * It[5] - It[1] * It[4]) * r;
            iv[3] = iv[7] = iv[11] = 0;
            mul0_333(It, I, iv);
            It[0] -= 1; It[5] -= 1; It[10] -= 1;
            float tau[3];
            mul0_331(tau, It, L);
            tacc[0] = tacc[0] + tau[0]; tacc[1] = tacc[1] + tau[1]; tacc[2] = tacc[2] + tau[2];
        }
    }
    B.facc[i] = make_float4(facc[0], facc[1], facc[2], 0.f);
    B.tacc[i] = make_float4(tacc[0], tacc[1], tacc[2], 0.f);
    store_rows3(B.invIw + 3 * i, invIw);
    const float rh = 1.0f / h;
    float rl[3], ra[3];
    rl[0] = -(facc[0] * invMass + lv.x * rh);
    rl[1] = -(facc[1] * invMass + lv.y * rh);
    rl[2] = -(facc[2] * invMass + lv.z * rh);
    mul0_331(ra, invIw, tacc);
    ra[0] = -(avel[0] * rh) - ra[0];
    ra[1] = -(avel[1] * rh) - ra[1];
    ra[2] = -(avel[2] * rh) - ra[2];
    B.rt[2 * i] = make_float4(rl[0], rl[1], rl[2], 0.f);
    B.rt[2 * i + 1] = make_float4(ra[0], ra[1], ra[2], 0.f);
    B.fc[2 * i] = make_float4(0.f, 0.f, 0.f, 0.f);
    B.fc[2 * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ rows
// joints/contact.cpp:49-122 getInfo1 (mu < 0 is treated as 0)
__device__ __forceinline__ int contact_m(const Surface &s) {
    int m = 1;
    if (s.mode & 0x001) {
        if (s.mu > 0) m++;
        if (s.mu2 > 0) m++;
        if (s.mode & 0x400) { if (!(s.rho < 0)) m++; if (!(s.rho2 < 0)) m++; if (!(s.rhoN < 0)) m++; }
    } else {
        if (s.mu > 0) m += 2;
        if (s.mode & 0x400) { if (!(s.rho < 0)) m += 3; }
    }
    return m;
}

__global__ void k_contact_m(const Contact *C, const Surface *S, const int *nc_dev, int *mcount) {
    int nc = *nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        mcount[c] = contact_m(S[C[c].surf]);
    }
}

// Rows over the capacity: the step keeps the first contacts whose rows fit
// (the solver's contact count is lowered with them), so every later stage
// sees one consistent, smaller problem, and ERR_ROW_OVERFLOW is reported.
__global__ void k_rows_total(DevCounters *dc, int row_cap, const int *rstart, const int *mcount, int *nc_dev) {
    if (dc->nrows > row_cap) {
        atomicOr(&dc->err, ERR_ROW_OVERFLOW);
        int lo = 0, hi = *nc_dev;  // the most leading contacts whose rows end within the capacity
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (rstart[mid - 1] + mcount[mid - 1] <= row_cap) lo = mid;
            else hi = mid - 1;
        }
        *nc_dev = lo;
        dc->nrows = lo > 0 ? rstart[lo - 1] + mcount[lo - 1] : 0;
    }
    dc->step_contacts = dc->ncontacts;
}

// Contact rows: getInfo2 (contact.cpp:126-347) + Stage2a scaling (quickstep.cpp
// :1555-1561) + Stage2c J*rhs_tmp (:1022-1055) + compute_invM_JT (:858-897) +
// Ad scaling (:2251-2316) for each of the contact's rows.
// Warm-start cache: (geom pair, contact slot) -> the contact's first three
// multipliers of the previous step, in an open-addressed table.
__device__ __forceinline__ unsigned long long warm_key(const Contact &k) {
    return ((unsigned long long)(unsigned)k.g1 << 40) ^ ((unsigned long long)(unsigned)k.g2 << 8) ^
           (unsigned long long)(unsigned)(k.slot & 0xff);
}
__device__ __forceinline__ unsigned warm_hash(unsigned long long k) {
    k ^= k >> 31; k *= 0x7fb5d329728ea185ull; k ^= k >> 27; k *= 0x81dadef4bc2dd44dull; k ^= k >> 33;
    return (unsigned)k;
}
// Two tables of mask+1 entries each; DevCounters.warm_parity (device-side,
// flipped by a kernel, so a recorded CUDA graph alternates them too) says
// which one holds the previous step.
struct WarmTable {
    const unsigned long long *keys;  // both tables (null: no warm start)
    const float4 *lam;
    unsigned mask;
    float scale;
};

// Stage2b/2c, compute_invM_JT and the Ad scaling (quickstep.cpp:1644-1747,
// :858-897, :2251-2316) for the m rows J[0..m) (layout of quickstep.cpp:
// 1500-1512, rhs and cfm not yet divided by h) of one constraint between
// bodies n0 and n1 (-1: static), written at rows r0..r0+m-1 with owner tag
// `owner` (contact index, or -1 - joint index) and starting multipliers lam0.
// Returns the effective mass 1 / (J M^-1 J^T) of the first row.
__device__ float finish_rows(float (*J)[16], const int *findex, int m, int r0, int n0, int n1, const Bodies &B,
                             const Rows &Rw, const SolverParams &P, int dyn_maxabs, int owner, const float *lam0) {
    const float rh = 1.0f / P.dt;
    float4 rt0l = B.rt[2 * n0], rt0a = B.rt[2 * n0 + 1];
    float4 rt1l = make_float4(0, 0, 0, 0), rt1a = rt1l;
    if (n1 >= 0) { rt1l = B.rt[2 * n1]; rt1a = B.rt[2 * n1 + 1]; }
    float I0[12], I1[12];
    float meff = 0.f;
    load_rows3(B.invIw + 3 * n0, I0);
    const float im0 = B.pos[n0].w;
    float im1 = 0.f;
    if (n1 >= 0) { load_rows3(B.invIw + 3 * n1, I1); im1 = B.pos[n1].w; }
    for (int r = 0; r < m; r++) {
        float *j = J[r];
        j[6] *= rh; j[7] *= rh;
        float in0[6] = {rt0l.x, rt0l.y, rt0l.z, rt0a.x, rt0a.y, rt0a.z};
        float sum = 0.f;
        for (int q = 0; q < 6; q++) sum += j[q] * in0[q];
        if (n1 >= 0) {
            float in1[6] = {rt1l.x, rt1l.y, rt1l.z, rt1a.x, rt1a.y, rt1a.z};
            for (int q = 0; q < 6; q++) sum += j[8 + q] * in1[q];
        }
        j[6] += sum;
        float M1[7], M2[7] = {0, 0, 0, 0, 0, 0, 0};
        M1[0] = im0 * j[0]; M1[1] = im0 * j[1]; M1[2] = im0 * j[2];
        mul0_331(M1 + 3, I0, j + 3);
        M1[6] = 0;
        if (dyn_maxabs) { float mx = fabsf(M1[0]); for (int q = 1; q < 6; q++) mx = fmaxf(mx, fabsf(M1[q])); M1[6] = mx; }
        if (n1 >= 0) {
            M2[0] = im1 * j[8]; M2[1] = im1 * j[9]; M2[2] = im1 * j[10];
            mul0_331(M2 + 3, I1, j + 11);
            if (dyn_maxabs) { float mx = fabsf(M2[0]); for (int q = 1; q < 6; q++) mx = fmaxf(mx, fabsf(M2[q])); M2[6] = mx; }
        }
        float sumA = 0.f;
        for (int q = 0; q < 6; q++) sumA += M1[q] * j[q];
        if (n1 >= 0) for (int q = 0; q < 6; q++) sumA += M2[q] * j[8 + q];
        if (r == 0) meff = sumA > 0.f ? 1.0f / sumA : 0.f;
        const float cfm_i = j[7];
        const float Ad = P.w / (sumA + cfm_i);
        const int gr = r0 + r;
        Rw.Ad[gr] = Ad;
        float jc = cfm_i * Ad, jr = j[6] * Ad;
        float s1[6], s2[6];
        for (int q = 0; q < 6; q++) s1[q] = j[q] * Ad;
        for (int q = 0; q < 6; q++) s2[q] = (n1 >= 0) ? j[8 + q] * Ad : j[8 + q];
        Rw.J1l[gr] = make_float4(s1[0], s1[1], s1[2], jr);
        Rw.J1a[gr] = make_float4(s1[3], s1[4], s1[5], jc);
        Rw.J2l[gr] = make_float4(s2[0], s2[1], s2[2], j[14]);
        Rw.J2a[gr] = make_float4(s2[3], s2[4], s2[5], j[15]);
        Rw.M1l[gr] = make_float4(M1[0], M1[1], M1[2], M1[6]);
        Rw.M1a[gr] = make_float4(M1[3], M1[4], M1[5], 0.f);
        Rw.M2l[gr] = make_float4(M2[0], M2[1], M2[2], M2[6]);
        Rw.M2a[gr] = make_float4(M2[3], M2[4], M2[5], 0.f);
        Rw.findex[gr] = findex[r] >= 0 ? r0 + findex[r] : -1;
        Rw.body[gr] = make_int2(n0, n1);
        Rw.contact[gr] = owner;
        Rw.lambda[gr] = lam0 ? lam0[r] : 0.f;
    }
    return meff;
}

// Per-contact inputs of the learned warm start (null pointers: not recorded)
struct LearnOut {
    float *feat;   // [contact][12]
    float *scale;  // [contact] weight scale s = m_eff * |g|
};

__global__ void k_rows(const Contact *C, const Surface *S, const int *nc_dev, const int *rstart, Bodies B,
                       Rows Rw, SolverParams P, int dyn_maxabs, WarmTable W, DevCounters *dc, LearnOut L) {
    const int nc = *nc_dev;
    const float h = P.dt, rh = 1.0f / h;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Contact k = C[c];
        Surface s = S[k.surf];
        const int m = contact_m(s);
        int r0 = rstart[c];
        if (r0 + m > Rw.n_cap) { atomicOr(&dc->err, ERR_ROW_OVERFLOW); continue; }
        // dJointAttach: a missing first body moves the second into slot 0
        int n0 = k.b1, n1 = k.b2, reverse = 0;
        if (n0 < 0) { n0 = k.b2; n1 = -1; reverse = 1; }
        float J[6][16];
        int findex[6];
        for (int r = 0; r < m; r++) {
            for (int q = 0; q < 16; q++) J[r][q] = 0.f;
            J[r][7] = P.cfm; J[r][14] = -INFINITY; J[r][15] = INFINITY;
            findex[r] = -1;
        }
        const int mode = s.mode;
        float erp = (mode & 0x008) ? s.soft_erp : P.erp;
        float kk = rh * erp;
        float depth = k.pos_depth.w - P.min_depth;
        if (depth < 0) depth = 0;
        float motionN = (mode & 0x080) ? s.motionN : 0.0f;
        const float pushout = kk * depth + motionN;
        bool bounce = (mode & 0x004) != 0 && s.bounce_vel >= 0;
        float outgoing = 0;
        float cval = pushout > P.max_vel ? P.max_vel : pushout;
        float normal[3] = {k.normal.x, k.normal.y, k.normal.z};
        if (reverse) { normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2]; }
        float cpos[3] = {k.pos_depth.x, k.pos_depth.y, k.pos_depth.z};
        float c1[3], c2[3] = {0, 0, 0};
        if (n1 >= 0) {
            float4 p1 = B.pos[n1];
            c2[0] = cpos[0] - p1.x; c2[1] = cpos[1] - p1.y; c2[2] = cpos[2] - p1.z;
            J[0][8] = -normal[0]; J[0][9] = -normal[1]; J[0][10] = -normal[2];
            cross3(&J[0][11], normal, c2);
            if (bounce) {
                float4 av = B.avel[n1], lv = B.lvel[n1];
                float a3[3] = {av.x, av.y, av.z}, l3[3] = {lv.x, lv.y, lv.z};
                outgoing = dot3(&J[0][11], a3) - dot3(normal, l3);
            }
        }
        {
            float4 p0 = B.pos[n0];
            c1[0] = cpos[0] - p0.x; c1[1] = cpos[1] - p0.y; c1[2] = cpos[2] - p0.z;
            J[0][0] = normal[0]; J[0][1] = normal[1]; J[0][2] = normal[2];
            cross3(&J[0][3], c1, normal);
            if (bounce) {
                float4 av = B.avel[n0], lv = B.lvel[n0];
                float a3[3] = {av.x, av.y, av.z}, l3[3] = {lv.x, lv.y, lv.z};
                outgoing += dot3(&J[0][3], a3) + dot3(normal, l3);
            }
        }
        if (bounce) {
            float neg = motionN - outgoing;
            if (neg > s.bounce_vel) {
                float newc = s.bounce * neg + motionN;
                if (newc > cval) cval = newc;
            }
        }
        J[0][6] = cval;
        if (mode & 0x010) J[0][7] = s.soft_cfm;
        J[0][14] = 0; J[0][15] = INFINITY;
        float tf1[3] = {0, 0, 0}, tf2[3] = {0, 0, 0};  // contact frame, for the learned features
        if (m > 1) {
            float t1[3], t2[3];
            if (mode & 0x002) {
                t1[0] = s.fdir1[0]; t1[1] = s.fdir1[1]; t1[2] = s.fdir1[2];
                cross3(t2, normal, t1);
            } else if (fabsf(normal[2]) > 0.7071067811865476f) {
                // odemath.cpp:224-251 dxPlaneSpace
                float a = normal[1] * normal[1] + normal[2] * normal[2];
                float kq = 1.0f / sqrtf(a);
                t1[0] = 0; t1[1] = -normal[2] * kq; t1[2] = normal[1] * kq;
                t2[0] = a * kq; t2[1] = -normal[0] * t1[2]; t2[2] = normal[0] * t1[1];
            } else {
                float a = normal[0] * normal[0] + normal[1] * normal[1];
                float kq = 1.0f / sqrtf(a);
                t1[0] = -normal[1] * kq; t1[1] = normal[0] * kq; t1[2] = 0;
                t2[0] = -normal[2] * t1[1]; t2[1] = normal[2] * t1[0]; t2[2] = a * kq;
            }
            for (int q = 0; q < 3; q++) { tf1[q] = t1[q]; tf2[q] = t2[q]; }
            int row = 1;
            const float mu = s.mu > 0 ? s.mu : 0.f;
            if (mu > 0) {
                float *r = J[row];
                r[0] = t1[0]; r[1] = t1[1]; r[2] = t1[2];
                cross3(r + 3, c1, t1);
                if (n1 >= 0) { r[8] = -t1[0]; r[9] = -t1[1]; r[10] = -t1[2]; cross3(r + 11, t1, c2); }
                if (mode & 0x020) r[6] = s.motion1;
                if (mode & 0x100) r[7] = s.slip1;
                r[14] = -mu; r[15] = mu;
                if (mode & 0x1000) findex[row] = 0;
                ++row;
            }
            const float mu2 = (mode & 0x001) ? (s.mu2 > 0 ? s.mu2 : 0.f) : mu;
            if (mu2 > 0) {
                float *r = J[row];
                r[0] = t2[0]; r[1] = t2[1]; r[2] = t2[2];
                cross3(r + 3, c1, t2);
                if (n1 >= 0) { r[8] = -t2[0]; r[9] = -t2[1]; r[10] = -t2[2]; cross3(r + 11, t2, c2); }
                if (mode & 0x040) r[6] = s.motion2;
                if (mode & 0x200) r[7] = s.slip2;
                r[14] = -mu2; r[15] = mu2;
                if (mode & 0x2000) findex[row] = 0;
                ++row;
            }
            if (mode & 0x400) {
                float rho[3] = {s.rho, (mode & 0x001) ? s.rho2 : s.rho, (mode & 0x001) ? s.rhoN : s.rho};
                const int bits[3] = {0x1000, 0x2000, 0x4000};
                const float *ax[3] = {t1, t2, normal};
                for (int q = 0; q < 3 && row < m; q++) {
                    if (rho[q] > 0) {
                        float *r = J[row];
                        r[3] = ax[q][0]; r[4] = ax[q][1]; r[5] = ax[q][2];
                        if (n1 >= 0) { r[11] = -ax[q][0]; r[12] = -ax[q][1]; r[13] = -ax[q][2]; }
                        r[14] = -rho[q]; r[15] = rho[q];
                        if (mode & bits[q]) findex[row] = 0;
                        ++row;
                    }
                    // rho == 0 is counted by getInfo1 but not written by getInfo2: the
                    // row stays as initialised (zero J, unbounded) at the end of the block
                }
            }
        }
        // warm start: the previous step's multipliers of this (geom pair, slot)
        float warm3[3] = {0.f, 0.f, 0.f};
        bool warm_found = false;
        if (W.keys) {
            const unsigned long long key = warm_key(k);
            const size_t tb = (size_t)(W.mask + 1) * dc->warm_parity;
            unsigned h = warm_hash(key) & W.mask;
            for (unsigned probe = 0; probe <= W.mask; probe++) {
                const unsigned long long kk = W.keys[tb + h];
                if (kk == key) {
                    const float4 l = W.lam[tb + h];
                    warm3[0] = l.x * W.scale; warm3[1] = l.y * W.scale; warm3[2] = l.z * W.scale;
                    warm_found = true;
                    break;
                }
                if (kk == ~0ull) break;
                h = (h + 1) & W.mask;
            }
        }
        float lam0[6] = {warm3[0], warm3[1], warm3[2], 0.f, 0.f, 0.f};
        const float meff = finish_rows(J, findex, m, r0, n0, n1, B, Rw, P, dyn_maxabs, c, lam0);
        if (L.feat) {
            // normal, contact-point relative velocity in the contact frame,
            // depth, effective mass, previous multipliers in units of s, found
            float v[3];
            {
                const float4 lv = B.lvel[n0], av = B.avel[n0];
                const float w[3] = {av.x, av.y, av.z};
                float wc[3];
                cross3(wc, w, c1);
                v[0] = lv.x + wc[0]; v[1] = lv.y + wc[1]; v[2] = lv.z + wc[2];
            }
            if (n1 >= 0) {
                const float4 lv = B.lvel[n1], av = B.avel[n1];
                const float w[3] = {av.x, av.y, av.z};
                float wc[3];
                cross3(wc, w, c2);
                v[0] -= lv.x + wc[0]; v[1] -= lv.y + wc[1]; v[2] -= lv.z + wc[2];
            }
            const float g = sqrtf(P.gravity[0] * P.gravity[0] + P.gravity[1] * P.gravity[1] + P.gravity[2] * P.gravity[2]);
            float sc = meff * (g > 0.f ? g : 1.f);
            if (!(sc > 0.f)) sc = 1.f;
            float *f = L.feat + (size_t)c * 12;
            f[0] = normal[0]; f[1] = normal[1]; f[2] = normal[2];
            f[3] = dot3(v, normal); f[4] = dot3(v, tf1); f[5] = dot3(v, tf2);
            f[6] = k.pos_depth.w; f[7] = meff;
            f[8] = warm3[0] / sc; f[9] = warm3[1] / sc; f[10] = warm3[2] / sc;
            f[11] = warm_found ? 1.f : 0.f;
            L.scale[c] = sc;
        }
    }
}

// ------------------------------------------------------------------ ball and hinge joints
// The joint table (uploaded when the joints change) and the per-step state.
struct JointTable {
    const int4 *info;  // type, node-0 body, node-1 body (-1: none), 1 if attached reversed
    const float4 *a1, *a2, *x1, *x2, *qrel;
    const float4 *l0;  // lostop histop vel fmax
    const float4 *l1;  // fudge bounce normal_cfm stop_erp
    const float4 *l2;  // stop_cfm, ball erp, ball cfm
    const float4 *v1, *v2;          // hinge2: angle vectors in body 1's frame; w = s0 / c0
    const float4 *m0, *m1, *m2;     // hinge2: axis-2 limot (as l0..l2), m2.y/z = suspension ERP/CFM
    int n;
    int *m, *rstart, *limit;
    float *lerr, *lam;  // limit error; [n][6] multipliers of the last step (warm start)
};

// dxPlaneSpace (odemath.cpp:224-251)
__device__ __forceinline__ void plane_space(const float *n, float *p, float *q) {
    if (fabsf(n[2]) > 0.7071067811865476f) {
        float a = n[1] * n[1] + n[2] * n[2];
        float k = 1.0f / sqrtf(a);
        p[0] = 0; p[1] = -n[2] * k; p[2] = n[1] * k;
        q[0] = a * k; q[1] = -n[0] * p[2]; q[2] = n[0] * p[1];
    } else {
        float a = n[0] * n[0] + n[1] * n[1];
        float k = 1.0f / sqrtf(a);
        p[0] = -n[1] * k; p[1] = n[0] * k; p[2] = 0;
        q[0] = -n[2] * p[1]; q[1] = n[2] * p[0]; q[2] = a * k;
    }
}
// device quaternions are stored (w, x, y, z) in float4 (x, y, z, w)
__device__ __forceinline__ void quat_of(float4 v, float *q) { q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w; }
// joint.cpp:421-492 getHingeAngle with rotation.cpp:201-228 dQMultiply1/2/3
__device__ float hinge_angle(const float *qb, const float *qc, const float *axis, const float *qi) {
    float qrel[4];
    if (qc) {
        float qq[4];
        qq[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
        qq[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
        qq[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
        qq[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
        qrel[0] = qq[0] * qi[0] + qq[1] * qi[1] + qq[2] * qi[2] + qq[3] * qi[3];
        qrel[1] = -qq[0] * qi[1] + qq[1] * qi[0] - qq[2] * qi[3] + qq[3] * qi[2];
        qrel[2] = -qq[0] * qi[2] + qq[2] * qi[0] - qq[3] * qi[1] + qq[1] * qi[3];
        qrel[3] = -qq[0] * qi[3] + qq[3] * qi[0] - qq[1] * qi[2] + qq[2] * qi[1];
    } else {
        qrel[0] = qb[0] * qi[0] - qb[1] * qi[1] - qb[2] * qi[2] - qb[3] * qi[3];
        qrel[1] = -qb[0] * qi[1] - qb[1] * qi[0] + qb[2] * qi[3] - qb[3] * qi[2];
        qrel[2] = -qb[0] * qi[2] - qb[2] * qi[0] + qb[3] * qi[1] - qb[1] * qi[3];
        qrel[3] = -qb[0] * qi[3] - qb[3] * qi[0] + qb[1] * qi[2] - qb[2] * qi[1];
    }
    const float cost2 = qrel[0];
    const float sint2 = sqrtf(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
    const float d = qrel[1] * axis[0] + qrel[2] * axis[1] + qrel[3] * axis[2];
    float theta = d >= 0 ? 2 * atan2f(sint2, cost2) : 2 * atan2f(sint2, -cost2);
    if (theta > 3.14159265358979323846f) theta -= 6.28318530717958647692f;
    return -theta;
}

// getInfo1 (ball.cpp:60-65, hinge.cpp:53-75) with the limit test
// (joint.cpp:574-593), and addLimot's motor torques for a powered joint at a
// limit (joint.cpp:655-700), which enter the bodies' torque accumulators
// before the right-hand side is formed.
__global__ void k_joint_m(JointTable T, Bodies B) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n; k += gridDim.x * blockDim.x) {
        const int4 in = T.info[k];
        if (B.asleep && B.asleep[in.y]) {  // the joint's component sleeps: no rows
            T.m[k] = 0;
            T.limit[k] = 0;
            continue;
        }
        int m = 3, limit = 0;
        float lerr = 0.f;
        if (in.x == 2) {  // dJointTypeHinge
            const float4 l0 = T.l0[k];
            const float lostop = l0.x, histop = l0.y, vel = l0.z, fmax = l0.w;
            m = fmax > 0 ? 6 : 5;
            if ((lostop >= -3.14159265358979323846f || histop <= 3.14159265358979323846f) && lostop <= histop) {
                float qb[4], qc[4], ax[3], qi[4];
                quat_of(B.q[in.y], qb);
                if (in.z >= 0) quat_of(B.q[in.z], qc);
                const float4 x1 = T.x1[k], qr = T.qrel[k];
                ax[0] = x1.x; ax[1] = x1.y; ax[2] = x1.z;
                qi[0] = qr.x; qi[1] = qr.y; qi[2] = qr.z; qi[3] = qr.w;
                const float angle = hinge_angle(qb, in.z >= 0 ? qc : nullptr, ax, qi);
                if (angle <= lostop) { limit = 1; lerr = angle - lostop; }
                else if (angle >= histop) { limit = 2; lerr = angle - histop; }
                if (limit) m = 6;
            }
            if (limit && fmax > 0 && lostop != histop) {
                float fm = fmax;
                if (vel > 0 || (vel == 0 && limit == 2)) fm = -fm;
                if ((limit == 1 && vel > 0) || (limit == 2 && vel < 0)) fm *= T.l1[k].x;
                float R0[12], a1[3], ax1[3];
                load_rows3(B.R + 3 * in.y, R0);
                const float4 x1 = T.x1[k];
                a1[0] = x1.x; a1[1] = x1.y; a1[2] = x1.z;
                mul0_331(ax1, R0, a1);
                const float t0 = fm * ax1[0], t1 = fm * ax1[1], t2 = fm * ax1[2];
                if (in.z >= 0) {
                    atomicAdd(&B.tacc[in.z].x, t0); atomicAdd(&B.tacc[in.z].y, t1); atomicAdd(&B.tacc[in.z].z, t2);
                }
                atomicAdd(&B.tacc[in.y].x, -t0); atomicAdd(&B.tacc[in.y].y, -t1); atomicAdd(&B.tacc[in.y].z, -t2);
            }
        }
        if (in.x == 6 && in.z >= 0) {  // dJointTypeHinge2 (hinge2.cpp:104-125)
            const float4 l0 = T.l0[k];
            const float lostop = l0.x, histop = l0.y, vel = l0.z, fmax = l0.w;
            m = 4;
            if ((lostop >= -3.14159265358979323846f || histop <= 3.14159265358979323846f) && lostop <= histop) {
                // measureAngle1 (hinge2.cpp:33-51)
                float R0[12], R1[12], p[3], q[3];
                load_rows3(B.R + 3 * in.y, R0);
                load_rows3(B.R + 3 * in.z, R1);
                const float4 x2 = T.x2[k], v1 = T.v1[k], v2 = T.v2[k];
                const float a2[3] = {x2.x, x2.y, x2.z};
                mul0_331(p, R1, a2);
                q[0] = R0[0] * p[0] + R0[4] * p[1] + R0[8] * p[2];  // dMultiply1_331
                q[1] = R0[1] * p[0] + R0[5] * p[1] + R0[9] * p[2];
                q[2] = R0[2] * p[0] + R0[6] * p[1] + R0[10] * p[2];
                const float x = v1.x * q[0] + v1.y * q[1] + v1.z * q[2];
                const float y = v2.x * q[0] + v2.y * q[1] + v2.z * q[2];
                const float angle = -atan2f(y, x);
                if (angle <= lostop) { limit = 1; lerr = angle - lostop; }
                else if (angle >= histop) { limit = 2; lerr = angle - histop; }
            }
            if (limit || fmax > 0) m++;
            if (T.m0[k].w > 0) m++;  // axis 2 is powered (never limited)
            if (limit && fmax > 0 && lostop != histop) {
                float fm = fmax;
                if (vel > 0 || (vel == 0 && limit == 2)) fm = -fm;
                if ((limit == 1 && vel > 0) || (limit == 2 && vel < 0)) fm *= T.l1[k].x;
                float R0[12], a1[3], ax1[3];
                load_rows3(B.R + 3 * in.y, R0);
                const float4 x1 = T.x1[k];
                a1[0] = x1.x; a1[1] = x1.y; a1[2] = x1.z;
                mul0_331(ax1, R0, a1);
                const float t0 = fm * ax1[0], t1 = fm * ax1[1], t2 = fm * ax1[2];
                atomicAdd(&B.tacc[in.z].x, t0); atomicAdd(&B.tacc[in.z].y, t1); atomicAdd(&B.tacc[in.z].z, t2);
                atomicAdd(&B.tacc[in.y].x, -t0); atomicAdd(&B.tacc[in.y].y, -t1); atomicAdd(&B.tacc[in.y].z, -t2);
            }
        }
        T.m[k] = m;
        T.limit[k] = limit;
        T.lerr[k] = lerr;
    }
}

// joint.cpp:596-790 addLimot, rotational, into one row r (J layout as k_rows)
__device__ void limot_row(float *r, const float *ax1, int n0, int n1, const Bodies &B, float fps, int limit,
                          float lerr, float4 l0, float4 l1, float stop_cfm) {
    const float lostop = l0.x, histop = l0.y, vel = l0.z, fmax = l0.w;
    const float bounce = l1.y, normal_cfm = l1.z, stop_erp = l1.w;
    r[3] = ax1[0]; r[4] = ax1[1]; r[5] = ax1[2];
    if (n1 >= 0) { r[11] = -ax1[0]; r[12] = -ax1[1]; r[13] = -ax1[2]; }
    int powered = fmax > 0;
    if (limit && lostop == histop) powered = 0;
    if (powered) {
        r[7] = normal_cfm;
        if (!limit) { r[6] = vel; r[14] = -fmax; r[15] = fmax; }
    }
    if (limit) {
        const float ks = fps * stop_erp;
        r[6] = -ks * lerr;
        r[7] = stop_cfm;
        if (lostop == histop) {
            r[14] = -INFINITY; r[15] = INFINITY;
        } else {
            if (limit == 1) { r[14] = 0; r[15] = INFINITY; }
            else { r[14] = -INFINITY; r[15] = 0; }
            if (bounce > 0) {
                const float4 w0 = B.avel[n0];
                float v = w0.x * ax1[0] + w0.y * ax1[1] + w0.z * ax1[2];
                if (n1 >= 0) { const float4 w1 = B.avel[n1]; v -= w1.x * ax1[0] + w1.y * ax1[1] + w1.z * ax1[2]; }
                if (limit == 1) { if (v < 0) { const float nc = -bounce * v; if (nc > r[6]) r[6] = nc; } }
                else { if (v > 0) { const float nc = -bounce * v; if (nc < r[6]) r[6] = nc; } }
            }
        }
    }
}

// odemath.cpp:95-151 dxSafeNormalize3
__device__ bool safe_normalize3(float *a) {
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

// joint.cpp:165-226 setBall2 into rows 0-2 of J: the first row along `axis`
__device__ void set_ball2(float (*J)[16], const Bodies &B, int n0, int n1, float fps, float erp, const float *anchor1,
                          const float *anchor2, const float *axis, float erp1) {
    float R0[12], a1[3], a2[3], q1[3], q2[3];
    plane_space(axis, q1, q2);
    const float *dirs[3] = {axis, q1, q2};
    load_rows3(B.R + 3 * n0, R0);
    mul0_331(a1, R0, anchor1);
    for (int r = 0; r < 3; r++) {
        for (int i = 0; i < 3; i++) J[r][i] = dirs[r][i];
        cross3(&J[r][3], a1, dirs[r]);
    }
    const float4 p0 = B.pos[n0];
    a1[0] += p0.x; a1[1] += p0.y; a1[2] += p0.z;
    const float k1 = fps * erp1, k = fps * erp;
    float d[3];
    if (n1 >= 0) {
        float R1[12];
        load_rows3(B.R + 3 * n1, R1);
        for (int r = 0; r < 3; r++)
            for (int i = 0; i < 3; i++) J[r][8 + i] = -dirs[r][i];
        mul0_331(a2, R1, anchor2);
        for (int r = 0; r < 3; r++) cross3(&J[r][11], dirs[r], a2);
        const float4 p1 = B.pos[n1];
        a2[0] += p1.x; a2[1] += p1.y; a2[2] += p1.z;
        d[0] = a2[0] - a1[0]; d[1] = a2[1] - a1[1]; d[2] = a2[2] - a1[2];
    } else {
        d[0] = anchor2[0] - a1[0]; d[1] = anchor2[1] - a1[1]; d[2] = anchor2[2] - a1[2];
    }
    J[0][6] = k1 * dot3(axis, d);
    J[1][6] = k * dot3(q1, d);
    J[2][6] = k * dot3(q2, d);
}

__global__ void k_joint_rows_total(DevCounters *dc, int row_cap) {
    dc->nrows_contacts = dc->nrows;
    int total = dc->nrows + dc->njoint_rows;
    if (total > row_cap) { atomicOr(&dc->err, ERR_ROW_OVERFLOW); total = row_cap; }
    dc->nrows = total;
}

// joint.cpp:111-157 setBall into rows 0-2 of J
__device__ void set_ball(float (*J)[16], const Bodies &B, int n0, int n1, float fps, float erp, const float *anchor1,
                         const float *anchor2) {
    float R0[12], a1[3], a2[3];
    load_rows3(B.R + 3 * n0, R0);
    J[0][0] = 1; J[1][1] = 1; J[2][2] = 1;
    mul0_331(a1, R0, anchor1);
    // dSetCrossMatrixMinus (odemath.h:288-297) into the angular block of body 1
    J[0][4] = a1[2]; J[0][5] = -a1[1];
    J[1][3] = -a1[2]; J[1][5] = a1[0];
    J[2][3] = a1[1]; J[2][4] = -a1[0];
    const float k = fps * erp;
    const float4 p0 = B.pos[n0];
    const float pos0[3] = {p0.x, p0.y, p0.z};
    if (n1 >= 0) {
        float R1[12];
        load_rows3(B.R + 3 * n1, R1);
        J[0][8] = -1; J[1][9] = -1; J[2][10] = -1;
        mul0_331(a2, R1, anchor2);
        // dSetCrossMatrixPlus (odemath.h:277-286) into the angular block of body 2
        J[0][12] = -a2[2]; J[0][13] = a2[1];
        J[1][11] = a2[2]; J[1][13] = -a2[0];
        J[2][11] = -a2[1]; J[2][12] = a2[0];
        const float4 p1 = B.pos[n1];
        const float pos1[3] = {p1.x, p1.y, p1.z};
        for (int j = 0; j < 3; j++) J[j][6] = k * (a2[j] + pos1[j] - a1[j] - pos0[j]);
    } else {
        for (int j = 0; j < 3; j++) J[j][6] = k * (anchor2[j] - a1[j] - pos0[j]);
    }
}

// getInfo2 of ball (ball.cpp:68-76) and hinge (hinge.cpp:78-150, with
// joint.cpp:596-790 addLimot for the limit/motor row), then the rows'
// finishing as for contacts.  Joint rows follow the contact rows.
__global__ void k_joint_rows(JointTable T, Bodies B, Rows Rw, SolverParams P, int dyn_maxabs, DevCounters *dc,
                             int warm) {
    const int base = dc->nrows_contacts;
    const float fps = 1.0f / P.dt;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n; k += gridDim.x * blockDim.x) {
        const int4 in = T.info[k];
        const int m = T.m[k], r0 = base + T.rstart[k];
        if (m == 0) continue;
        if (r0 + m > Rw.n_cap) { atomicOr(&dc->err, ERR_ROW_OVERFLOW); continue; }
        const int n0 = in.y, n1 = in.z;
        float J[6][16];
        int findex[6];
        for (int r = 0; r < m; r++) {
            for (int q = 0; q < 16; q++) J[r][q] = 0.f;
            J[r][7] = P.cfm; J[r][14] = -INFINITY; J[r][15] = INFINITY;
            findex[r] = -1;
        }
        const float4 fa1 = T.a1[k], fa2 = T.a2[k];
        const float anchor1[3] = {fa1.x, fa1.y, fa1.z}, anchor2[3] = {fa2.x, fa2.y, fa2.z};
        if (in.x == 1) {  // ball: its own ERP and CFM
            const float4 l2 = T.l2[k];
            J[0][7] = l2.z; J[1][7] = l2.z; J[2][7] = l2.z;
            set_ball(J, B, n0, n1, fps, l2.y, anchor1, anchor2);
        } else if (in.x == 6) {  // hinge2 (hinge2.cpp:147-207)
            float R0[12], R1[12], ax1[3], ax2[3], q[3];
            load_rows3(B.R + 3 * n0, R0);
            load_rows3(B.R + 3 * n1, R1);
            const float4 x1 = T.x1[k], x2 = T.x2[k], v1 = T.v1[k], v2 = T.v2[k], m2 = T.m2[k];
            const float axis1[3] = {x1.x, x1.y, x1.z}, axis2[3] = {x2.x, x2.y, x2.z};
            mul0_331(ax1, R0, axis1);
            mul0_331(ax2, R1, axis2);
            cross3(q, ax1, ax2);
            const float sa = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            const float ca = dot3(ax1, ax2);
            safe_normalize3(q);
            set_ball2(J, B, n0, n1, fps, P.erp, anchor1, anchor2, ax1, m2.y);
            J[0][7] = m2.z;  // suspension CFM
            for (int i = 0; i < 3; i++) { J[3][3 + i] = q[i]; J[3][11 + i] = -q[i]; }
            J[3][6] = fps * P.erp * (v2.w * sa - v1.w * ca);  // k * (c0 * s - s0 * c)
            int row = 4;
            const float4 l0 = T.l0[k];
            const int limit = T.limit[k];
            if (limit || l0.w > 0) {
                limot_row(J[row], ax1, n0, n1, B, fps, limit, T.lerr[k], l0, T.l1[k], T.l2[k].x);
                ++row;
            }
            if (T.m0[k].w > 0) limot_row(J[row], ax2, n0, n1, B, fps, 0, 0.f, T.m0[k], T.m1[k], m2.x);
        } else {  // hinge
            set_ball(J, B, n0, n1, fps, P.erp, anchor1, anchor2);
            float R0[12], ax1[3], p[3], q[3], b[3];
            load_rows3(B.R + 3 * n0, R0);
            const float4 x1 = T.x1[k], x2 = T.x2[k];
            const float axis1[3] = {x1.x, x1.y, x1.z}, axis2[3] = {x2.x, x2.y, x2.z};
            mul0_331(ax1, R0, axis1);
            plane_space(ax1, p, q);
            for (int i = 0; i < 3; i++) { J[3][3 + i] = p[i]; J[4][3 + i] = q[i]; }
            if (n1 >= 0) {
                for (int i = 0; i < 3; i++) { J[3][11 + i] = -p[i]; J[4][11 + i] = -q[i]; }
                float R1[12], ax2[3];
                load_rows3(B.R + 3 * n1, R1);
                mul0_331(ax2, R1, axis2);
                cross3(b, ax1, ax2);
            } else {
                cross3(b, ax1, axis2);
            }
            const float kk = fps * P.erp;
            J[3][6] = kk * dot3(b, p);
            J[4][6] = kk * dot3(b, q);
            if (m == 6)  // addLimot, rotational
                limot_row(J[5], ax1, n0, n1, B, fps, T.limit[k], T.lerr[k], T.l0[k], T.l1[k], T.l2[k].x);
        }
        float lam0[6] = {0, 0, 0, 0, 0, 0};
        if (warm)
            for (int r = 0; r < m; r++) lam0[r] = T.lam[6 * k + r];
        finish_rows(J, findex, m, r0, n0, n1, B, Rw, P, dyn_maxabs, -1 - k, lam0);
    }
}

// the joints' multipliers after the solve, for the next step's start
__global__ void k_joint_store(JointTable T, Rows Rw, const DevCounters *dc) {
    const int base = dc->nrows_contacts;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n; k += gridDim.x * blockDim.x) {
        const int m = T.m[k], r0 = base + T.rstart[k];
        if (m == 0) continue;  // not solved this step: the multipliers are kept
        for (int r = 0; r < 6; r++) T.lam[6 * k + r] = r < m ? Rw.lambda[r0 + r] : 0.f;
    }
}

// Learned start: the MLP's prediction (units of s) for every triplet contact,
// projected onto the rows' bounds (normal >= 0, |friction| <= mu * normal);
// the plain start (previous-step multipliers) is kept in lam_alt.
__global__ void k_learned_apply(const int *nc_dev, const int *rstart, const int *mcount, const float *scale,
                                const float *pred, Rows Rw, float *lam_alt, const DevCounters *dc) {
    const int nc = *nc_dev;
    for (int r = dc->nrows_contacts + blockIdx.x * blockDim.x + threadIdx.x; r < dc->nrows; r += gridDim.x * blockDim.x)
        lam_alt[r] = Rw.lambda[r];  // joint rows keep their start
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int r0 = rstart[c], m = mcount[c];
        for (int r = r0; r < r0 + m; r++) lam_alt[r] = Rw.lambda[r];
        if (m != 3 || Rw.findex[r0] >= 0 || Rw.findex[r0 + 1] != r0 || Rw.findex[r0 + 2] != r0) continue;
        const float s = scale[c];
        const float ln = fmaxf(pred[3 * c] * s, 0.f);
        const float h1 = fabsf(Rw.J2a[r0 + 1].w * ln), h2 = fabsf(Rw.J2a[r0 + 2].w * ln);
        Rw.lambda[r0] = ln;
        Rw.lambda[r0 + 1] = fminf(fmaxf(pred[3 * c + 1] * s, -h1), h1);
        Rw.lambda[r0 + 2] = fminf(fmaxf(pred[3 * c + 2] * s, -h2), h2);
    }
}

// clear the table the step writes (the one not holding the previous step)
__global__ void k_warm_clear(unsigned long long *keys, unsigned mask, const DevCounters *dc) {
    unsigned long long *t = keys + (size_t)(mask + 1) * (dc->warm_parity ^ 1);
    for (size_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= mask; i += (size_t)gridDim.x * blockDim.x) t[i] = ~0ull;
}
__global__ void k_warm_flip(DevCounters *dc) { dc->warm_parity ^= 1; }

__global__ void k_warm_store(const Contact *C, const int *nc_dev, const int *rstart, const int *mcount, Rows Rw,
                             unsigned long long *keys_all, float4 *lam_all, unsigned mask, const DevCounters *dc) {
    const int nc = *nc_dev;
    const size_t tb = (size_t)(mask + 1) * (dc->warm_parity ^ 1);
    unsigned long long *keys = keys_all + tb;
    float4 *lam = lam_all + tb;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Contact k = C[c];
        const unsigned long long key = warm_key(k);
        unsigned h = warm_hash(key) & mask;
        for (unsigned probe = 0; probe <= mask; probe++) {
            unsigned long long prev = atomicCAS(&keys[h], ~0ull, key);
            if (prev == ~0ull || prev == key) {
                const int r0 = rstart[c], m = mcount[c];
                lam[h] = make_float4(Rw.lambda[r0], m > 1 ? Rw.lambda[r0 + 1] : 0.f, m > 2 ? Rw.lambda[r0 + 2] : 0.f, 0.f);
                break;
            }
            h = (h + 1) & mask;
        }
    }
}

// ------------------------------------------------------------------ manifolds + colouring
// A manifold is a maximal run of consecutive contacts on the same geom pair
// (hence the same body pair); its rows are relaxed by one thread in sequence,
// so manifolds, not rows, are what the colouring separates.
__global__ void k_manifold_heads(const Contact *C, const int *nc_dev, int *head) {
    int nc = *nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        int h = 1;
        if (c > 0) {
            const Contact a = C[c - 1], b = C[c];
            int a0 = a.b1 >= 0 ? a.b1 : a.b2, a1 = a.b1 >= 0 ? a.b2 : -1;
            int b0 = b.b1 >= 0 ? b.b1 : b.b2, b1 = b.b1 >= 0 ? b.b2 : -1;
            // one manifold per geom pair: a body against two static planes
            // (a box in a corner) gives two manifolds, each at most maxc contacts
            h = !(a0 == b0 && a1 == b1 && a.g1 == b.g1 && a.g2 == b.g2);
        }
        head[c] = h;
    }
}
__global__ void k_manifold_starts(const int *nc_dev, const int *head, const int *mid, int *mstart, DevCounters *dc) {
    int nc = *nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (head[c]) mstart[mid[c]] = c;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) mstart[dc->nmanifolds] = nc;
}

// Constraint groups: the contact manifolds, then one group per ball/hinge
// joint; each with the body pair the colouring separates.
__global__ void k_groups(const Contact *C, const int *mstart, const int4 *jinfo, int nj, DevCounters *dc,
                         int2 *gbody) {
    const int ncm = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ncm + nj; e += gridDim.x * blockDim.x) {
        if (e < ncm) {
            const Contact k = C[mstart[e]];
            gbody[e] = make_int2(k.b1 >= 0 ? k.b1 : k.b2, k.b1 >= 0 ? k.b2 : -1);
        } else {
            const int4 in = jinfo[e - ncm];
            gbody[e] = make_int2(in.y, in.z);
        }
    }
}
__global__ void k_groups_total(DevCounters *dc, int nj) {
    dc->ncmanifolds = dc->nmanifolds;
    dc->nmanifolds += nj;
}

#define GB_MAX_COLOURS 128
// Speculative first-fit colouring (rounds of: pick the lowest colour free at
// both bodies; per (body, colour) the lowest manifold index wins; losers
// retry).  One cooperative launch; every barrier is bounded.
// With `cls` (two-level sweep) the groups form two classes coloured
// independently: cross groups (cls < 0) take colours 0-63, a part's interior
// groups (cls >= 0) 64-127; dc->ncolours counts the first, dc->nicolours the
// second.  Interior groups of different parts share no body, so one colouring
// serves every part.
__global__ void k_colour(const int2 *gbody, DevCounters *dc, unsigned long long *mask, int *claim, int *colour,
                         int *tent, int nb, const int *cls, int climit) {
    unsigned gen = 0;
    const int nm = dc->nmanifolds;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int e = tid; e < nm; e += nth) colour[e] = -1;
    for (int round = 0; round < 4 * GB_MAX_COLOURS; round++) {
        if (!grid_sync(&dc->gsync, &dc->err, gen)) return;
        if (tid == 0) dc->uncoloured = 0;
        // phase A: tentative colour + claim
        for (int e = tid; e < nm; e += nth) {
            if (colour[e] >= 0) continue;
            const int2 gb = gbody[e];
            const int n0 = gb.x, n1 = gb.y;
            unsigned long long m0 = __ldcg(&mask[2 * n0]), m0b = __ldcg(&mask[2 * n0 + 1]);
            unsigned long long m1 = 0, m1b = 0;
            if (n1 >= 0) { m1 = __ldcg(&mask[2 * n1]); m1b = __ldcg(&mask[2 * n1 + 1]); }
            unsigned long long lo = m0 | m1, hi = m0b | m1b;
            int c;
            // climit: the colours a class may use (GB_MAX_COLOURS, or 64 a
            // class; lower only in the error-path tests).  Past it the last
            // colour is reused and ERR_COLOUR_OVERFLOW reported.
            if (cls) {
                const bool in = cls[e] >= 0;
                const unsigned long long used = in ? hi : lo;
                const int lim = climit < 64 ? climit : 64;
                int k = ~used ? __ffsll(~used) - 1 : 64;
                if (k >= lim) { atomicOr(&dc->err, ERR_COLOUR_OVERFLOW); k = lim - 1; }
                c = (in ? 64 : 0) + k;
            } else {
                int k = ~lo ? __ffsll(~lo) - 1 : (~hi ? 64 + __ffsll(~hi) - 1 : GB_MAX_COLOURS);
                if (k >= climit) { atomicOr(&dc->err, ERR_COLOUR_OVERFLOW); k = climit - 1; }
                c = k;
            }
            tent[e] = c;
            atomicMin(&claim[n0 * GB_MAX_COLOURS + c], e);
            if (n1 >= 0) atomicMin(&claim[n1 * GB_MAX_COLOURS + c], e);
        }
        if (!grid_sync(&dc->gsync, &dc->err, gen)) return;
        // phase B: winners commit
        for (int e = tid; e < nm; e += nth) {
            if (colour[e] >= 0) continue;
            const int2 gb = gbody[e];
            const int n0 = gb.x, n1 = gb.y;
            int c = tent[e];
            bool win = __ldcg(&claim[n0 * GB_MAX_COLOURS + c]) == e &&
                       (n1 < 0 || __ldcg(&claim[n1 * GB_MAX_COLOURS + c]) == e);
            if (win) {
                colour[e] = c;
                unsigned long long bit = 1ull << (c & 63);
                atomicOr(&mask[2 * n0 + (c >> 6)], bit);
                if (n1 >= 0) atomicOr(&mask[2 * n1 + (c >> 6)], bit);
                if (cls && c >= 64) atomicMax(&dc->nicolours, c - 63);
                else atomicMax(&dc->ncolours, c + 1);
            }
        }
        if (!grid_sync(&dc->gsync, &dc->err, gen)) return;
        // phase C: losers release claims they still hold
        for (int e = tid; e < nm; e += nth) {
            if (colour[e] >= 0) continue;
            const int2 gb = gbody[e];
            const int n0 = gb.x, n1 = gb.y;
            int c = tent[e];
            atomicCAS(&claim[n0 * GB_MAX_COLOURS + c], e, 0x7fffffff);
            if (n1 >= 0) atomicCAS(&claim[n1 * GB_MAX_COLOURS + c], e, 0x7fffffff);
            atomicAdd(&dc->uncoloured, 1);
        }
        if (!grid_sync(&dc->gsync, &dc->err, gen)) return;
        if (__ldcg(&dc->uncoloured) == 0) break;
        if (round == 4 * GB_MAX_COLOURS - 1 && tid == 0) atomicOr(&dc->err, ERR_COLOUR_OVERFLOW);
    }
}

// Colour lists: counts per colour, then every group placed in its colour's
// list.  Each block first counts its chunk of groups in shared memory and
// then touches each colour's global counter once (thousands of groups share a
// colour: one global atomic each would serialise on a few addresses).  The
// order inside a colour is free (its groups share no body).
__global__ void k_colour_count(const int *colour, DevCounters *dc, int *ccount) {
    __shared__ int h[GB_MAX_COLOURS];
    const int nm = dc->nmanifolds;
    for (int base = blockIdx.x * blockDim.x; base < nm; base += gridDim.x * blockDim.x) {
        for (int c = threadIdx.x; c < GB_MAX_COLOURS; c += blockDim.x) h[c] = 0;
        __syncthreads();
        const int e = base + threadIdx.x;
        const int c = e < nm ? colour[e] : -1;
        if (c >= 0) atomicAdd(&h[c], 1);
        __syncthreads();
        for (int k = threadIdx.x; k < GB_MAX_COLOURS; k += blockDim.x)
            if (h[k]) atomicAdd(&ccount[k], h[k]);
        __syncthreads();
    }
}
__global__ void k_colour_fill(const int *colour, DevCounters *dc, const int *cstart, int *cfill, int *list) {
    __shared__ int h[GB_MAX_COLOURS], at[GB_MAX_COLOURS];
    const int nm = dc->nmanifolds;
    for (int base = blockIdx.x * blockDim.x; base < nm; base += gridDim.x * blockDim.x) {
        for (int c = threadIdx.x; c < GB_MAX_COLOURS; c += blockDim.x) h[c] = 0;
        __syncthreads();
        const int e = base + threadIdx.x;
        const int c = e < nm ? colour[e] : -1;
        const int rank = c >= 0 ? atomicAdd(&h[c], 1) : 0;
        __syncthreads();
        for (int k = threadIdx.x; k < GB_MAX_COLOURS; k += blockDim.x)
            if (h[k]) at[k] = cstart[k] + atomicAdd(&cfill[k], h[k]);
        __syncthreads();
        if (c >= 0) list[at[c] + rank] = e;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ PGS row update
// quickstep.cpp:2917-3033 Stage4LCP_IterationStep for one row, with the body
// accumulators held by the caller.
__device__ __forceinline__ void relax_row(const Rows &Rw, int r, float4 &f1l, float4 &f1a, float4 &f2l, float4 &f2a,
                                          bool two) {
    const float4 j1l = Rw.J1l[r], j1a = Rw.J1a[r], j2l = Rw.J2l[r], j2a = Rw.J2a[r];
    const float old = Rw.lambda[r];
    float delta = j1l.w - old * j1a.w;
    delta -= f1l.x * j1l.x + f1l.y * j1l.y + f1l.z * j1l.z + f1a.x * j1a.x + f1a.y * j1a.y + f1a.z * j1a.z;
    if (two) delta -= f2l.x * j2l.x + f2l.y * j2l.y + f2l.z * j2l.z + f2a.x * j2a.x + f2a.y * j2a.y + f2a.z * j2a.z;
    float lo, hi;
    const int fi = Rw.findex[r];
    if (fi >= 0) { hi = fabsf(j2a.w * Rw.lambda[fi]); lo = -hi; }
    else { hi = j2a.w; lo = j2l.w; }
    float nl = old + delta;
    if (nl < lo) { delta = lo - old; nl = lo; }
    else if (nl > hi) { delta = hi - old; nl = hi; }
    Rw.lambda[r] = nl;
    if (delta != 0) {
        const float4 m1l = Rw.M1l[r], m1a = Rw.M1a[r];
        f1l.x += delta * m1l.x; f1l.y += delta * m1l.y; f1l.z += delta * m1l.z;
        f1a.x += delta * m1a.x; f1a.y += delta * m1a.y; f1a.z += delta * m1a.z;
        if (two) {
            const float4 m2l = Rw.M2l[r], m2a = Rw.M2a[r];
            f2l.x += delta * m2l.x; f2l.y += delta * m2l.y; f2l.z += delta * m2l.z;
            f2a.x += delta * m2a.x; f2a.y += delta * m2a.y; f2a.z += delta * m2a.z;
        }
    }
}

// natural-map residual of one row at the current fc (no update)
__device__ __forceinline__ float row_residual(const Rows &Rw, const float4 *fc, int r, float w_sor) {
    const float4 j1l = Rw.J1l[r], j1a = Rw.J1a[r], j2l = Rw.J2l[r], j2a = Rw.J2a[r];
    const int2 b = Rw.body[r];
    const float lam = __ldcg(&Rw.lambda[r]);
    const float4 f1l = ldcg4(&fc[2 * b.x]), f1a = ldcg4(&fc[2 * b.x + 1]);
    float delta = j1l.w - lam * j1a.w;
    delta -= f1l.x * j1l.x + f1l.y * j1l.y + f1l.z * j1l.z + f1a.x * j1a.x + f1a.y * j1a.y + f1a.z * j1a.z;
    if (b.y >= 0) {
        const float4 f2l = ldcg4(&fc[2 * b.y]), f2a = ldcg4(&fc[2 * b.y + 1]);
        delta -= f2l.x * j2l.x + f2l.y * j2l.y + f2l.z * j2l.z + f2a.x * j2a.x + f2a.y * j2a.y + f2a.z * j2a.z;
    }
    float lo, hi;
    const int fi = Rw.findex[r];
    if (fi >= 0) { hi = fabsf(j2a.w * __ldcg(&Rw.lambda[fi])); lo = -hi; }
    else { hi = j2a.w; lo = j2l.w; }
    float t = lam + delta / w_sor;
    t = fminf(fmaxf(t, lo), hi);
    return fabsf(lam - t);
}

struct PgsArgs {
    Rows Rw;
    float4 *fc;
    const int4 *desc;            // per colour slot: first row, row count, body 1, body 2 (-1: static)
    const int *cstart, *ccount;  // colour ranges of desc
    DevCounters *dc;
    int iterations, max_iterations, check_every;
    float target, w_sor;
    int warm;          // lambda starts non-zero: fc = M^-1 J^T lambda is formed first
    int nb;            // bodies
    int reform_every;  // sweeps between re-formations of fc from lambda (residual-target mode)
    int predict_checks;  // residual checks at half the predicted distance to the target (CheckPlan)
    const float4 *packed;                     // staged rows, chunk by chunk
    const int *chunk_start, *chunk_rows;      // per wave: first row in `packed`, rows
    const int *wcount, *wbase;                // per (colour, block): waves, index of the first
    const int *sched;                         // per wave and thread: the colour slot, or -1
    int learned;      // lambda holds the learned start, lam_alt the plain one: keep the better
    float *lam_alt;
    int passes;       // passes over a manifold's rows each time it is relaxed (>= 1)
    int poison_stage; // error-path tests: the staging waits name a copy that is never issued
    int chunk_cap;    // staged rows per shared-memory buffer (the waves were cut to it)
    float momentum;   // momentum between sweeps (used when lprev is set)
    float *lprev;     // [rows]: every multiplier as the previous sweep left it (null: no momentum)
    float4 *fcprev;   // [2 * bodies]: every body's accumulators as the previous sweep left them
};

// Manifold descriptors in colour-slot order: the solver reads one int4 per
// manifold instead of walking colour list -> manifold -> contact -> row ->
// bodies, four dependent memory round trips on every visit.
//   x: first row, y: row count | GB_DESC_TRIPLETS, z: body 1, w: body 2 (-1: static)
// GB_DESC_TRIPLETS marks the common shape of a contact manifold under
// dContactApprox1 with mu > 0 (contact.cpp:49-122): 1..4 contacts of three
// consecutive rows, the two friction rows' findex naming the normal row.
#define GB_DESC_TRIPLETS (1 << 30)
// GB_DESC_PLAIN marks a group of at most 12 rows none of which has a findex
// (ball and hinge joints, frictionless contacts): relaxed in row order.
#define GB_DESC_PLAIN (1 << 29)
#define GB_DESC_STAGED (GB_DESC_TRIPLETS | GB_DESC_PLAIN)
__device__ __forceinline__ int desc_rows(int4 d) { return d.y & 0xffff; }

// The descriptor of constraint group e (a contact manifold, or a ball/hinge
// joint whose rows follow the contact rows).
__device__ __forceinline__ int4 group_desc(int e, const int *mstart, const int *rstart, const int *mcount,
                                           const int2 *rbody, const int *findex, const DevCounters *dc,
                                           const int *jrstart, const int *jm, const int2 *gbody) {
    const int ncm = dc->ncmanifolds;
    if (e >= ncm) {
        const int k = e - ncm;
        const int2 b = gbody[e];
        return make_int4(dc->nrows_contacts + jrstart[k], jm[k] | GB_DESC_PLAIN, b.x, b.y);
    }
    const int c0 = mstart[e], c1 = mstart[e + 1];
    const int r0 = rstart[c0];
    const int r1 = rstart[c1 - 1] + mcount[c1 - 1];
    const int2 b = rbody[r0];
    bool tri = c1 - c0 <= 4;
    for (int c = c0; c < c1 && tri; c++) {
        const int r = r0 + 3 * (c - c0);
        tri = mcount[c] == 3 && rstart[c] == r && findex[r] < 0 && findex[r + 1] == r && findex[r + 2] == r;
    }
    bool plain = !tri && r1 - r0 <= 12;
    for (int r = r0; r < r1 && plain; r++) plain = findex[r] < 0;
    return make_int4(r0, (r1 - r0) | (tri ? GB_DESC_TRIPLETS : 0) | (plain ? GB_DESC_PLAIN : 0), b.x, b.y);
}

__global__ void k_manifold_desc(const int *clist, const int *mstart, const int *rstart, const int *mcount,
                                const int2 *rbody, const int *findex, DevCounters *dc, int4 *desc,
                                const int *jrstart, const int *jm, const int2 *gbody) {
    const int total = dc->colour_total;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x)
        desc[j] = group_desc(clist[j], mstart, rstart, mcount, rbody, findex, dc, jrstart, jm, gbody);
}

// the same descriptors indexed by group (the two-level sweep classifies groups before colouring)
__global__ void k_group_desc(const int *mstart, const int *rstart, const int *mcount, const int2 *rbody,
                             const int *findex, DevCounters *dc, int4 *gdesc, const int *jrstart, const int *jm,
                             const int2 *gbody) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x)
        gdesc[e] = group_desc(e, mstart, rstart, mcount, rbody, findex, dc, jrstart, jm, gbody);
}

// Prefetch a manifold's rows into L1.  The row arrays are read-only while the
// solver runs and a manifold's rows are contiguous, so the relaxation, issued
// after the next grid barrier, finds them in L1 instead of paying L2 round
// trips inside its row-to-row dependency chain.
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_span(const void *b, const void *e) {
    for (const char *q = (const char *)((uintptr_t)b & ~(uintptr_t)127); q < (const char *)e; q += 128) prefetch_l1(q);
}
__device__ __forceinline__ void prefetch_rows(const Rows &Rw, int r0, int r1) {
    const float4 *arr[8] = {Rw.J1l, Rw.J1a, Rw.J2l, Rw.J2a, Rw.M1l, Rw.M1a, Rw.M2l, Rw.M2a};
#pragma unroll
    for (int a = 0; a < 8; a++) prefetch_span(arr[a] + r0, arr[a] + r1);
    prefetch_span(Rw.findex + r0, Rw.findex + r1);
    prefetch_span(Rw.lambda + r0, Rw.lambda + r1);
}

// fc += M^-1 J^T lambda for one manifold's rows (warm start, re-formation)
__device__ __forceinline__ void apply_desc(const PgsArgs &A, int4 d) {
    const bool two = d.w >= 0;
    float4 f1l = ldcg4(&A.fc[2 * d.z]), f1a = ldcg4(&A.fc[2 * d.z + 1]);
    float4 f2l = make_float4(0, 0, 0, 0), f2a = f2l;
    if (two) { f2l = ldcg4(&A.fc[2 * d.w]); f2a = ldcg4(&A.fc[2 * d.w + 1]); }
    for (int r = d.x; r < d.x + desc_rows(d); r++) {
        const float l = __ldcg(&A.Rw.lambda[r]);
        if (l == 0.f) continue;
        const float4 m1l = __ldg(&A.Rw.M1l[r]), m1a = __ldg(&A.Rw.M1a[r]);
        f1l.x += l * m1l.x; f1l.y += l * m1l.y; f1l.z += l * m1l.z;
        f1a.x += l * m1a.x; f1a.y += l * m1a.y; f1a.z += l * m1a.z;
        if (two) {
            const float4 m2l = __ldg(&A.Rw.M2l[r]), m2a = __ldg(&A.Rw.M2a[r]);
            f2l.x += l * m2l.x; f2l.y += l * m2l.y; f2l.z += l * m2l.z;
            f2a.x += l * m2a.x; f2a.y += l * m2a.y; f2a.z += l * m2a.z;
        }
    }
    stcg4(&A.fc[2 * d.z], f1l); stcg4(&A.fc[2 * d.z + 1], f1a);
    if (two) { stcg4(&A.fc[2 * d.w], f2l); stcg4(&A.fc[2 * d.w + 1], f2a); }
}

__device__ __forceinline__ float atomic_max_pos(float *addr, float v) {
    return __int_as_float(atomicMax((int *)addr, __float_as_int(v)));
}

// Rows of one manifold whose multipliers stay in thread-local storage while
// the manifold is relaxed: the rows' own previous values and the normal-row
// multipliers the friction bounds read are then register / L1 hits instead of
// round trips inside the row-to-row dependency chain.
#define GB_MANIFOLD_ROWS 24

// quickstep.cpp:2917-3033 for one row, multipliers from the local copy, the
// read-only row arrays through the non-coherent cache
__device__ __forceinline__ void relax_row_local(const Rows &Rw, int r, float &lam_r, float lam_f, bool has_f,
                                                float4 &f1l, float4 &f1a, float4 &f2l, float4 &f2a, bool two) {
    const float4 j1l = __ldg(&Rw.J1l[r]), j1a = __ldg(&Rw.J1a[r]), j2l = __ldg(&Rw.J2l[r]), j2a = __ldg(&Rw.J2a[r]);
    const float old = lam_r;
    float delta = j1l.w - old * j1a.w;
    delta -= f1l.x * j1l.x + f1l.y * j1l.y + f1l.z * j1l.z + f1a.x * j1a.x + f1a.y * j1a.y + f1a.z * j1a.z;
    if (two) delta -= f2l.x * j2l.x + f2l.y * j2l.y + f2l.z * j2l.z + f2a.x * j2a.x + f2a.y * j2a.y + f2a.z * j2a.z;
    float lo, hi;
    if (has_f) { hi = fabsf(j2a.w * lam_f); lo = -hi; }
    else { hi = j2a.w; lo = j2l.w; }
    float nl = old + delta;
    if (nl < lo) { delta = lo - old; nl = lo; }
    else if (nl > hi) { delta = hi - old; nl = hi; }
    lam_r = nl;
    if (delta != 0) {
        const float4 m1l = __ldg(&Rw.M1l[r]), m1a = __ldg(&Rw.M1a[r]);
        f1l.x += delta * m1l.x; f1l.y += delta * m1l.y; f1l.z += delta * m1l.z;
        f1a.x += delta * m1a.x; f1a.y += delta * m1a.y; f1a.z += delta * m1a.z;
        if (two) {
            const float4 m2l = __ldg(&Rw.M2l[r]), m2a = __ldg(&Rw.M2a[r]);
            f2l.x += delta * m2l.x; f2l.y += delta * m2l.y; f2l.z += delta * m2l.z;
            f2a.x += delta * m2a.x; f2a.y += delta * m2a.y; f2a.z += delta * m2a.z;
        }
    }
}

// Momentum between sweeps (PgsArgs::momentum = beta, lprev set): after sweep k
// every multiplier moves on from that sweep's projected Gauss-Seidel result
// y_k to y_k + beta (y_k - y_{k-1}) before sweep k + 1 starts from it, and every
// body's accumulators fc = M^-1 J^T lambda by the same rule, which keeps fc and
// the multipliers consistent (the map is linear).  This is the extrapolation
// step of Nesterov's accelerated gradient method with a fixed coefficient
// (Y. Nesterov, "A method for solving the convex programming problem with
// convergence rate O(1/k^2)", 1983), applied to the iterates of the projected
// Gauss-Seidel sweep, as nonsmooth nonlinear conjugate gradient methods apply
// their direction to them (M. Silcowitz, S. Niebe, K. Erleben, "A nonsmooth
// nonlinear conjugate gradient method for interactive contact force
// problems", The Visual Computer 26, 2010).  The limit is the same LCP
// solution: a fixed point of the sweep is one of the extrapolation.  A sweep
// that ends in a residual check, the first and the last sweep use beta = 0,
// so every check and the final multipliers are plain Gauss-Seidel results; a
// check whose residual rose halves beta for the rest of the solve, and below
// an eighth of the value set the sweeps go on without momentum (letting beta
// grow back after a falling check let cyclic states recur).  A row's
// multiplier is moved on by the thread that relaxed it, when it stores the
// result; a body's accumulators at the end of the sweep.
__device__ __forceinline__ float mom_halved(float mom, float set) { return 0.5f * mom < 0.125f * set ? 0.f : 0.5f * mom; }
__device__ __forceinline__ void store_lambda(const PgsArgs &A, int r, float out, float beta) {
    if (A.lprev) {
        float v = out;
        if (beta > 0.f) v = fmaf(beta, out - __ldcg(&A.lprev[r]), out);
        __stcg(&A.lprev[r], out);
        A.Rw.lambda[r] = v;
    } else {
        A.Rw.lambda[r] = out;
    }
}
// body b's accumulators (l, a) as the sweep left them: kept in fcprev, and
// moved on by beta times their change over the sweep
__device__ __forceinline__ void body_momentum(const PgsArgs &A, int b, float4 &l, float4 &a, float beta) {
    if (beta > 0.f) {
        const float4 pl = ldcg4(&A.fcprev[2 * b]), pa = ldcg4(&A.fcprev[2 * b + 1]);
        stcg4(&A.fcprev[2 * b], l);
        stcg4(&A.fcprev[2 * b + 1], a);
        l = make_float4(fmaf(beta, l.x - pl.x, l.x), fmaf(beta, l.y - pl.y, l.y), fmaf(beta, l.z - pl.z, l.z), l.w);
        a = make_float4(fmaf(beta, a.x - pa.x, a.x), fmaf(beta, a.y - pa.y, a.y), fmaf(beta, a.z - pa.z, a.z), a.w);
    } else {
        stcg4(&A.fcprev[2 * b], l);
        stcg4(&A.fcprev[2 * b + 1], a);
    }
}

// One manifold by one thread: the normal (findex < 0) rows of all its
// contacts first, then the friction rows, mirroring the reference's findex
// partition (quickstep.cpp:2329-2355).  lambda of a manifold is read and
// written only by the thread that owns the manifold's slot.
__device__ __forceinline__ void relax_desc(const PgsArgs &A, int4 d, float beta = 0.f) {
    const int r0 = d.x, n = desc_rows(d), r1 = d.x + n;
    const bool two = d.w >= 0;
    float4 f1l = ldcg4(&A.fc[2 * d.z]), f1a = ldcg4(&A.fc[2 * d.z + 1]);
    float4 f2l = make_float4(0, 0, 0, 0), f2a = f2l;
    if (two) { f2l = ldcg4(&A.fc[2 * d.w]); f2a = ldcg4(&A.fc[2 * d.w + 1]); }
    if (n <= GB_MANIFOLD_ROWS) {
        float lam[GB_MANIFOLD_ROWS];
        int fi[GB_MANIFOLD_ROWS];
        for (int k = 0; k < n; k++) {
            lam[k] = A.Rw.lambda[r0 + k];
            const int f = __ldg(&A.Rw.findex[r0 + k]);
            fi[k] = (f >= r0 && f < r1) ? f - r0 : (f >= 0 ? GB_MANIFOLD_ROWS + f : -1);
        }
        for (int pass = 0; pass < A.passes; pass++) {
            for (int k = 0; k < n; k++)
                if (fi[k] < 0) relax_row_local(A.Rw, r0 + k, lam[k], 0.f, false, f1l, f1a, f2l, f2a, two);
            for (int k = 0; k < n; k++) {
                if (fi[k] < 0) continue;
                // findex always names a row of the same contact, hence of this
                // manifold; a row elsewhere is read from memory
                const float lf = fi[k] < GB_MANIFOLD_ROWS ? lam[fi[k]] : __ldcg(&A.Rw.lambda[fi[k] - GB_MANIFOLD_ROWS]);
                relax_row_local(A.Rw, r0 + k, lam[k], lf, true, f1l, f1a, f2l, f2a, two);
            }
        }
        for (int k = 0; k < n; k++) store_lambda(A, r0 + k, lam[k], beta);
    } else {
        for (int r = r0; r < r1; r++)
            if (A.Rw.findex[r] < 0) relax_row(A.Rw, r, f1l, f1a, f2l, f2a, two);
        for (int r = r0; r < r1; r++)
            if (A.Rw.findex[r] >= 0) relax_row(A.Rw, r, f1l, f1a, f2l, f2a, two);
        if (A.lprev)
            for (int r = r0; r < r1; r++) store_lambda(A, r, A.Rw.lambda[r], beta);
    }
    stcg4(&A.fc[2 * d.z], f1l); stcg4(&A.fc[2 * d.z + 1], f1a);
    if (two) { stcg4(&A.fc[2 * d.w], f2l); stcg4(&A.fc[2 * d.w + 1], f2a); }
}

// Packed staging of the staged slots (triplet manifolds and plain groups).
//
// The slots of colour c that belong to block b are k = b, b + B, b + 2B, ...
// (B blocks; colour slots interleave over the blocks, so every colour spreads
// over all SMs).  They are cut, in that order, into waves of at most T slots
// (T threads a block) and GB_CHUNK_ROWS staged rows; thread t of the block
// relaxes slot t of each wave, and the same thread relaxes the same manifold in
// every sweep.  A colour that fits (the usual case for a single large world)
// is one wave: slot k = b + t B for thread t.  Before the solve the rows of
// every wave's staged slots are packed into one contiguous chunk, 128 B per
// row, the 8 float4 of a row XOR-swizzled by the row's index in the chunk so
// that the LDS.128 of threads reading different rows spread over the banks.
// During the sweeps one thread per block copies the next wave's chunk into
// the other of two shared-memory buffers with a single bulk asynchronous copy
// (TMA) completing on that buffer's mbarrier, so a wave's rows are on chip
// when it starts.  Waves of one colour are separated by a block barrier only;
// colours by a grid barrier.  A slot's offset in its chunk lives in bits 16-27
// of its descriptor's y.
#define GB_PGS_THREADS 256  // threads a block of the sweep kernels by default (128 is the other instance)
#define GB_STAGED_ROWS 12  // rows of a staged slot at most (4 contacts x 3, or a plain group)

// a staged slot's relaxed multipliers out to global memory; with momentum
// `prev` holds the slot's previous-sweep results (staged beside the
// multipliers by the one-level sweep, loaded before the relaxation by the
// two-level sweep)
__device__ __forceinline__ void store_staged(const PgsArgs &A, int x, const float (&lout)[GB_STAGED_ROWS], int n,
                                             float beta, const float (&prev)[GB_STAGED_ROWS]) {
    if (!A.lprev) {
#pragma unroll
        for (int k = 0; k < GB_STAGED_ROWS; k++)
            if (k < n) A.Rw.lambda[x + k] = lout[k];
        return;
    }
#pragma unroll
    for (int k = 0; k < GB_STAGED_ROWS; k++)
        if (k < n) {
            const float out = lout[k];
            A.Rw.lambda[x + k] = beta > 0.f ? fmaf(beta, out - prev[k], out) : out;
            __stcg(&A.lprev[x + k], out);
        }
}
#define GB_CHUNK_ROWS 800  // staged rows per buffer by default: 2 x 100 KB of shared memory (at most)
#define GB_CHUNK_ROWS_MOM 792  // at most, with momentum (room for 12 floats a thread beside the buffers)
__device__ __forceinline__ int desc_chunk_off(int4 d) { return (d.y >> 16) & 0xfff; }
__device__ __forceinline__ int swz(int row, int a) { return row * 8 + (a ^ (row & 7)); }

// The greedy cut of one (colour, block)'s slots into waves; `visit(wave, t,
// k, offset)` for every slot (offset -1: not staged), returns the wave count.
template <class F>
__device__ int cut_waves(const int4 *desc, int s0, int n, int b, int B, int chunk_cap, int T, F visit) {
    int waves = 0, t = T, rows = 0;
    for (int k = b; k < n; k += B) {
        const int4 d = desc[s0 + k];
        const int r = (d.y & GB_DESC_STAGED) ? desc_rows(d) : 0;
        if (t == T || rows + r > chunk_cap) { ++waves; t = 0; rows = 0; }
        visit(waves - 1, t, k, r > 0 ? rows : -1);
        rows += r;
        ++t;
    }
    return waves;
}

// The same greedy cut by one warp: the (colour, block)'s slots are taken 32
// at a time, lane j holding slot b + (i + j) B.  With the state (slots t0 and
// rows rows0 of the open wave) at the first unplaced lane p, a lane j >= p
// opens a new wave iff t0 + (j - p) == T or rows0 + (rows of lanes p..j) >
// chunk_cap -- the serial rule -- so the first such lane (a prefix sum and a
// ballot) ends the open wave; the loop repeats from it with the state (0, 0).
// `visit(wave, t, k, offset)` runs on each lane for its own slot; returns the
// wave count (every lane).
template <class F>
__device__ int warp_cut_waves(const int4 *desc, int s0, int n, int b, int B, int chunk_cap, int T, F visit) {
    const int lane = threadIdx.x & 31;
    int waves = 0, t0 = T, rows0 = 0;  // t0 = T: the first slot opens a wave
    for (int base = b; base < n; base += 32 * B) {
        const int k = base + lane * B;
        const bool have = k < n;
        int4 d = make_int4(0, 0, 0, 0);
        if (have) d = desc[s0 + k];
        const int r = have && (d.y & GB_DESC_STAGED) ? desc_rows(d) : 0;
        const int nl = min(32, (n - base + B - 1) / B);  // lanes holding a slot
        int p = 0;
        while (p < nl) {
            // inclusive prefix of the rows of lanes p..j
            int x = lane >= p ? r : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            const bool brk = lane >= p && lane < nl && (t0 + (lane - p) >= T || rows0 + x > chunk_cap);
            const unsigned m = __ballot_sync(0xffffffffu, brk);
            const int q = m ? __ffs(m) - 1 : nl;  // lanes p..q-1 join the open wave
            if (lane >= p && lane < q) visit(waves - 1, t0 + (lane - p), k, r > 0 ? rows0 + x - r : -1);
            const int xq = __shfl_sync(0xffffffffu, x, (q > 0 ? q : 1) - 1);  // rows of lanes p..q-1
            if (q < nl) {
                ++waves;  // lane q opens a new wave
                t0 = 0;
                rows0 = 0;
            } else {
                t0 += q - p;
                rows0 += q > p ? xq : 0;
            }
            p = q;
        }
    }
    return waves;
}

// The slots of (colour c, block b): every B-th from b, or (xstart given: the
// two-level sweep's cross colours listed owner block by owner block) the
// xcnt[c B + b] slots from list position xstart[c B + b].  Returns the first
// list position, the count and stride of the cut, and the offset from the
// colour's first slot.
struct SlotRange { int s0, n, b, B, koff; };
__device__ __forceinline__ SlotRange slot_range(const int *cstart, const int *ccount, const int *xstart,
                                                const int *xcnt, int c, int b, int B) {
    if (xstart && c < 64) {
        const int s0 = xstart[c * B + b];
        return SlotRange{s0, xcnt[c * B + b], 0, 1, s0 - cstart[c]};
    }
    return SlotRange{cstart[c], ccount[c], b, B, 0};
}

// pass 1, one warp per (colour, block): waves of each (at least one, so
// every block takes part in every colour's barrier)
__global__ void k_wave_count(const int *cstart, const int *ccount, const DevCounters *dc, const int4 *desc,
                             int *wcount, int B, int chunk_cap, int T, const int *xstart, const int *xcnt) {
    const int cb = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (cb >= GB_MAX_COLOURS * B) return;
    const int c = cb / B, b = cb % B;
    if (c >= dc->ncolours) {
        if ((threadIdx.x & 31) == 0) wcount[cb] = 0;
        return;
    }
    const SlotRange r = slot_range(cstart, ccount, xstart, xcnt, c, b, B);
    const int w = warp_cut_waves(desc, r.s0, r.n, r.b, r.B, chunk_cap, T, [](int, int, int, int) {});
    if ((threadIdx.x & 31) == 0) wcount[cb] = w > 0 ? w : 1;
}

// pass 2, one warp per (colour, block): the chunk offsets in the
// descriptors, the schedule, rows per wave
__global__ void k_wave_fill(const int *cstart, const int *ccount, DevCounters *dc, int4 *desc, const int *wcount,
                            const int *wbase, int *sched, int *wrows, int *wcol, int wave_cap, int B,
                            int chunk_cap, int T, const int *xstart, const int *xcnt) {
    const int cb = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (cb >= GB_MAX_COLOURS * B) return;
    const int c = cb / B, b = cb % B;
    if (c >= dc->ncolours) return;
    const int base = wbase[cb], nw = wcount[cb];
    if (base + nw > wave_cap) {
        if (lane == 0) atomicOr(&dc->err, ERR_ROW_OVERFLOW);
        return;
    }
    for (int w = lane; w < nw; w += 32) {
        wrows[base + w] = 0;
        wcol[base + w] = c;
    }
    for (int i = lane; i < nw * T; i += 32) sched[(size_t)base * T + i] = -1;
    __syncwarp();
    const SlotRange r = slot_range(cstart, ccount, xstart, xcnt, c, b, B);
    const int s0 = r.s0;
    warp_cut_waves(desc, s0, r.n, r.b, r.B, chunk_cap, T, [&](int w, int t, int k, int off) {
        sched[(size_t)(base + w) * T + t] = k + r.koff;
        if (off >= 0) {
            int4 d = desc[s0 + k];
            d.y = (d.y & ~(0xfff << 16)) | (off << 16);
            desc[s0 + k] = d;
            atomicMax(&wrows[base + w], off + desc_rows(d));
        }
    });
}
__global__ void k_wave_total(DevCounters *dc, const int *wcount, const int *wbase, int B) {
    const int last = GB_MAX_COLOURS * B - 1;
    dc->nwaves = wbase[last] + wcount[last];
}

// copy the rows of every staged slot into its wave's chunk (swizzled); one
// block per wave, one thread per slot.  With split classes (nsplit: groups of
// each class touching each body) a crossing group's rows are packed for mass
// splitting: a body shared by n groups of the class enters each with 1/n of
// its mass, so the row's scaled Jacobian, right-hand side and cfm (all
// carrying Ad = W / (J M^-1 J^T + cfm)) are rescaled to W / (n1 D1 + n2 D2 +
// cfm) -- D1, D2 the two bodies' shares of J M^-1 J^T -- and M^-1 J^T by n1
// and n2 (the group's local copies of the bodies move n times as far); n1 and
// n2 ride in the otherwise unused M1a.w and M2a.w, the bodies' masks of
// shared classes (k_split_mask) in M1l.w and M2l.w.
__global__ void k_pack_rows(Rows Rw, const int *cstart, const DevCounters *dc, const int4 *desc, const int *sched,
                            const int *wcol, const int *chunk_start, float4 *packed, const int *nsplit,
                            const int *smask, int nb) {
    const int nw = dc->nwaves;
    const bool split = nsplit && dc->split_k > 0;
    for (int wv = blockIdx.x; wv < nw; wv += gridDim.x) {
        const int k = sched[(size_t)wv * blockDim.x + threadIdx.x];
        if (k < 0) continue;
        const int c = wcol[wv];
        const int4 d = desc[cstart[c] + k];
        if (!(d.y & GB_DESC_STAGED)) continue;
        const int n = desc_rows(d), off = desc_chunk_off(d);
        float4 *dst = packed + (size_t)chunk_start[wv] * 8;
        const float4 *arr[8] = {Rw.J1l, Rw.J1a, Rw.J2l, Rw.J2a, Rw.M1l, Rw.M1a, Rw.M2l, Rw.M2a};
        float n1 = 1.f, n2 = 1.f;
        int m1 = 0, m2 = 0;
        if (split) {
            n1 = (float)max(1, nsplit[(size_t)c * nb + d.z]);
            m1 = smask[d.z];
            if (d.w >= 0) {
                n2 = (float)max(1, nsplit[(size_t)c * nb + d.w]);
                m2 = smask[d.w];
            }
        }
        for (int i = 0; i < n; i++) {
            float4 v[8];
#pragma unroll
            for (int a = 0; a < 8; a++) v[a] = arr[a][d.x + i];
            if (split) {
                const float ad = Rw.Ad[d.x + i];
                const float d1 = (v[0].x * v[4].x + v[0].y * v[4].y + v[0].z * v[4].z + v[1].x * v[5].x +
                                  v[1].y * v[5].y + v[1].z * v[5].z) / ad;
                const float d2 = d.w >= 0 ? (v[2].x * v[6].x + v[2].y * v[6].y + v[2].z * v[6].z + v[3].x * v[7].x +
                                             v[3].y * v[7].y + v[3].z * v[7].z) / ad
                                          : 0.f;
                const float cfm = v[1].w / ad;
                const float s = (d1 + d2 + cfm) / (n1 * d1 + n2 * d2 + cfm);
                v[0].x *= s; v[0].y *= s; v[0].z *= s; v[0].w *= s;
                v[1].x *= s; v[1].y *= s; v[1].z *= s; v[1].w *= s;
                v[2].x *= s; v[2].y *= s; v[2].z *= s;  // w: lo
                v[3].x *= s; v[3].y *= s; v[3].z *= s;  // w: hi
                v[4].x *= n1; v[4].y *= n1; v[4].z *= n1; v[4].w = __int_as_float(m1);
                v[5].x *= n1; v[5].y *= n1; v[5].z *= n1; v[5].w = n1;
                v[6].x *= n2; v[6].y *= n2; v[6].z *= n2; v[6].w = __int_as_float(m2);
                v[7].x *= n2; v[7].y *= n2; v[7].z *= n2; v[7].w = n2;
            }
#pragma unroll
            for (int a = 0; a < 8; a++) dst[swz(off + i, a)] = v[a];
        }
    }
}

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *m) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *m, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *m, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *m) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(m))
                 : "memory");
}
// bounded wait for a phase of an mbarrier (at most 2^limit_log2 tries)
__device__ __forceinline__ bool mbar_wait(unsigned long long *m, unsigned parity, unsigned *err, int limit_log2 = 22) {
    long long tries = 0;
    while (!mbar_try_wait(m, parity)) {
        if (++tries > (1ll << limit_log2)) {
            atomicOr(err, ERR_STAGE_TIMEOUT);
            return false;
        }
    }
    return true;
}

// The residual-check schedule of residual-target mode (the same on every
// block: it depends only on the checks' results).  Fixed: every `every`
// sweeps.  Predicted: the residual's tail decays about geometrically, so
// from the last two checks (sweeps s0 < s1, residuals r0 > r1) the target is
// n = ln(target / r1) / ln(r1 / r0) * (s1 - s0) sweeps away; the next check
// comes half that distance later (at least `every`, at most 64 sweeps): a
// rate misjudged either way costs a few checks or a few sweeps.  After a
// check whose residual did not fall, the next is `every` sweeps later.
struct CheckPlan {
    int next, s_prev;
    float r_prev;
    __device__ void init(int every) { next = every; s_prev = -1; r_prev = 0.f; }
    __device__ void after(int it, float r, float target, int every, bool predict) {
        int gap = every;
        if (predict && s_prev >= 0 && r < r_prev && r > target) {
            const float per = logf(r / r_prev) / (float)(it - s_prev);  // < 0
            const float n = logf(target / r) / per;                     // > 0
            gap = max(every, min(64, (int)(0.5f * n)));
        }
        s_prev = it;
        r_prev = r;
        next = it + gap;
    }
};

// Staged triplet manifold (GB_DESC_TRIPLETS): the rows' operations of
// quickstep.cpp:2917-3033 with a shorter dependency chain -- the 12-term
// products J.fc summed as a tree with fused multiply-adds, the clamp as
// min/max, and fc += delta * M^-1 J^T as independent fused multiply-adds.  The
// values differ from relax_desc's in rounding only; the order of the rows
// (all normal rows, then the friction pairs) is the same.
template <bool TWO>
__device__ __forceinline__ float dot_fc(const float4 *row, const float4 &f1l, const float4 &f1a, const float4 &f2l,
                                        const float4 &f2a) {
    const float4 j1l = row[0], j1a = row[1];
    float a = fmaf(f1l.x, j1l.x, f1l.y * j1l.y);
    float b = fmaf(f1l.z, j1l.z, f1a.x * j1a.x);
    float c = fmaf(f1a.y, j1a.y, f1a.z * j1a.z);
    if (TWO) {
        const float4 j2l = row[2], j2a = row[3];
        a = fmaf(f2l.x, j2l.x, a);
        b = fmaf(f2l.y, j2l.y, b);
        c = fmaf(f2l.z, j2l.z, c);
        a = fmaf(f2a.x, j2a.x, a);
        b = fmaf(f2a.y, j2a.y, b);
        c = fmaf(f2a.z, j2a.z, c);
    }
    return (a + b) + c;
}

template <bool TWO>
__device__ __forceinline__ void relax_fast_row(const float4 *row, float &lam, float lo, float hi, float4 &f1l,
                                               float4 &f1a, float4 &f2l, float4 &f2a) {
    const float rhs = row[0].w, cfm = row[1].w;
    const float old = lam;
    float delta = fmaf(-old, cfm, rhs) - dot_fc<TWO>(row, f1l, f1a, f2l, f2a);
    const float nl = old + delta;
    const float cl = fminf(fmaxf(nl, lo), hi);
    if (cl != nl) delta = cl - old;
    lam = cl;
    const float4 m1l = row[4], m1a = row[5];
    f1l.x = fmaf(delta, m1l.x, f1l.x); f1l.y = fmaf(delta, m1l.y, f1l.y); f1l.z = fmaf(delta, m1l.z, f1l.z);
    f1a.x = fmaf(delta, m1a.x, f1a.x); f1a.y = fmaf(delta, m1a.y, f1a.y); f1a.z = fmaf(delta, m1a.z, f1a.z);
    if (TWO) {
        const float4 m2l = row[6], m2a = row[7];
        f2l.x = fmaf(delta, m2l.x, f2l.x); f2l.y = fmaf(delta, m2l.y, f2l.y); f2l.z = fmaf(delta, m2l.z, f2l.z);
        f2a.x = fmaf(delta, m2a.x, f2a.x); f2a.y = fmaf(delta, m2a.y, f2a.y); f2a.z = fmaf(delta, m2a.z, f2a.z);
    }
}

__device__ __forceinline__ void cp_async4(void *smem, const void *g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// A staged triplet manifold: rows from the chunk buffer, multipliers from the
// thread's shared-memory slot.  One code path for one- and two-body
// manifolds (a static second body contributes fc = 0 and is not written
// back), loops kept rolled: the solver's inner code stays small enough for
// the instruction caches.
// The multipliers come back in lout (registers): the caller stores them after
// its barrier arrival, so those stores do not delay the release.
// The rows of a staged triplet manifold against the accumulators f1*, f2*.
__device__ __forceinline__ void triplet_rows(int passes, int nct, int off, const float4 *buf, float *lam,
                                             float4 &f1l, float4 &f1a, float4 &f2l, float4 &f2a) {
    float4 row[8];
#pragma unroll 1
    for (int pass = 0; pass < passes; pass++) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (c >= nct) break;
            const int r = off + 3 * c;
#pragma unroll
            for (int a = 0; a < 8; a++) row[a] = buf[swz(r, a)];
            relax_fast_row<true>(row, lam[3 * c], row[2].w, row[3].w, f1l, f1a, f2l, f2a);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (c >= nct) break;
            const float ln = lam[3 * c];
#pragma unroll
            for (int q = 1; q < 3; q++) {
                const int r = off + 3 * c + q;
#pragma unroll
                for (int a = 0; a < 8; a++) row[a] = buf[swz(r, a)];
                const float hi = fabsf(row[3].w * ln);
                relax_fast_row<true>(row, lam[3 * c + q], -hi, hi, f1l, f1a, f2l, f2a);
            }
        }
    }
}
__device__ __forceinline__ void relax_triplets(const PgsArgs &A, int4 d, const float4 *buf, float *lam,
                                               float (&lout)[GB_STAGED_ROWS]) {
    const int nct = desc_rows(d) / 3, off = desc_chunk_off(d);
    const bool two = d.w >= 0;
    float4 f1l = ldcg4(&A.fc[2 * d.z]), f1a = ldcg4(&A.fc[2 * d.z + 1]);
    float4 f2l = make_float4(0, 0, 0, 0), f2a = f2l;
    if (two) { f2l = ldcg4(&A.fc[2 * d.w]); f2a = ldcg4(&A.fc[2 * d.w + 1]); }
    cp_async_wait_all();
    triplet_rows(A.passes, nct, off, buf, lam, f1l, f1a, f2l, f2a);
#pragma unroll
    for (int k = 0; k < GB_STAGED_ROWS; k++) lout[k] = k < 3 * nct ? lam[k] : 0.f;
    stcg4(&A.fc[2 * d.z], f1l); stcg4(&A.fc[2 * d.z + 1], f1a);
    if (two) { stcg4(&A.fc[2 * d.w], f2l); stcg4(&A.fc[2 * d.w + 1], f2a); }
}

// A staged plain group (GB_DESC_PLAIN): every row in order with its own bounds.
__device__ __forceinline__ void plain_rows(int passes, int n, int off, const float4 *buf, float *lam,
                                           float4 &f1l, float4 &f1a, float4 &f2l, float4 &f2a) {
    float4 row[8];
#pragma unroll 1
    for (int pass = 0; pass < passes; pass++) {
#pragma unroll 1
        for (int k = 0; k < n; k++) {
#pragma unroll
            for (int a = 0; a < 8; a++) row[a] = buf[swz(off + k, a)];
            relax_fast_row<true>(row, lam[k], row[2].w, row[3].w, f1l, f1a, f2l, f2a);
        }
    }
}
__device__ __forceinline__ void relax_plain(const PgsArgs &A, int4 d, const float4 *buf, float *lam,
                                            float (&lout)[GB_STAGED_ROWS]) {
    const int n = desc_rows(d), off = desc_chunk_off(d);
    const bool two = d.w >= 0;
    float4 f1l = ldcg4(&A.fc[2 * d.z]), f1a = ldcg4(&A.fc[2 * d.z + 1]);
    float4 f2l = make_float4(0, 0, 0, 0), f2a = f2l;
    if (two) { f2l = ldcg4(&A.fc[2 * d.w]); f2a = ldcg4(&A.fc[2 * d.w + 1]); }
    cp_async_wait_all();
    plain_rows(A.passes, n, off, buf, lam, f1l, f1a, f2l, f2a);
#pragma unroll
    for (int k = 0; k < GB_STAGED_ROWS; k++) lout[k] = k < n ? lam[k] : 0.f;
    stcg4(&A.fc[2 * d.z], f1l); stcg4(&A.fc[2 * d.z + 1], f1a);
    if (two) { stcg4(&A.fc[2 * d.w], f2l); stcg4(&A.fc[2 * d.w + 1], f2a); }
}

// The coloured SOR sweeps, one persistent cooperative launch.
//
// Colour slots interleave over the blocks and are cut per block into waves
// (see the staging comment above), so a colour's manifolds spread over every
// SM and the same thread relaxes the same manifold in every sweep.  While a
// wave is relaxed the block's next chunk streams into the other shared-memory
// buffer, and each thread loads its next manifold's descriptor and
// multipliers while it waits at the barrier; after the barrier only the body
// accumulators fc (written by the previous colour) are read through L2.
template <int T>
__global__ void __launch_bounds__(T, 1) k_pgs(PgsArgs A) {
    unsigned gen = 0;
    DevCounters *dc = A.dc;
    __shared__ int s_cstart[GB_MAX_COLOURS], s_ccount[GB_MAX_COLOURS], s_wcount[GB_MAX_COLOURS], s_wbase[GB_MAX_COLOURS];
    __shared__ unsigned long long s_mbar[3];  // two chunk buffers; [2] is never armed (poison_stage)
    __shared__ int s_abort;                   // a staging wait of this block ran out
    __shared__ float s_lam[T * 13];  // per thread: the next manifold's multipliers
    extern __shared__ float4 pgs_smem[];  // two buffers of A.chunk_cap rows
    const int ncol = dc->ncolours;
    const int nrows = dc->nrows;
    for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
        s_cstart[c] = A.cstart[c];
        s_ccount[c] = A.ccount[c];
        s_wcount[c] = A.wcount[c * gridDim.x + blockIdx.x];
        s_wbase[c] = A.wbase[c * gridDim.x + blockIdx.x];
    }
    if (threadIdx.x == 0) {
        mbar_init(&s_mbar[0]);
        mbar_init(&s_mbar[1]);
        mbar_init(&s_mbar[2]);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const bool residual_mode = A.target > 0;
    const int itmax = residual_mode ? A.max_iterations : A.iterations;
    int it = 0, check = 0, last_reform = 0;
    CheckPlan plan;
    plan.init(A.check_every);
    float mom = A.lprev ? A.momentum : 0.f;  // momentum between sweeps (halved when a check's residual rises)
    float *slots = dc->racc;  // [2][2]: residual, max|lambda| per check parity
    // fc = M^-1 J^T lambda, colour by colour so no two manifolds of a pass touch one body
    auto form_fc = [&](bool zero) -> bool {
        if (zero) {
            for (int b = tid; b < A.nb; b += nth) {
                stcg4(&A.fc[2 * b], make_float4(0.f, 0.f, 0.f, 0.f));
                stcg4(&A.fc[2 * b + 1], make_float4(0.f, 0.f, 0.f, 0.f));
            }
            if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
        }
        for (int c = 0; c < ncol; c++) {
            for (int k = tid; k < s_ccount[c]; k += nth) apply_desc(A, __ldg(&A.desc[s_cstart[c] + k]));
            if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
        }
        return true;
    };
    // FP32 natural-map residual of every row at the current fc, relative to max(1, max|lambda|)
    auto residual_rel = [&](float &rel) -> bool {
        float *acc = slots + 2 * (check & 1);
        float rmax = 0.f, lmax = 0.f;
        for (int r = tid; r < nrows; r += nth) {
            rmax = fmaxf(rmax, row_residual(A.Rw, A.fc, r, A.w_sor));
            lmax = fmaxf(lmax, fabsf(__ldcg(&A.Rw.lambda[r])));
        }
        for (int o = 16; o > 0; o >>= 1) {
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
            lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        }
        if ((threadIdx.x & 31) == 0) { atomic_max_pos(&acc[0], rmax); atomic_max_pos(&acc[1], lmax); }
        if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
        const float rr = __ldcg(&acc[0]), ll = __ldcg(&acc[1]);
        rel = rr / fmaxf(1.0f, ll);
        if (tid == 0) {
            float *other = slots + 2 * ((check + 1) & 1);
            other[0] = 0.f; other[1] = 0.f;
            dc->resid = rel; dc->maxlam = ll;
            if (check < 256) { dc->rhist[check] = rel; dc->rsweep[check] = it; dc->nhist = check + 1; }
        }
        ++check;
        return true;
    };
    auto swap_alt = [&]() -> bool {
        for (int r = tid; r < nrows; r += nth) {
            const float a = __ldcg(&A.Rw.lambda[r]), b = __ldcg(&A.lam_alt[r]);
            __stcg(&A.Rw.lambda[r], b);
            __stcg(&A.lam_alt[r], a);
        }
        return grid_sync(&dc->gsync, &dc->err, gen);
    };
    if (A.learned) {
        // The learned start has to earn its place: its residual against the
        // plain (previous-step) start's; the better one starts the sweeps.
        float r_mlp = 0.f, r_plain = 0.f;
        if (!form_fc(true) || !residual_rel(r_mlp)) return;
        if (!swap_alt() || !form_fc(true) || !residual_rel(r_plain)) return;
        const bool use = r_mlp < r_plain;
        if (use && (!swap_alt() || !form_fc(true))) return;
        if (tid == 0) {
            dc->learn_stats[0] = use ? 1.f : 0.f;
            dc->learn_stats[1] = r_mlp;
            dc->learn_stats[2] = r_plain;
        }
    } else if (A.warm) {
        if (!form_fc(false)) return;
    }
    // The sweep is a sequence of steps (colour c, wave w): the waves of a
    // colour in order, then the next colour.  Buffer q & 1 holds step number q
    // (counted over all sweeps); its use number q >> 1 is the mbarrier phase to
    // wait for.
    struct Step { int c, w; };
    auto step_after = [&](Step t) -> Step {
        if (t.w + 1 < s_wcount[t.c]) return Step{t.c, t.w + 1};
        return Step{t.c + 1 < ncol ? t.c + 1 : 0, 0};
    };
    unsigned q = 0;
    unsigned nissued = 0, nwaited = 0;  // thread 0: chunk copies issued / waited for, in step order
    // thread 0: the chunk (first row, rows) of the step to issue next, loaded
    // one issue ahead so that no global load sits in front of a copy
    int pend_start = 0, pend_rows = 0;
    auto chunk_of = [&](Step t) {  // loads only: nothing uses them before the next issue
        const int wv = s_wbase[t.c] + t.w;
        pend_start = __ldg(&A.chunk_start[wv]);
        pend_rows = __ldg(&A.chunk_rows[wv]);
    };
    auto issue = [&](Step t) {  // thread 0: the copy for step number nissued (t); loads t's successor's chunk
        const unsigned qq = nissued++;
        unsigned long long *m = &s_mbar[qq & 1];
        const unsigned bytes = 128u * (unsigned)min(pend_rows, A.chunk_cap);
        // the block's reads of this buffer (two steps ago) come before the copy's writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(m, bytes);
        if (bytes) bulk_g2s(pgs_smem + (qq & 1) * (A.chunk_cap * 8), A.packed + (size_t)pend_start * 8, bytes, m);
        chunk_of(step_after(t));
    };
    auto retire = [&]() {  // thread 0: wait for the oldest copy not yet waited for
        const unsigned qq = nwaited++;
        return mbar_wait(&s_mbar[qq & 1], (qq >> 1) & 1, &dc->err);
    };
    auto drain = [&]() {  // no copy may still be writing shared memory when the block exits
        cp_async_wait_all();
        if (threadIdx.x == 0)
            while (nwaited < nissued) retire();
    };
    float *my_lam = s_lam + threadIdx.x * 13;
    // with momentum: the next slot's previous-sweep results, copied beside its
    // multipliers (after the two chunk buffers), so storing needs no load
    float *my_lp = A.lprev ? (float *)(pgs_smem + (size_t)2 * A.chunk_cap * 8) + threadIdx.x * GB_STAGED_ROWS : nullptr;
    // Two-deep descriptor pipeline: `ahead` (the slot of the step after the
    // next one) is loaded a step early, so the multiplier copies for `next`
    // can be issued at once, without waiting for a descriptor load.
    int4 next = make_int4(0, 0, -1, -1), ahead = next;
    bool has_next = false, staged = false, has_ahead = false;
    auto load_ahead = [&](Step t) {
        // a colour in one wave: slot b + t B for thread t (no schedule load)
        int k = blockIdx.x + threadIdx.x * (int)gridDim.x;
        if (s_wcount[t.c] == 1) k = k < s_ccount[t.c] ? k : -1;
        else k = __ldg(&A.sched[(size_t)(s_wbase[t.c] + t.w) * T + threadIdx.x]);
        has_ahead = k >= 0;
        if (has_ahead) ahead = __ldg(&A.desc[s_cstart[t.c] + k]);
    };
    auto fetch = [&](Step t_after) {
        has_next = has_ahead;
        next = ahead;
        staged = false;
        if (has_next) {
            const int n = desc_rows(next);
            staged = (next.y & GB_DESC_STAGED) && desc_chunk_off(next) + n <= A.chunk_cap;
            if (staged) {
                for (int k = 0; k < n; k++) cp_async4(&my_lam[k], &A.Rw.lambda[next.x + k]);
                if (my_lp)
                    for (int k = 0; k < n; k++) cp_async4(&my_lp[k], &A.lprev[next.x + k]);
                cp_async_commit();
            }
        }
        load_ahead(t_after);
    };
    if (ncol > 0) {
        const Step s0{0, 0};
        if (threadIdx.x == 0) {
            chunk_of(s0);
            issue(s0);
        }
        load_ahead(s0);
        fetch(step_after(s0));
    }
    for (; it < itmax && ncol > 0;) {
        Step cur{0, 0};
        // plain Gauss-Seidel results for the first sweep, the last and every checked one
        const bool check_this = residual_mode && (it + 1 >= plan.next || it + 1 == itmax);
        const float beta = (mom > 0.f && it > 0 && it + 1 < itmax && !check_this) ? mom : 0.f;
        for (;;) {
            const Step nxt = step_after(cur), nnx = step_after(nxt);
            const bool last_wave = cur.w + 1 == s_wcount[cur.c];
            // inside a colour the next wave's rows stream in while this one is
            // relaxed (its buffer was last read two steps ago, before a barrier);
            // after a colour's last wave they are issued once the block arrives
            if (threadIdx.x == 0 && !last_wave) issue(nxt);
            float lout[GB_STAGED_ROWS];
            int nout = 0, xout = 0;
            if (has_next) {
                if (!staged) {
                    relax_desc(A, next, beta);
                } else if (A.poison_stage ? mbar_wait(&s_mbar[2], 0, &dc->err, 16)
                                          : mbar_wait(&s_mbar[q & 1], (q >> 1) & 1, &dc->err)) {
                    const float4 *buf = pgs_smem + (q & 1) * (A.chunk_cap * 8);
                    if (next.y & GB_DESC_TRIPLETS) relax_triplets(A, next, buf, my_lam, lout);
                    else relax_plain(A, next, buf, my_lam, lout);
                    nout = desc_rows(next);
                    xout = next.x;
                } else {
                    s_abort = 1;  // the whole block leaves after the next block barrier
                }
            }
            float prev[GB_STAGED_ROWS];  // (a staged slot's copy arrived before its relaxation)
#pragma unroll
            for (int k = 0; k < GB_STAGED_ROWS; k++) prev[k] = (beta > 0.f && k < nout) ? my_lp[k] : 0.f;
            const bool sweep_end = last_wave && cur.c == ncol - 1;
            if (!last_wave) {
                // another wave of this colour follows: a block barrier (the
                // colour's slots share no body, so no other block waits on these)
                store_staged(A, xout, lout, nout, beta, prev);
                fetch(nnx);
                __syncthreads();
                if (s_abort) { drain(); return; }
            } else {
                // arrive (the accumulators fc are out), then store the staged
                // slot's multipliers -- read again only by this thread a sweep
                // later and by re-formations after a later barrier -- and
                // prefetch the next slot while the other blocks arrive.  Before a
                // residual check (which reads every multiplier right after this
                // barrier) they go out before the arrival.
                const bool check_next = check_this && sweep_end;
                if (check_next) store_staged(A, xout, lout, nout, beta, prev);
                unsigned target = 0;
                grid_arrive(&dc->gsync, gen, target);
                if (threadIdx.x == 0) issue(nxt);
                if (!check_next) store_staged(A, xout, lout, nout, beta, prev);
                fetch(nnx);
                if (!grid_wait(&dc->gsync, &dc->err, gen, target) || s_abort) { drain(); return; }
            }
            // the copy for this step has completed before its buffer's mbarrier
            // is armed again (threads with no staged slot never waited)
            if (threadIdx.x == 0) retire();
            ++q;
            if (sweep_end) break;
            cur = nxt;
        }
        ++it;
        if (check_this) {
            // Re-form fc = M^-1 J^T lambda from lambda every reform_every sweeps:
            // thousands of incremental FP32 updates let fc drift from the
            // multipliers it stands for, and relaxation against a drifted fc
            // stalls at a residual of ~1e-4..1e-3 on deep piles.  A check
            // that passes on accumulators not formed afresh is repeated on
            // re-formed ones: the residual that ends the solve is the
            // multipliers' own.
            bool fresh = false;
            if (it - last_reform >= A.reform_every || it == itmax) {
                last_reform = it;
                fresh = true;
                if (!form_fc(true)) { drain(); return; }
            }
            float rel;
            if (!residual_rel(rel)) { drain(); return; }
            if (rel <= A.target && !fresh) {
                last_reform = it;
                if (!form_fc(true) || !residual_rel(rel)) { drain(); return; }
            }
            if (rel <= A.target) break;
            if (mom > 0.f && plan.s_prev >= 0 && rel > plan.r_prev) mom = mom_halved(mom, A.momentum);
            plan.after(it, rel, A.target, A.check_every, A.predict_checks);
        }
        if (mom > 0.f && it < itmax) {
            // momentum: the bodies' accumulators after the sweep (the rows'
            // multipliers moved on when they were stored); the barrier keeps
            // the next sweep's updates out of what this pass reads
            // (four bodies a thread at a time, their loads issued together)
            for (int b0 = tid; b0 < A.nb; b0 += 4 * nth) {
                float4 l[4], a[4], pl[4], pa[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int b = b0 + j * nth;
                    if (b < A.nb) {
                        l[j] = ldcg4(&A.fc[2 * b]);
                        a[j] = ldcg4(&A.fc[2 * b + 1]);
                        if (beta > 0.f) {
                            pl[j] = ldcg4(&A.fcprev[2 * b]);
                            pa[j] = ldcg4(&A.fcprev[2 * b + 1]);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int b = b0 + j * nth;
                    if (b >= A.nb) continue;
                    stcg4(&A.fcprev[2 * b], l[j]);
                    stcg4(&A.fcprev[2 * b + 1], a[j]);
                    if (beta > 0.f) {
                        const float4 x = l[j], y = a[j];
                        stcg4(&A.fc[2 * b], make_float4(fmaf(beta, x.x - pl[j].x, x.x), fmaf(beta, x.y - pl[j].y, x.y),
                                                        fmaf(beta, x.z - pl[j].z, x.z), x.w));
                        stcg4(&A.fc[2 * b + 1], make_float4(fmaf(beta, y.x - pa[j].x, y.x),
                                                            fmaf(beta, y.y - pa[j].y, y.y),
                                                            fmaf(beta, y.z - pa[j].z, y.z), y.w));
                    }
                }
            }
            if (!grid_sync(&dc->gsync, &dc->err, gen)) { drain(); return; }
        }
    }
    drain();  // the copy issued for the colour after the last one relaxed
    if (tid == 0) {
        dc->iterations = it;
        dc->mom_final = mom;
    }
}

#include "pgs_slab.cuh"

// ------------------------------------------------------------------ reference-order islands
// One block per island, rows relaxed by thread 0 in the reference's order
// (island joint order, findex<0 rows first: quickstep.cpp:2329-2355), with
// the reference's dynamic iteration rule per island (quickstep.cpp:1823-1856,
// :3253-3285) when enabled.
struct IslandArgs {
    Rows Rw;
    float4 *fc;
    float *fa;  // [2*nb] force max adjustments (negative, positive)
    const int *order, *start, *bodies, *bstart;
    int iterations;
    unsigned max_extra;
    float premature, extra_delta;
    int dyn;
    DevCounters *dc;
};

__global__ void k_islands(IslandArgs A) {
    const int isl = blockIdx.x;
    if (threadIdx.x != 0) return;
    const int r0 = A.start[isl], r1 = A.start[isl + 1];
    const int b0 = A.bstart[isl], b1 = A.bstart[isl + 1];
    if (r1 == r0) return;
    for (int k = b0; k < b1; k++) { int bd = A.bodies[k]; A.fa[2 * bd] = 0.f; A.fa[2 * bd + 1] = 0.f; }
    float premature = A.premature;
    unsigned iteration = 0, extra = 0;
    for (;;) {
        for (int k = r0; k < r1; k++) {
            const int r = A.order[k];
            const int2 b = A.Rw.body[r];
            const bool two = b.y >= 0;
            float4 f1l = A.fc[2 * b.x], f1a = A.fc[2 * b.x + 1];
            float4 f2l = make_float4(0, 0, 0, 0), f2a = f2l;
            if (two) { f2l = A.fc[2 * b.y]; f2a = A.fc[2 * b.y + 1]; }
            const float old = A.Rw.lambda[r];
            const float4 j1l = A.Rw.J1l[r], j1a = A.Rw.J1a[r], j2l = A.Rw.J2l[r], j2a = A.Rw.J2a[r];
            float delta = j1l.w - old * j1a.w;
            delta -= f1l.x * j1l.x + f1l.y * j1l.y + f1l.z * j1l.z + f1a.x * j1a.x + f1a.y * j1a.y + f1a.z * j1a.z;
            if (two) delta -= f2l.x * j2l.x + f2l.y * j2l.y + f2l.z * j2l.z + f2a.x * j2a.x + f2a.y * j2a.y + f2a.z * j2a.z;
            float lo, hi;
            const int fi = A.Rw.findex[r];
            if (fi >= 0) { hi = fabsf(j2a.w * A.Rw.lambda[fi]); lo = -hi; }
            else { hi = j2a.w; lo = j2l.w; }
            float nl = old + delta;
            if (nl < lo) { delta = lo - old; nl = lo; }
            else if (nl > hi) { delta = hi - old; nl = hi; }
            A.Rw.lambda[r] = nl;
            if (delta != 0) {
                const float4 m1l = A.Rw.M1l[r], m1a = A.Rw.M1a[r];
                const int pos = delta > 0;
                f1l.x += delta * m1l.x; f1l.y += delta * m1l.y; f1l.z += delta * m1l.z;
                f1a.x += delta * m1a.x; f1a.y += delta * m1a.y; f1a.z += delta * m1a.z;
                A.fc[2 * b.x] = f1l; A.fc[2 * b.x + 1] = f1a;
                A.fa[2 * b.x + pos] += delta * m1l.w;
                if (two) {
                    const float4 m2l = A.Rw.M2l[r], m2a = A.Rw.M2a[r];
                    A.fa[2 * b.y + pos] += delta * m2l.w;
                    f2l.x += delta * m2l.x; f2l.y += delta * m2l.y; f2l.z += delta * m2l.z;
                    f2a.x += delta * m2a.x; f2a.y += delta * m2a.y; f2a.z += delta * m2a.z;
                    A.fc[2 * b.y] = f2l; A.fc[2 * b.y + 1] = f2a;
                }
            }
        }
        ++iteration;
        if (iteration - extra == (unsigned)A.iterations) {
            if (extra != 0 || A.max_extra == 0) break;
            extra = A.max_extra;
            premature = A.extra_delta;
        }
        if (A.dyn) {
            bool hit = false;
            if (premature == 0) {
                for (int k = b0; k < b1; k++) { int bd = A.bodies[k]; A.fa[2 * bd] = 0; A.fa[2 * bd + 1] = 0; }
                hit = true;
            } else {
                for (int k = b0; k < b1; k++) {
                    int bd = A.bodies[k];
                    if (!(A.fa[2 * bd + 1] < premature) || !(-A.fa[2 * bd] < premature)) {
                        for (int q = k; q < b1; q++) { int bq = A.bodies[q]; A.fa[2 * bq] = 0; A.fa[2 * bq + 1] = 0; }
                        hit = true;
                        break;
                    }
                    A.fa[2 * bd] = 0; A.fa[2 * bd + 1] = 0;
                }
            }
            if (!hit) break;
        }
        if (iteration > 100000u) break;
    }
    atomicMax(&A.dc->iterations, (int)iteration);
}

// ------------------------------------------------------------------ integration
// quickstep.cpp:3082-3182 (Stage4b velocity), :3299-3337 (Stage6a),
// :3409-3439 + util.cpp:583-692 (Stage6b, dxStepBody)
__global__ void k_integrate(Bodies B, SolverParams P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    if (B.asleep && B.asleep[i]) return;  // a sleeping component: not moved, accumulators kept
    const float h = P.dt;
    float4 lv = B.lvel[i], av = B.avel[i], ps = B.pos[i], q4 = B.q[i];
    const float4 fl = B.fc[2 * i], fa = B.fc[2 * i + 1], facc = B.facc[i], tacc4 = B.tacc[i];
    float lvel[3] = {lv.x, lv.y, lv.z}, avel[3] = {av.x, av.y, av.z};
    lvel[0] += h * fl.x; lvel[1] += h * fl.y; lvel[2] += h * fl.z;
    avel[0] += h * fa.x; avel[1] += h * fa.y; avel[2] += h * fa.z;
    const float ims = h * ps.w;
    float tacc[3];
    lvel[0] += ims * facc.x; tacc[0] = tacc4.x * h;
    lvel[1] += ims * facc.y; tacc[1] = tacc4.y * h;
    lvel[2] += ims * facc.z; tacc[2] = tacc4.z * h;
    float invIw[12], tmp[3];
    load_rows3(B.invIw + 3 * i, invIw);
    mul0_331(tmp, invIw, tacc);
    avel[0] = avel[0] + tmp[0]; avel[1] = avel[1] + tmp[1]; avel[2] = avel[2] + tmp[2];
    // dxStepBody (util.cpp:583-692; infinitesimal rotation, no finite-rotation mode)
    const float maxw = B.maxw[i];
    if (maxw < INFINITY) {  // the angular speed cap
        const float aspeed = avel[0] * avel[0] + avel[1] * avel[1] + avel[2] * avel[2];
        if (aspeed > maxw * maxw) {
            const float coef = maxw / sqrtf(aspeed);
            avel[0] *= coef; avel[1] *= coef; avel[2] *= coef;
        }
    }
    float pos[3] = {ps.x + h * lvel[0], ps.y + h * lvel[1], ps.z + h * lvel[2]};
    float q[4] = {q4.x, q4.y, q4.z, q4.w};
    const float *w = avel;
    float dq[4];
    dq[0] = 0.5f * (-w[0] * q[1] - w[1] * q[2] - w[2] * q[3]);
    dq[1] = 0.5f * (w[0] * q[0] + w[1] * q[3] - w[2] * q[2]);
    dq[2] = 0.5f * (-w[0] * q[3] + w[1] * q[0] + w[2] * q[1]);
    dq[3] = 0.5f * (w[0] * q[2] - w[1] * q[1] + w[2] * q[0]);
    for (int j = 0; j < 4; j++) q[j] += h * dq[j];
    float l = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (l > 0) { l = 1.0f / sqrtf(l); q[0] *= l; q[1] *= l; q[2] *= l; q[3] *= l; }
    else { q[0] = 1; q[1] = q[2] = q[3] = 0; }
    float R[12];
    float qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
    R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]);
    R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]);
    R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2;
    R[3] = R[7] = R[11] = 0;
    const float4 dm = B.damp[i];  // damping after the move (util.cpp:675-691)
    if (dm.x != 0.f) {
        const float s2 = lvel[0] * lvel[0] + lvel[1] * lvel[1] + lvel[2] * lvel[2];
        if (s2 > dm.z) { const float k = 1 - dm.x; lvel[0] *= k; lvel[1] *= k; lvel[2] *= k; }
    }
    if (dm.y != 0.f) {
        const float s2 = avel[0] * avel[0] + avel[1] * avel[1] + avel[2] * avel[2];
        if (s2 > dm.w) { const float k = 1 - dm.y; avel[0] *= k; avel[1] *= k; avel[2] *= k; }
    }
    B.pos[i] = make_float4(pos[0], pos[1], pos[2], ps.w);
    B.q[i] = make_float4(q[0], q[1], q[2], q[3]);
    store_rows3(B.R + 3 * i, R);
    B.lvel[i] = make_float4(lvel[0], lvel[1], lvel[2], lv.w);
    B.avel[i] = make_float4(avel[0], avel[1], avel[2], av.w);
    B.facc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    B.tacc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ FP64 residual
// A = J M^-1 J^T + diag(cfm), b = rhs, both as formed before Ad scaling
// (unscaled here by the stored Ad); bounds per quickstep.cpp:2972-2978.
__global__ void k_res_force(Rows Rw, const int *nrows_dev, double *f) {
    int n = *nrows_dev;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int2 b = Rw.body[r];
        const double ad = (double)Rw.Ad[r];
        const double l = (double)Rw.lambda[r] / ad;  // unscaled J = J'/Ad, so J^T lambda = J'^T lambda / Ad
        float4 a = Rw.J1l[r], c = Rw.J1a[r];
        atomicAdd(&f[6 * b.x + 0], a.x * l); atomicAdd(&f[6 * b.x + 1], a.y * l); atomicAdd(&f[6 * b.x + 2], a.z * l);
        atomicAdd(&f[6 * b.x + 3], c.x * l); atomicAdd(&f[6 * b.x + 4], c.y * l); atomicAdd(&f[6 * b.x + 5], c.z * l);
        if (b.y >= 0) {
            a = Rw.J2l[r]; c = Rw.J2a[r];
            atomicAdd(&f[6 * b.y + 0], a.x * l); atomicAdd(&f[6 * b.y + 1], a.y * l); atomicAdd(&f[6 * b.y + 2], a.z * l);
            atomicAdd(&f[6 * b.y + 3], c.x * l); atomicAdd(&f[6 * b.y + 4], c.y * l); atomicAdd(&f[6 * b.y + 5], c.z * l);
        }
    }
}
__global__ void k_res_vel(Bodies B, const double *f, double *v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    double im = B.pos[i].w;
    for (int k = 0; k < 3; k++) v[6 * i + k] = im * f[6 * i + k];
    for (int k = 0; k < 3; k++) {
        float4 row = B.invIw[3 * i + k];
        v[6 * i + 3 + k] = (double)row.x * f[6 * i + 3] + (double)row.y * f[6 * i + 4] + (double)row.z * f[6 * i + 5];
    }
}
__device__ __forceinline__ void atomic_max_d(double *addr, double v) {
    unsigned long long *a = (unsigned long long *)addr;
    unsigned long long nv = __double_as_longlong(v);
    atomicMax(a, nv);  // v >= 0: bit order equals value order
}
__global__ void k_res_rows(Rows Rw, Bodies B, const int *nrows_dev, const double *v, double *out) {
    int n = *nrows_dev;
    double rmax = 0, cmax = 0, lmax = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int2 b = Rw.body[r];
        const double ad = (double)Rw.Ad[r];
        float4 j1l = Rw.J1l[r], j1a = Rw.J1a[r], j2l = Rw.J2l[r], j2a = Rw.J2a[r];
        double J[12] = {j1l.x / ad, j1l.y / ad, j1l.z / ad, j1a.x / ad, j1a.y / ad, j1a.z / ad,
                        j2l.x / ad, j2l.y / ad, j2l.z / ad, j2a.x / ad, j2a.y / ad, j2a.z / ad};
        double rhs = j1l.w / ad, cfm = j1a.w / ad;
        double lam = Rw.lambda[r];
        double Av = 0, D = 0;
        for (int k = 0; k < 6; k++) Av += J[k] * v[6 * b.x + k];
        double im = B.pos[b.x].w;
        float I[12];
        load_rows3(B.invIw + 3 * b.x, I);
        for (int k = 0; k < 3; k++) D += J[k] * J[k] * im;
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) D += J[3 + a] * (double)I[4 * a + c] * J[3 + c];
        if (b.y >= 0) {
            for (int k = 0; k < 6; k++) Av += J[6 + k] * v[6 * b.y + k];
            double im2 = B.pos[b.y].w;
            load_rows3(B.invIw + 3 * b.y, I);
            for (int k = 0; k < 3; k++) D += J[6 + k] * J[6 + k] * im2;
            for (int a = 0; a < 3; a++)
                for (int c = 0; c < 3; c++) D += J[9 + a] * (double)I[4 * a + c] * J[9 + c];
        }
        double w = Av + cfm * lam - rhs;
        D += cfm;
        double lo, hi;
        int fi = Rw.findex[r];
        if (fi >= 0) { hi = fabs((double)j2a.w * (double)Rw.lambda[fi]); lo = -hi; }
        else { lo = j2l.w; hi = j2a.w; }
        double t = lam - w / D;
        t = fmin(fmax(t, lo), hi);
        rmax = fmax(rmax, fabs(lam - t));
        // complementarity, min-map form in the units of lambda (w / A_ii):
        // max(min(lambda - lo, w+ / D), min(hi - lambda, w- / D))
        const double wp = fmax(w, 0.0) / D, wm = fmax(-w, 0.0) / D;
        const double c = fmax(fmin(lam - lo, wp), fmin(hi - lam, wm));
        cmax = fmax(cmax, fabs(c));
        lmax = fmax(lmax, fabs(lam));
    }
    atomic_max_d(&out[0], rmax);
    atomic_max_d(&out[1], cmax);
    atomic_max_d(&out[2], lmax);
}

// joint feedback per contact: f = J^T lambda with the unscaled rows
// Records: the contacts' first (orig: solver contact -> caller's contact index
// when sleeping compacted the list, else null), then the ball/hinge/hinge2
// joints' from record nc on; word 3 of a record is set to 1 when it was solved
__global__ void k_feedback(Rows Rw, const int *nrows_dev, const int *orig, int nc, float *fb) {
    int n = *nrows_dev;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int c = Rw.contact[r];
        if (c < 0) c = nc + (-1 - c);  // joint k's row: owner -1 - k
        else {
            if (orig) c = orig[c];
            if (c >= nc) continue;  // contacts without a record (made on the device): no feedback
        }
        const int2 b = Rw.body[r];
        const float l = Rw.lambda[r] / Rw.Ad[r];
        float4 a = Rw.J1l[r], d = Rw.J1a[r];
        float *o = fb + 16 * c;
        o[3] = 1.f;
        atomicAdd(&o[0], a.x * l); atomicAdd(&o[1], a.y * l); atomicAdd(&o[2], a.z * l);
        atomicAdd(&o[4], d.x * l); atomicAdd(&o[5], d.y * l); atomicAdd(&o[6], d.z * l);
        if (b.y >= 0) {
            a = Rw.J2l[r]; d = Rw.J2a[r];
            atomicAdd(&o[8], a.x * l); atomicAdd(&o[9], a.y * l); atomicAdd(&o[10], a.z * l);
            atomicAdd(&o[12], d.x * l); atomicAdd(&o[13], d.y * l); atomicAdd(&o[14], d.z * l);
        }
    }
}

// ------------------------------------------------------------------ host side
static int grid_for(int n, int block) { return n <= 0 ? 1 : (n + block - 1) / block; }

Bodies bodies_view(Workspace &ws, int nb) {
    Bodies B;
    B.pos = ws.b_pos.as<float4>(); B.q = ws.b_q.as<float4>(); B.R = ws.b_R.as<float4>();
    B.lvel = ws.b_lvel.as<float4>(); B.avel = ws.b_avel.as<float4>(); B.facc = ws.b_facc.as<float4>();
    B.tacc = ws.b_tacc.as<float4>(); B.Ib = ws.b_Ib.as<float4>(); B.invIb = ws.b_invIb.as<float4>();
    B.invIw = ws.b_invIw.as<float4>(); B.fc = ws.b_fc.as<float4>(); B.rt = ws.b_rt.as<float4>();
    B.damp = ws.b_damp.as<float4>(); B.maxw = ws.b_maxw.as<float>();
    B.asleep = ws.sleep_on ? ws.b_asleep.as<int>() : nullptr;
    B.n = nb;
    return B;
}

bool ensure_bodies(Workspace &ws, int nb) {
    size_t n = nb > 0 ? nb : 1;
    return ws.b_pos.ensure(n * 16) && ws.b_q.ensure(n * 16) && ws.b_R.ensure(n * 48) && ws.b_lvel.ensure(n * 16) &&
           ws.b_avel.ensure(n * 16) && ws.b_facc.ensure(n * 16) && ws.b_tacc.ensure(n * 16) && ws.b_Ib.ensure(n * 48) &&
           ws.b_invIb.ensure(n * 48) && ws.b_invIw.ensure(n * 48) && ws.b_fc.ensure(n * 32) && ws.b_rt.ensure(n * 32) &&
           ws.b_fa.ensure(n * 8) && ws.m_mask.ensure(n * 16) && ws.m_claim.ensure(n * GB_MAX_COLOURS * 4) &&
           ws.res_f.ensure(n * 48) && ws.res_v.ensure(n * 48) && ws.b_damp.ensure(n * 16) && ws.b_maxw.ensure(n * 4);
}

bool ensure_rows(Workspace &ws, int ncap, int nj) {
    size_t nc = ncap > 0 ? ncap : 1;
    size_t ng = nc + (nj > 0 ? nj : 0);  // constraint groups: contact manifolds (at most one per contact) + joints
    // rows: up to 3 per contact (6 when a surface uses rolling friction), 6 per joint
    size_t rows = nc * (size_t)(ws.rows_per_contact > 0 ? ws.rows_per_contact : 6) + (size_t)(nj > 0 ? nj : 0) * 6;
    bool ok = ws.c_mcount.ensure((nc + 1) * 4) && ws.c_rstart.ensure((nc + 1) * 4) && ws.m_head.ensure((nc + 1) * 4) &&
              ws.m_id.ensure((nc + 1) * 4) && ws.m_start.ensure((nc + 2) * 4) && ws.m_colour.ensure((ng + 1) * 4) &&
              ws.m_tent.ensure((ng + 1) * 4) && ws.col_count.ensure(GB_MAX_COLOURS * 4 + 4) &&
              ws.col_start.ensure(GB_MAX_COLOURS * 4 + 4) && ws.col_fill.ensure(GB_MAX_COLOURS * 4 + 4) &&
              ws.col_list.ensure((ng + 1) * 4) && ws.m_desc.ensure((ng + 1) * 16) && ws.grp_body.ensure((ng + 1) * 8);
    if (!ok) return false;
    if (ws.row_cap < (int)rows) {
        ok = ws.r_J1l.ensure(rows * 16) && ws.r_J1a.ensure(rows * 16) && ws.r_J2l.ensure(rows * 16) &&
             ws.r_J2a.ensure(rows * 16) && ws.r_M1l.ensure(rows * 16) && ws.r_M1a.ensure(rows * 16) &&
             ws.r_M2l.ensure(rows * 16) && ws.r_M2a.ensure(rows * 16) && ws.r_lambda.ensure(rows * 4) &&
             ws.r_Ad.ensure(rows * 4) && ws.r_findex.ensure(rows * 4) && ws.r_contact.ensure(rows * 4) &&
             ws.r_body.ensure(rows * 8);
        if (!ok) return false;
        ws.row_cap = (int)rows;
    }
    return true;
}

static JointTable joint_view(Workspace &ws) {
    JointTable T;
    T.info = ws.j_info.as<int4>();
    T.a1 = ws.j_a1.as<float4>(); T.a2 = ws.j_a2.as<float4>();
    T.x1 = ws.j_x1.as<float4>(); T.x2 = ws.j_x2.as<float4>(); T.qrel = ws.j_qrel.as<float4>();
    T.l0 = ws.j_l0.as<float4>(); T.l1 = ws.j_l1.as<float4>(); T.l2 = ws.j_l2.as<float4>();
    T.v1 = ws.j_v1.as<float4>(); T.v2 = ws.j_v2.as<float4>();
    T.m0 = ws.j_m0.as<float4>(); T.m1 = ws.j_m1.as<float4>(); T.m2 = ws.j_m2.as<float4>();
    T.n = ws.njoints;
    T.m = ws.j_m.as<int>(); T.rstart = ws.j_rstart.as<int>(); T.limit = ws.j_limit.as<int>();
    T.lerr = ws.j_lerr.as<float>(); T.lam = ws.j_lam.as<float>();
    return T;
}

bool joint_table_upload(Workspace &ws, int n, const std::vector<const void *> &src, cudaStream_t s) {
    const size_t nn = n > 0 ? n : 1;
    DBuf *f4[13] = {&ws.j_a1, &ws.j_a2, &ws.j_x1, &ws.j_x2, &ws.j_qrel, &ws.j_l0, &ws.j_l1, &ws.j_l2,
                    &ws.j_v1, &ws.j_v2, &ws.j_m0, &ws.j_m1, &ws.j_m2};
    bool ok = ws.j_info.ensure(nn * 16) && ws.j_m.ensure((nn + 1) * 4) && ws.j_rstart.ensure((nn + 1) * 4) &&
              ws.j_limit.ensure(nn * 4) && ws.j_lerr.ensure(nn * 4) && ws.j_lam.ensure(nn * 24);
    for (DBuf *b : f4) ok = ok && b->ensure(nn * 16);
    if (!ok || src.size() != 14) return false;
    ws.njoints = n;
    if (n == 0) return true;
    cudaMemcpyAsync(ws.j_info.p, src[0], (size_t)n * 16, cudaMemcpyHostToDevice, s);
    for (int i = 0; i < 13; i++) cudaMemcpyAsync(f4[i]->p, src[1 + i], (size_t)n * 16, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(ws.j_lam.p, 0, (size_t)n * 24, s);  // a new table starts its joints from zero
    // the set of jointed body pairs, open addressing with the narrow phase's hash
    unsigned sz = 64;
    while (sz < 4u * (unsigned)n) sz <<= 1;
    std::vector<unsigned long long> keys(sz, ~0ull);
    const int4 *info = (const int4 *)src[0];
    for (int k = 0; k < n; k++) {
        const int a = info[k].y, b = info[k].z;
        if (a < 0 || b < 0) continue;
        const unsigned long long key = ((unsigned long long)(unsigned)std::min(a, b) << 32) | (unsigned)std::max(a, b);
        unsigned long long x = key;  // the same mixing as hash64 in collide.cu
        x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
        unsigned h = (unsigned)x & (sz - 1);
        while (keys[h] != ~0ull && keys[h] != key) h = (h + 1) & (sz - 1);
        keys[h] = key;
    }
    if (!ws.j_pairs.ensure((size_t)sz * 8)) return false;
    ws.j_pair_mask = sz - 1;
    cudaMemcpyAsync(ws.j_pairs.p, keys.data(), (size_t)sz * 8, cudaMemcpyHostToDevice, s);
    return cudaStreamSynchronize(s) == cudaSuccess;  // the host arrays die at return
}

static Rows rows_view(Workspace &ws) {
    Rows R;
    R.J1l = ws.r_J1l.as<float4>(); R.J1a = ws.r_J1a.as<float4>(); R.J2l = ws.r_J2l.as<float4>();
    R.J2a = ws.r_J2a.as<float4>(); R.M1l = ws.r_M1l.as<float4>(); R.M1a = ws.r_M1a.as<float4>();
    R.M2l = ws.r_M2l.as<float4>(); R.M2a = ws.r_M2a.as<float4>();
    R.lambda = ws.r_lambda.as<float>(); R.Ad = ws.r_Ad.as<float>(); R.findex = ws.r_findex.as<int>();
    R.contact = ws.r_contact.as<int>(); R.body = ws.r_body.as<int2>();
    R.n_cap = ws.row_cap;
    return R;
}

static int coop_blocks(const void *kernel, int block, int max_per_sm) {
    // queried once per (kernel, block size): the answer does not change, and no
    // query then runs while a step is recorded into a graph
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find({kernel, block});
        if (it != cache.end()) per_sm = it->second;
        else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
            cache[{kernel, block}] = per_sm;
        }
    }
    if (per_sm < 1) per_sm = 1;
    if (per_sm > max_per_sm) per_sm = max_per_sm;
    return per_sm * num_sms();
}

// Per-part capacities of the two-level sweep from the shared memory a block
// may opt into (once; thread-safe static initialisation): bodies and groups
// fixed, the rest for interior rows.  Sized for the 32,768-body pile on 152
// columns (per column at most ~240 bodies, ~520 interior manifolds and ~1,920
// interior rows), whose every column then keeps its interior manifolds.
struct SlabCaps {
    int bcap, gcap, rcap;
    size_t smem;
};
template <int T>
static SlabCaps slab_caps_t() {
    static const SlabCaps caps = []() {
        SlabCaps c{288, 560, 0, 0};
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, (const void *)k_pgs_slab<T>) != cudaSuccess) return c;
        const long long fixed = (long long)fa.sharedSizeBytes + (long long)slab_smem_bytes(GB_SLAB_XCHUNK, 0, c.bcap, c.gcap);
        const long long room = (long long)optin - fixed - 256;  // a little kept for the runtime's own use
        c.rcap = room > 0 ? (int)(room / 84) : 0;
        c.smem = slab_smem_bytes(GB_SLAB_XCHUNK, c.rcap, c.bcap, c.gcap);
        if (c.rcap > 0 &&
            cudaFuncSetAttribute((const void *)k_pgs_slab<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)c.smem) != cudaSuccess)
            c.rcap = 0;
        return c;
    }();
    return caps;
}
static SlabCaps slab_caps(int threads) { return threads == 128 ? slab_caps_t<128>() : slab_caps_t<256>(); }

// The one-level sweep kernel's shared-memory opt-in (two buffers of at most
// GB_CHUNK_ROWS rows) and its co-residency, once per instance.
template <int T>
static int pgs_per_sm() {
    static const int v = []() {
        const size_t smem = (size_t)2 * GB_CHUNK_ROWS * 128;
        const size_t smem_mom = (size_t)2 * GB_CHUNK_ROWS_MOM * 128 + (size_t)T * GB_STAGED_ROWS * 4;
        cudaFuncSetAttribute((const void *)k_pgs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(smem > smem_mom ? smem : smem_mom));
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(&n, (const void *)k_pgs<T>, T, smem, 0);
        return n;
    }();
    return v;
}

static bool ensure_warm(Workspace &ws) {
    unsigned want = 1024;
    while (want < 2u * (unsigned)(ws.contact_cap > 0 ? ws.contact_cap : 1) && want < (1u << 23)) want <<= 1;
    if (ws.warm_mask + 1 != want) {
        ws.warm_valid = false;  // a grown table holds no previous step, whether or not both grow
        if (!(ws.w_keys.ensure((size_t)2 * want * 8) && ws.w_lambda.ensure((size_t)2 * want * 16))) return false;
        ws.warm_mask = want - 1;
    }
    return true;
}

static WarmTable warm_lookup(Workspace &ws, const SolverParams &P) {
    WarmTable W{nullptr, nullptr, 0, 0.f};
    if (P.warm_mode && ws.warm_valid) {
        W.keys = ws.w_keys.as<unsigned long long>();
        W.lam = ws.w_lambda.as<float4>();
        W.mask = ws.warm_mask;
        W.scale = P.warm_scale;
    }
    return W;
}

// The contacts the solver reads: all of them, or, when the sleep stage ran in
// this step, the compacted contacts of awake components.
static const Contact *solve_contacts(Workspace &ws) {
    return ws.use_awake ? ws.c_awake.as<Contact>() : ws.contacts.as<Contact>();
}
static const int *solve_count(Workspace &ws) { return ws.use_awake ? &ws.dc->nawake : &ws.dc->ncontacts; }

static void warm_store(Workspace &ws, cudaStream_t s) {
    unsigned long long *keys = ws.w_keys.as<unsigned long long>();
    float4 *lam = ws.w_lambda.as<float4>();
    k_warm_clear<<<4 * num_sms(), 256, 0, s>>>(keys, ws.warm_mask, ws.dc);
    k_warm_store<<<4 * num_sms(), 256, 0, s>>>(solve_contacts(ws), solve_count(ws), ws.c_rstart.as<int>(),
                                               ws.c_mcount.as<int>(), rows_view(ws), keys, lam, ws.warm_mask, ws.dc);
    k_warm_flip<<<1, 1, 0, s>>>(ws.dc);
    count_launch(3);
    ws.warm_valid = true;
}

// Sizes of the coloured solver's per-step buffers (host-known: capacities,
// joints, blocks, the two-level sweep's partition).
struct ColouredPlan {
    int pgs_blocks, sx, sy, chunk_cap, ncb, threads;
    int split;  // split classes asked for (two-level sweep), 0: none
    bool slab;
    SlabCaps caps;
    size_t ngroups, wave_cap;
};
static ColouredPlan plan_coloured(const Workspace &ws, const SolverParams &P) {
    ColouredPlan c;
    c.pgs_blocks = P.pgs_blocks > 0 && P.pgs_blocks < num_sms() ? P.pgs_blocks : num_sms();
    c.threads = P.pgs_threads == 128 ? 128 : GB_PGS_THREADS;
    c.caps = slab_caps(c.threads);
    c.slab = P.pgs_two_level && c.pgs_blocks >= 2 && c.caps.rcap > 0;
    c.split = c.slab && P.pgs_split >= 2 ? P.pgs_split : 0;
    c.ngroups = (size_t)(ws.contact_cap > 0 ? ws.contact_cap : 1) + (ws.njoints > 0 ? ws.njoints : 0);
    c.sx = 1;
    if (c.slab)
        for (int d = 1; d * d <= c.pgs_blocks; d++)
            if (c.pgs_blocks % d == 0) c.sx = d;
    c.sy = c.pgs_blocks / c.sx;
    c.ncb = GB_MAX_COLOURS * c.pgs_blocks;
    const int chunk = P.pgs_chunk > 0 ? (P.pgs_chunk < 64 ? 64 : (P.pgs_chunk > GB_CHUNK_ROWS ? GB_CHUNK_ROWS : P.pgs_chunk))
                                      : GB_CHUNK_ROWS;
    c.chunk_cap = c.slab ? GB_SLAB_XCHUNK : chunk;
    // momentum on the one-level sweep stages each thread's previous-sweep
    // results beside the chunk buffers (GB_STAGED_ROWS floats a thread)
    if (!c.slab && P.momentum > 0.f && c.chunk_cap > GB_CHUNK_ROWS_MOM) c.chunk_cap = GB_CHUNK_ROWS_MOM;
    // waves: one per (colour, block) at least, plus one per T slots and per chunk_cap - 12 staged rows
    c.wave_cap = 2 * (size_t)c.ncb + c.ngroups / c.threads + (size_t)ws.row_cap / (c.chunk_cap - 12) + 16;
    return c;
}

static bool ensure_coloured(Workspace &ws, int nb, const ColouredPlan &c) {
    if (!(ws.p_rows.ensure((size_t)ws.row_cap * 128) && ws.wv_count.ensure((size_t)c.ncb * 4) &&
          ws.wv_base.ensure((size_t)c.ncb * 4 + 4) && ws.chunk_rows.ensure(c.wave_cap * 4) &&
          ws.chunk_start.ensure(c.wave_cap * 4) && ws.wv_col.ensure(c.wave_cap * 4) &&
          ws.wv_sched.ensure(c.wave_cap * c.threads * 4)))
        return false;
    if (!c.slab) return true;
    const size_t nbb = nb > 0 ? nb : 1, npc = (size_t)c.pgs_blocks * GB_SLAB_COLOURS;
    const size_t nh = (size_t)GB_SLAB_NBIN * (1 + c.sx), ng = c.ngroups;
    return ws.s_bw.ensure(nbb * 4) && ws.s_part.ensure(nbb * 4) && ws.s_blocal.ensure(nbb * 4) &&
           ws.s_pbcount.ensure((size_t)c.pgs_blocks * 4) && ws.s_pbody.ensure((size_t)c.pgs_blocks * c.caps.bcap * 4) &&
           ws.s_prow.ensure((size_t)c.pgs_blocks * 4) && ws.s_pgrp.ensure((size_t)c.pgs_blocks * 4) &&
           ws.s_gpart.ensure((ng + 1) * 4) && ws.s_gdesc.ensure((ng + 1) * 16) && ws.s_pccount.ensure(npc * 4) &&
           ws.s_pcstart.ensure((npc + 1) * 4) && ws.s_pcfill.ensure(npc * 4) && ws.s_ilist.ensure((ng + 1) * 4) &&
           ws.s_irown.ensure((ng + 1) * 4) && ws.s_irowoff.ensure((ng + 1) * 4) && ws.s_idesc.ensure((ng + 1) * 16) &&
           ws.s_ipack.ensure((size_t)ws.row_cap * 80) && ws.s_hist.ensure(nh * 4) && ws.s_binpart.ensure(nh * 4) &&
           ws.x_cnt.ensure((size_t)64 * c.pgs_blocks * 4) && ws.x_start.ensure((size_t)64 * c.pgs_blocks * 4 + 4) &&
           ws.x_fill.ensure((size_t)64 * c.pgs_blocks * 4) && ws.x_accn.ensure(nbb * 4) &&
           ws.x_acc.ensure(nbb * GB_XACC * 4) && ws.x_adj.ensure((size_t)c.pgs_blocks * GB_XADJ_WORDS * 4) &&
           ws.x_prog.ensure((size_t)c.pgs_blocks * 4) &&
           ws.x_dacc.ensure((size_t)(c.split > 0 ? c.split : 1) * nbb * 48) &&
           (!c.split || (ws.x_nsplit.ensure((size_t)c.split * nbb * 4) && ws.x_smask.ensure(nbb * 4)));
}

// Every device buffer a step writes, allocated before its first kernel: an
// allocation that fails leaves the world's state as it was (the step returns
// 0 having launched nothing).
static bool reserve_step(Workspace &ws, int nb, const SolverParams &P, bool coloured) {
    const int nj = ws.njoints;
    if (!ensure_rows(ws, ws.contact_cap, nj)) return false;
    if (P.warm_mode && !ensure_warm(ws)) return false;
    const size_t nc = ws.contact_cap > 0 ? ws.contact_cap : 1;
    if (ws.sleep_on && !(ws.c_keep.ensure(nc * 4) && ws.c_kpos.ensure(nc * 4) &&
                         ws.c_awake.ensure(nc * sizeof(Contact)) && ws.c_orig.ensure(nc * 4)))
        return false;
    if ((P.learned || P.learn_capture) &&
        !(ws.l_feat.ensure(nc * GB_MLP_IN * 4) && ws.l_scale.ensure(nc * 4) && ws.l_pred.ensure(nc * GB_MLP_OUT * 4)))
        return false;
    if (P.learned && !ws.l_alt.ensure((size_t)ws.row_cap * 4)) return false;
    // the scan scratch for the longest scan of the step
    size_t nscan = nc + 1;
    nscan = std::max(nscan, (size_t)(nj > 0 ? nj : 1));
    nscan = std::max(nscan, (size_t)(nb > 0 ? nb : 1));
    nscan = std::max(nscan, (size_t)GB_MAX_COLOURS);
    if (coloured) {
        const ColouredPlan c = plan_coloured(ws, P);
        if (!ensure_coloured(ws, nb, c)) return false;
        if (P.momentum > 0.f &&
            !(ws.m_lprev.ensure((size_t)ws.row_cap * 4) && ws.b_fcprev.ensure((size_t)(nb > 0 ? nb : 1) * 32)))
            return false;
        nscan = std::max(nscan, std::max((size_t)c.ncb, c.wave_cap));
        nscan = std::max(nscan, std::max((size_t)c.pgs_blocks * GB_SLAB_COLOURS, c.ngroups));
    }
    return ws.scan_tmp.ensure(sizeof(int) * ((nscan + 1023) / 1024 + 2));
}

static bool assemble(Workspace &ws, int nb, const SolverParams &P, cudaStream_t s, bool coloured = false) {
    Bodies B = bodies_view(ws, nb);
    const int nj = ws.njoints;
    if (!reserve_step(ws, nb, P, coloured)) return false;
    JointTable T = joint_view(ws);
    // sleeping: the idle test and the island rule decide which bodies, joints
    // and contacts this step processes (skipped when the caller ran it already
    // and handed over the contacts of awake components only)
    ws.use_awake = false;
    if (ws.sleep_on && !ws.sleep_precomputed) {
        if (!launch_sleep(ws, nb, P.dt, s)) return false;
        ws.use_awake = true;
    }
    ws.sleep_precomputed = false;
    // joint getInfo1 first: a powered hinge at its limit adds motor torques to
    // the bodies before their right-hand side is formed
    if (nj > 0) {
        k_joint_m<<<grid_for(nj, 128), 128, 0, s>>>(T, B);
        count_launch();
    }
    k_bodies<<<grid_for(nb, 128), 128, 0, s>>>(B, P);
    int grid = 4 * num_sms();
    const Contact *C = solve_contacts(ws);
    const int *ncp = solve_count(ws);
    const Surface *S = ws.surfaces.as<Surface>();
    k_contact_m<<<grid, 256, 0, s>>>(C, S, ncp, ws.c_mcount.as<int>());
    scan_exclusive(ws.c_mcount.as<int>(), ws.c_rstart.as<int>(), ncp, ws.contact_cap, &ws.dc->nrows, ws, s);
    // the capacity the assembly sees (lowered only by the error-path tests, in worlds without joints)
    const int row_cap_seen = g_test.row_cap > 0 && nj == 0 && g_test.row_cap < ws.row_cap ? g_test.row_cap : ws.row_cap;
    k_rows_total<<<1, 1, 0, s>>>(ws.dc, row_cap_seen, ws.c_rstart.as<int>(), ws.c_mcount.as<int>(),
                                 const_cast<int *>(ncp));
    if (nj > 0) scan_exclusive(T.m, T.rstart, nullptr, nj, &ws.dc->njoint_rows, ws, s);
    else cudaMemsetAsync(&ws.dc->njoint_rows, 0, 4, s);
    k_joint_rows_total<<<1, 1, 0, s>>>(ws.dc, ws.row_cap);
    count_launch();
    const int dyn = (P.solver == 1) && (P.premature_delta != 0 || P.extra_factor != 0);
    LearnOut L = {nullptr, nullptr};
    if (P.learned || P.learn_capture) {
        L.feat = ws.l_feat.as<float>();
        L.scale = ws.l_scale.as<float>();
    }
    k_rows<<<grid, 64, 0, s>>>(C, S, ncp, ws.c_rstart.as<int>(), B, rows_view(ws), P, dyn,
                               warm_lookup(ws, P), ws.dc, L);
    count_launch(4);
    if (nj > 0) {
        k_joint_rows<<<grid_for(nj, 64), 64, 0, s>>>(T, B, rows_view(ws), P, dyn, ws.dc, P.warm_mode != 0);
        count_launch();
    }
    if (P.learned) {
        if (!ws.mlp_wb.p) return false;
        if (!mlp_infer(ws.mlp_wb.as<unsigned char>(), ws.l_feat.as<float>(), 0, ncp, ws.l_pred.as<float>(),
                       &ws.dc->err, s))
            return false;
        k_learned_apply<<<grid, 128, 0, s>>>(ncp, ws.c_rstart.as<int>(), ws.c_mcount.as<int>(),
                                             ws.l_scale.as<float>(), ws.l_pred.as<float>(), rows_view(ws),
                                             ws.l_alt.as<float>(), ws.dc);
        count_launch();
    }
    return true;
}

bool assemble_step(Workspace &ws, int nb, const SolverParams &P, cudaStream_t s) {
    cudaMemsetAsync(&ws.dc->iterations, 0, 4, s);
    return assemble(ws, nb, P, s);
}
bool launch_integrate(Workspace &ws, int nb, const SolverParams &P, cudaStream_t s) {
    k_integrate<<<grid_for(nb, 128), 128, 0, s>>>(bodies_view(ws, nb), P);
    count_launch();
    return cudaGetLastError() == cudaSuccess;
}
Rows rows_view_public(Workspace &ws) { return rows_view(ws); }

// The solver's contacts of the last assembly (all of them, or those of awake
// components), with their bodies (static: -1) and row ranges; syncs.
int download_solver_contacts(Workspace &ws, std::vector<int2> &bodies, std::vector<int> &rstart,
                             std::vector<int> &mcount, cudaStream_t s) {
    int nc = 0;
    cudaMemcpyAsync(&nc, solve_count(ws), 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    std::vector<Contact> C(nc > 0 ? nc : 1);
    rstart.assign(nc > 0 ? nc : 1, 0);
    mcount.assign(nc > 0 ? nc : 1, 0);
    if (nc > 0) {
        cudaMemcpyAsync(C.data(), solve_contacts(ws), (size_t)nc * sizeof(Contact), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(rstart.data(), ws.c_rstart.p, (size_t)nc * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(mcount.data(), ws.c_mcount.p, (size_t)nc * 4, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    }
    bodies.resize(nc > 0 ? nc : 1);
    for (int k = 0; k < nc; k++) bodies[k] = make_int2(C[k].b1, C[k].b2);
    return nc;
}

bool launch_quickstep(Workspace &ws, int nb, int, const SolverParams &P, cudaStream_t s, cudaEvent_t ev0,
                      cudaEvent_t ev1) {
    if (!assemble(ws, nb, P, s, true)) return false;
    const Contact *C = solve_contacts(ws);
    const int *ncp = solve_count(ws);
    int grid = 4 * num_sms();
    // manifolds
    k_manifold_heads<<<grid, 256, 0, s>>>(C, ncp, ws.m_head.as<int>());
    scan_exclusive(ws.m_head.as<int>(), ws.m_id.as<int>(), ncp, ws.contact_cap, &ws.dc->nmanifolds, ws, s);
    k_manifold_starts<<<grid, 256, 0, s>>>(ncp, ws.m_head.as<int>(), ws.m_id.as<int>(), ws.m_start.as<int>(),
                                           ws.dc);
    k_groups<<<grid, 256, 0, s>>>(C, ws.m_start.as<int>(), ws.j_info.as<int4>(), ws.njoints, ws.dc,
                                  ws.grp_body.as<int2>());
    k_groups_total<<<1, 1, 0, s>>>(ws.dc, ws.njoints);
    count_launch(2);
    // the buffers below were reserved before the step's first kernel (reserve_step)
    const ColouredPlan plan = plan_coloured(ws, P);
    const int pgs_blocks = plan.pgs_blocks;
    // two-level sweep: parts, interior / cross classes of the groups
    const SlabCaps caps = plan.caps;
    const bool slab = plan.slab;
    const size_t ngroups = plan.ngroups;
    const int sx = plan.sx, sy = plan.sy;
    if (slab) {
        const size_t nbb = nb > 0 ? nb : 1;
        const size_t nh = (size_t)GB_SLAB_NBIN * (1 + sx);
        Bodies B = bodies_view(ws, nb);
        cudaMemsetAsync(ws.s_bw.p, 0, nbb * 4, s);
        cudaMemsetAsync(ws.s_hist.p, 0, nh * 4, s);
        cudaMemsetAsync(ws.s_pbcount.p, 0, (size_t)pgs_blocks * 4, s);
        cudaMemsetAsync(ws.s_prow.p, 0, (size_t)pgs_blocks * 4, s);
        cudaMemsetAsync(ws.s_pgrp.p, 0, (size_t)pgs_blocks * 4, s);
        k_group_desc<<<grid, 256, 0, s>>>(ws.m_start.as<int>(), ws.c_rstart.as<int>(), ws.c_mcount.as<int>(),
                                          ws.r_body.as<int2>(), ws.r_findex.as<int>(), ws.dc, ws.s_gdesc.as<int4>(),
                                          ws.j_rstart.as<int>(), ws.j_m.as<int>(), ws.grp_body.as<int2>());
        k_slab_weight<<<grid, 256, 0, s>>>(C, ncp, ws.s_bw.as<int>(), ws.dc);
        k_slab_range<<<grid, 256, 0, s>>>(B, ws.s_bw.as<int>(), ws.dc);
        k_slab_hist<<<grid, 256, 0, s>>>(B, ws.s_bw.as<int>(), ws.dc, ws.s_binpart.as<int>(), ws.s_hist.as<int>(), 0);
        k_slab_cut<<<1, GB_SLAB_NBIN, 0, s>>>(ws.s_hist.as<int>(), ws.s_binpart.as<int>(), sx);
        k_slab_hist<<<grid, 256, 0, s>>>(B, ws.s_bw.as<int>(), ws.dc, ws.s_binpart.as<int>(), ws.s_hist.as<int>(), 1);
        k_slab_cut<<<sx, GB_SLAB_NBIN, 0, s>>>(ws.s_hist.as<int>() + GB_SLAB_NBIN,
                                               ws.s_binpart.as<int>() + GB_SLAB_NBIN, sy);
        k_slab_assign<<<grid, 256, 0, s>>>(B, ws.s_bw.as<int>(), ws.dc, ws.s_binpart.as<int>(), sy,
                                           ws.s_part.as<int>(), ws.s_blocal.as<int>(), ws.s_pbcount.as<int>(),
                                           ws.s_pbody.as<int>(), caps.bcap);
        k_slab_classify<<<grid, 256, 0, s>>>(ws.s_gdesc.as<int4>(), ws.dc, ws.s_part.as<int>(), ws.s_gpart.as<int>(),
                                             ws.s_prow.as<int>(), ws.s_pgrp.as<int>());
        k_slab_demote<<<grid, 256, 0, s>>>(ws.dc, ws.s_prow.as<int>(), ws.s_pgrp.as<int>(), ws.s_pbcount.as<int>(),
                                           caps.rcap, caps.gcap, caps.bcap, ws.s_gpart.as<int>());
        count_launch(10);
    }
    // colouring
    cudaMemsetAsync(ws.m_mask.p, 0, (size_t)(nb > 0 ? nb : 1) * 16, s);
    cudaMemsetAsync(ws.m_claim.p, 0x7f, (size_t)(nb > 0 ? nb : 1) * GB_MAX_COLOURS * 4, s);
    cudaMemsetAsync(&ws.dc->ncolours, 0, 4, s);
    cudaMemsetAsync(&ws.dc->nicolours, 0, 4, s);
    cudaMemsetAsync(&ws.dc->slab_sync, 0, 4, s);
    cudaMemsetAsync(&ws.dc->slab_rows, 0, 4, s);
    cudaMemsetAsync(&ws.dc->gsync, 0, sizeof(GridSync), s);
    {
        int blocks = coop_blocks((const void *)k_colour, 256, 2);
        unsigned long long *mask = ws.m_mask.as<unsigned long long>();
        int *claim = ws.m_claim.as<int>(), *colour = ws.m_colour.as<int>(), *tent = ws.m_tent.as<int>();
        const int2 *gbody = ws.grp_body.as<int2>();
        DevCounters *dc = ws.dc;
        const int *cls = slab ? ws.s_gpart.as<int>() : nullptr;
        int climit = g_test.colour_cap > 0 && g_test.colour_cap < GB_MAX_COLOURS ? g_test.colour_cap : GB_MAX_COLOURS;
        void *args[] = {(void *)&gbody, (void *)&dc, (void *)&mask, (void *)&claim, (void *)&colour, (void *)&tent,
                        (void *)&nb, (void *)&cls, (void *)&climit};
        if (cudaLaunchCooperativeKernel((const void *)k_colour, blocks, 256, args, 0, s) != cudaSuccess) return false;
    }
    // split classes: the crossing colours merged into plan.split classes
    const int nsplit = plan.split;
    cudaMemsetAsync(&ws.dc->split_off, 0, 4, s);
    cudaMemsetAsync(&ws.dc->split_k, 0, 4, s);
    if (nsplit) {
        const size_t nbb = nb > 0 ? nb : 1;
        k_split_check<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.s_gdesc.as<int4>(), ws.grp_body.as<int2>(),
                                           ws.s_part.as<int>(), ws.s_blocal.as<int>(), caps.bcap);
        k_split_classes<<<1, 1, 0, s>>>(ws.dc, nsplit);
        k_split_remap<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>());
        cudaMemsetAsync(ws.x_nsplit.p, 0, (size_t)nsplit * nbb * 4, s);
        k_split_count<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.grp_body.as<int2>(), nb,
                                           ws.x_nsplit.as<int>());
        k_split_mask<<<grid, 256, 0, s>>>(ws.dc, ws.x_nsplit.as<int>(), nb, ws.x_smask.as<int>());
        count_launch(5);
    }
    // momentum between sweeps on the two-level sweep: every body a crossing group touches is in a column's list
    cudaMemsetAsync(&ws.dc->mom_off, 0, 4, s);
    if (slab && P.momentum > 0.f) {
        k_mom_check<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.grp_body.as<int2>(), ws.s_part.as<int>(),
                                         ws.s_blocal.as<int>(), caps.bcap);
        count_launch();
    }
    cudaMemsetAsync(ws.col_count.p, 0, GB_MAX_COLOURS * 4, s);
    cudaMemsetAsync(ws.col_fill.p, 0, GB_MAX_COLOURS * 4, s);
    k_colour_count<<<grid, 256, 0, s>>>(ws.m_colour.as<int>(), ws.dc, ws.col_count.as<int>());
    scan_exclusive(ws.col_count.as<int>(), ws.col_start.as<int>(), nullptr, GB_MAX_COLOURS, &ws.dc->colour_total, ws, s);
    k_colour_fill<<<grid, 256, 0, s>>>(ws.m_colour.as<int>(), ws.dc, ws.col_start.as<int>(), ws.col_fill.as<int>(),
                                       ws.col_list.as<int>());
    // two-level sweep with neighbour waits: the cross colours' lists owner block by owner block
    const bool xspatial = slab && !P.pgs_grid_sync;
    const int *xstart = nullptr, *xcnt = nullptr;
    if (xspatial) {
        const size_t nx = (size_t)64 * pgs_blocks;
        cudaMemsetAsync(ws.x_cnt.p, 0, nx * 4, s);
        cudaMemsetAsync(ws.x_fill.p, 0, nx * 4, s);
        k_xown_count<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.grp_body.as<int2>(), ws.s_part.as<int>(),
                                          pgs_blocks, ws.x_cnt.as<int>());
        scan_exclusive(ws.x_cnt.as<int>(), ws.x_start.as<int>(), nullptr, (int)nx, nullptr, ws, s);
        k_xown_fill<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.grp_body.as<int2>(), ws.s_part.as<int>(),
                                         pgs_blocks, ws.x_start.as<int>(), ws.x_fill.as<int>(), ws.col_list.as<int>());
        count_launch(2);
        xstart = ws.x_start.as<int>();
        xcnt = ws.x_cnt.as<int>();
    }
    k_manifold_desc<<<grid, 256, 0, s>>>(ws.col_list.as<int>(), ws.m_start.as<int>(), ws.c_rstart.as<int>(),
                                         ws.c_mcount.as<int>(), ws.r_body.as<int2>(), ws.r_findex.as<int>(), ws.dc,
                                         ws.m_desc.as<int4>(), ws.j_rstart.as<int>(), ws.j_m.as<int>(),
                                         ws.grp_body.as<int2>());
    // cut every (colour, block)'s slots into waves and pack their rows chunk by
    // chunk for the solver's blocks
    const int ncb = plan.ncb;
    const int chunk_cap = plan.chunk_cap;
    const size_t wave_cap = plan.wave_cap;
    const int threads = plan.threads;
    {
        const int g1 = (ncb * 32 + 127) / 128;  // a warp per (colour, block)
        k_wave_count<<<g1, 128, 0, s>>>(ws.col_start.as<int>(), ws.col_count.as<int>(), ws.dc, ws.m_desc.as<int4>(),
                                        ws.wv_count.as<int>(), pgs_blocks, chunk_cap, threads, xstart, xcnt);
        scan_exclusive(ws.wv_count.as<int>(), ws.wv_base.as<int>(), nullptr, ncb, nullptr, ws, s);
        k_wave_total<<<1, 1, 0, s>>>(ws.dc, ws.wv_count.as<int>(), ws.wv_base.as<int>(), pgs_blocks);
        k_wave_fill<<<g1, 128, 0, s>>>(ws.col_start.as<int>(), ws.col_count.as<int>(), ws.dc, ws.m_desc.as<int4>(),
                                       ws.wv_count.as<int>(), ws.wv_base.as<int>(), ws.wv_sched.as<int>(),
                                       ws.chunk_rows.as<int>(), ws.wv_col.as<int>(), (int)wave_cap, pgs_blocks,
                                       chunk_cap, threads, xstart, xcnt);
        scan_exclusive(ws.chunk_rows.as<int>(), ws.chunk_start.as<int>(), &ws.dc->nwaves, (int)wave_cap, nullptr, ws, s);
        k_pack_rows<<<grid, threads, 0, s>>>(rows_view(ws), ws.col_start.as<int>(), ws.dc, ws.m_desc.as<int4>(),
                                                    ws.wv_sched.as<int>(), ws.wv_col.as<int>(),
                                                    ws.chunk_start.as<int>(), ws.p_rows.as<float4>(),
                                                    nsplit ? ws.x_nsplit.as<int>() : nullptr, ws.x_smask.as<int>(),
                                                    nb);
        count_launch(4);
    }
    if (slab) {
        // interior groups part by part, colour by colour; their rows packed
        const int npc = pgs_blocks * GB_SLAB_COLOURS;
        int *pcstart = ws.s_pcstart.as<int>();
        cudaMemsetAsync(ws.s_pccount.p, 0, (size_t)npc * 4, s);
        cudaMemsetAsync(ws.s_pcfill.p, 0, (size_t)npc * 4, s);
        k_slab_count<<<grid, 256, 0, s>>>(ws.dc, ws.s_gpart.as<int>(), ws.m_colour.as<int>(), ws.s_pccount.as<int>());
        scan_exclusive(ws.s_pccount.as<int>(), pcstart, nullptr, npc, pcstart + npc, ws, s);
        k_slab_fill<<<grid, 256, 0, s>>>(ws.dc, ws.s_gpart.as<int>(), ws.m_colour.as<int>(), ws.s_gdesc.as<int4>(),
                                         pcstart, ws.s_pcfill.as<int>(), ws.s_ilist.as<int>(), ws.s_irown.as<int>());
        scan_exclusive(ws.s_irown.as<int>(), ws.s_irowoff.as<int>(), pcstart + npc, (int)ngroups, nullptr, ws, s);
        k_slab_pack<<<grid, 256, 0, s>>>(rows_view(ws), bodies_view(ws, nb), ws.s_gpart.as<int>(),
                                         ws.s_gdesc.as<int4>(), ws.s_ilist.as<int>(), ws.s_irowoff.as<int>(),
                                         ws.s_irown.as<int>(), pcstart, ws.s_blocal.as<int>(), npc,
                                         ws.s_idesc.as<int4>(), ws.s_ipack.as<float4>(), ws.dc);
        count_launch(3);
    }
    if (xspatial || nsplit) {
        // the blocks touching each body, and every two of them adjacent
        const size_t nbb = nb > 0 ? nb : 1;
        cudaMemsetAsync(ws.x_accn.p, 0, nbb * 4, s);
        cudaMemsetAsync(&ws.dc->slab_nbr_over, 0, 4, s);
        k_xacc<<<grid, 256, 0, s>>>(ws.dc, ws.m_colour.as<int>(), ws.grp_body.as<int2>(), ws.s_part.as<int>(),
                                    pgs_blocks, ws.x_accn.as<int>(), ws.x_acc.as<int>());
        count_launch();
        if (xspatial) {
            cudaMemsetAsync(ws.x_adj.p, 0, (size_t)pgs_blocks * GB_XADJ_WORDS * 4, s);
            k_xadj<<<grid, 256, 0, s>>>(ws.x_accn.as<int>(), ws.x_acc.as<int>(), ws.s_part.as<int>(), nb,
                                        ws.x_adj.as<unsigned>());
            cudaMemsetAsync(ws.x_prog.p, 0, (size_t)pgs_blocks * 4, s);
            count_launch();
        }
    }
    // the two-level sweep re-forms the accumulators in fixed-point integer
    // slots (one per body and class; class 0 without split classes)
    if (slab) cudaMemsetAsync(ws.x_dacc.p, 0, (size_t)(nsplit > 0 ? nsplit : 1) * (nb > 0 ? nb : 1) * 48, s);
    // solve
    cudaMemsetAsync(&ws.dc->gsync, 0, sizeof(GridSync), s);
    if (g_test.barrier) {
        // error-path tests: the counter starts one arrival short, so the
        // solver's first grid barrier never completes and its bounded wait runs out
        cudaMemsetAsync(&ws.dc->gsync.count, 0xff, sizeof(unsigned), s);
        // and every block's step counter one step short: the first neighbour wait runs out
        if (xspatial) cudaMemsetAsync(ws.x_prog.p, 0xff, (size_t)pgs_blocks * 4, s);
        g_test.barrier = 0;
    }
    cudaMemsetAsync(ws.dc->racc, 0, 4 * sizeof(float), s);
    cudaMemsetAsync(&ws.dc->iterations, 0, 4, s);
    cudaMemsetAsync(&ws.dc->nhist, 0, 4, s);
    cudaMemsetAsync(&ws.dc->mom_final, 0, 4, s);
    if (ev0) cudaEventRecord(ev0, s);
    {
        PgsArgs A;
        A.Rw = rows_view(ws);
        A.fc = ws.b_fc.as<float4>();
        A.desc = ws.m_desc.as<int4>();
        A.cstart = ws.col_start.as<int>(); A.ccount = ws.col_count.as<int>();
        A.dc = ws.dc;
        A.iterations = P.iterations;
        A.max_iterations = P.max_iterations > 0 ? P.max_iterations : P.iterations;
        A.check_every = P.check_every > 0 ? P.check_every : 10;
        A.target = P.residual_target;
        A.w_sor = P.w;
        A.warm = P.warm_mode != 0;
        A.nb = nb;
        A.reform_every = P.reform_every > 0 ? P.reform_every : 500;
        A.predict_checks = P.fixed_checks ? 0 : 1;
        A.learned = P.learned;
        A.lam_alt = P.learned ? ws.l_alt.as<float>() : nullptr;
        A.passes = P.pgs_passes > 1 ? P.pgs_passes : 1;
        A.poison_stage = g_test.stage;
        g_test.stage = 0;
        A.packed = ws.p_rows.as<float4>();
        A.chunk_start = ws.chunk_start.as<int>();
        A.chunk_rows = ws.chunk_rows.as<int>();
        A.wcount = ws.wv_count.as<int>();
        A.wbase = ws.wv_base.as<int>();
        A.sched = ws.wv_sched.as<int>();
        A.chunk_cap = chunk_cap;
        A.momentum = P.momentum;
        A.lprev = P.momentum > 0.f ? ws.m_lprev.as<float>() : nullptr;
        A.fcprev = P.momentum > 0.f ? ws.b_fcprev.as<float4>() : nullptr;
        // one block per SM (the grid barrier's cost grows with the block count;
        // the chunk packing above assumes exactly pgs_blocks blocks)
        // two chunk buffers, and with momentum the threads' previous-sweep results
        const size_t smem = (size_t)2 * chunk_cap * 128 + (A.lprev ? (size_t)threads * GB_STAGED_ROWS * 4 : 0);
        const int per_sm = threads == 128 ? pgs_per_sm<128>() : pgs_per_sm<256>();
        if (per_sm < 1) return false;
        const int blocks = pgs_blocks;
        if (slab) {
            SlabArgs SA;
            SA.A = A;
            SA.pcstart = ws.s_pcstart.as<int>();
            SA.irowoff = ws.s_irowoff.as<int>();
            SA.irown = ws.s_irown.as<int>();
            SA.idesc = ws.s_idesc.as<int4>();
            SA.ipack = ws.s_ipack.as<float4>();
            SA.pbody = ws.s_pbody.as<int>();
            SA.pbcount = ws.s_pbcount.as<int>();
            SA.bcap = caps.bcap; SA.rcap = caps.rcap; SA.gcap = caps.gcap;
            SA.chunk_cap = GB_SLAB_XCHUNK;
            SA.ipasses = P.pgs_two_level;
            SA.xspatial = xspatial ? 1 : 0;
            SA.xcnt = ws.x_cnt.as<int>();
            SA.xadj = ws.x_adj.as<unsigned>();
            SA.xprog = ws.x_prog.as<unsigned>();
            SA.split = nsplit;
            SA.dstride = nsplit > 0 ? nsplit : 1;
            SA.dacc = ws.x_dacc.as<long long>();
            SA.smask = ws.x_smask.as<int>();
            void *args[] = {(void *)&SA};
            const void *k = threads == 128 ? (const void *)k_pgs_slab<128> : (const void *)k_pgs_slab<256>;
            if (cudaLaunchCooperativeKernel(k, blocks, threads, args, caps.smem, s) != cudaSuccess) return false;
        } else {
            void *args[] = {(void *)&A};
            const void *k = threads == 128 ? (const void *)k_pgs<128> : (const void *)k_pgs<256>;
            if (cudaLaunchCooperativeKernel(k, blocks, threads, args, smem, s) != cudaSuccess) return false;
        }
    }
    if (ev1) cudaEventRecord(ev1, s);
    if (P.warm_mode) warm_store(ws, s);
    if (P.warm_mode && ws.njoints > 0) {
        k_joint_store<<<grid_for(ws.njoints, 128), 128, 0, s>>>(joint_view(ws), rows_view(ws), ws.dc);
        count_launch();
    }
    k_integrate<<<grid_for(nb, 128), 128, 0, s>>>(bodies_view(ws, nb), P);
    count_launch(10);
    return cudaGetLastError() == cudaSuccess;
}

bool launch_quickstep_islands(Workspace &ws, int nb, const SolverParams &P, const IslandSchedule &sch, cudaStream_t s,
                              cudaEvent_t ev0, cudaEvent_t ev1) {
    // the island schedule's buffers first: nothing has run if one cannot be allocated
    int nisl = (int)sch.start.size() - 1;
    if (nisl > 0) {
        size_t no = sch.order.size() > 0 ? sch.order.size() : 1;
        if (!(ws.i_order.ensure(no * 4) && ws.i_start.ensure((nisl + 1) * 4) &&
              ws.i_bodies.ensure((sch.bodies.size() + 1) * 4) && ws.i_bstart.ensure((nisl + 1) * 4)))
            return false;
    }
    if (!assemble(ws, nb, P, s)) return false;
    if (nisl > 0) {
        if (!sch.order.empty()) cudaMemcpyAsync(ws.i_order.p, sch.order.data(), sch.order.size() * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ws.i_start.p, sch.start.data(), (nisl + 1) * 4, cudaMemcpyHostToDevice, s);
        if (!sch.bodies.empty()) cudaMemcpyAsync(ws.i_bodies.p, sch.bodies.data(), sch.bodies.size() * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ws.i_bstart.p, sch.bstart.data(), (nisl + 1) * 4, cudaMemcpyHostToDevice, s);
    }
    cudaMemsetAsync(&ws.dc->iterations, 0, 4, s);
    if (ev0) cudaEventRecord(ev0, s);
    if (nisl > 0) {
        IslandArgs A;
        A.Rw = rows_view(ws);
        A.fc = ws.b_fc.as<float4>();
        A.fa = ws.b_fa.as<float>();
        A.order = ws.i_order.as<int>(); A.start = ws.i_start.as<int>();
        A.bodies = ws.i_bodies.as<int>(); A.bstart = ws.i_bstart.as<int>();
        A.iterations = P.iterations;
        A.max_extra = (unsigned)((float)P.iterations * P.extra_factor);
        A.premature = P.premature_delta;
        A.extra_delta = P.extra_delta;
        A.dyn = (A.max_extra != 0 || A.premature != 0) ? 1 : 0;
        A.dc = ws.dc;
        k_islands<<<nisl, 32, 0, s>>>(A);
        count_launch();
    }
    if (ev1) cudaEventRecord(ev1, s);
    k_integrate<<<grid_for(nb, 128), 128, 0, s>>>(bodies_view(ws, nb), P);
    count_launch();
    // (the reference-order schedule's host vectors are copied before return)
    cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess;
}

double last_residual(Workspace &ws, int nb, double *compl_err, double *maxlam, cudaStream_t s) {
    if (!(ws.res_f.ensure((size_t)(nb > 0 ? nb : 1) * 48) && ws.res_v.ensure((size_t)(nb > 0 ? nb : 1) * 48 + 64))) {
        report_error("gbodeWorldLastResidual: device allocation");
        if (compl_err) *compl_err = NAN;
        if (maxlam) *maxlam = NAN;
        return NAN;
    }
    cudaMemsetAsync(ws.res_f.p, 0, (size_t)(nb > 0 ? nb : 1) * 48, s);
    double *out = (double *)((char *)ws.res_v.p + (size_t)(nb > 0 ? nb : 1) * 48);
    cudaMemsetAsync(out, 0, 24, s);
    int grid = 4 * num_sms();
    Rows R = rows_view(ws);
    Bodies B = bodies_view(ws, nb);
    k_res_force<<<grid, 256, 0, s>>>(R, &ws.dc->nrows, ws.res_f.as<double>());
    k_res_vel<<<grid_for(nb, 128), 128, 0, s>>>(B, ws.res_f.as<double>(), ws.res_v.as<double>());
    k_res_rows<<<grid, 256, 0, s>>>(R, B, &ws.dc->nrows, ws.res_v.as<double>(), out);
    count_launch(3);
    double h[3] = {0, 0, 0};
    cudaMemcpyAsync(h, out, 24, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (compl_err) *compl_err = h[1];
    if (maxlam) *maxlam = h[2];
    return h[0];
}

// Learned-warm-start training samples of the last step (syncs): per contact
// [12 features][s][lambda of its 3 rows after the solve][1 if a triplet]
int learn_samples(Workspace &ws, float *out, int cap, cudaStream_t s) {
    int n = 0;
    cudaMemcpyAsync(&n, ws.use_awake ? &ws.dc->nawake : &ws.dc->step_contacts, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    if (!out || cap <= 0 || n <= 0 || !ws.l_feat.p) return ws.l_feat.p ? n : 0;
    const int k = n < cap ? n : cap;
    std::vector<float> feat((size_t)k * GB_MLP_IN), sc(k), lam;
    std::vector<int> rstart(k), mcount(k), fi;
    cudaMemcpyAsync(feat.data(), ws.l_feat.p, feat.size() * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(sc.data(), ws.l_scale.p, (size_t)k * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(rstart.data(), ws.c_rstart.p, (size_t)k * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(mcount.data(), ws.c_mcount.p, (size_t)k * 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    const int nr = rstart[k - 1] + mcount[k - 1];
    lam.resize(nr);
    fi.resize(nr);
    cudaMemcpyAsync(lam.data(), ws.r_lambda.p, (size_t)nr * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(fi.data(), ws.r_findex.p, (size_t)nr * 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    for (int c = 0; c < k; c++) {
        float *o = out + (size_t)c * 17;
        for (int q = 0; q < GB_MLP_IN; q++) o[q] = feat[(size_t)c * GB_MLP_IN + q];
        o[12] = sc[c];
        const int r0 = rstart[c], m = mcount[c];
        for (int q = 0; q < 3; q++) o[13 + q] = q < m ? lam[r0 + q] : 0.f;
        o[16] = (m == 3 && fi[r0] < 0 && fi[r0 + 1] == r0 && fi[r0 + 2] == r0) ? 1.f : 0.f;
    }
    return k;
}

int copy_last_rows(Workspace &ws, float *rows, int cap, cudaStream_t s) {
    int n = 0;
    cudaMemcpyAsync(&n, &ws.dc->nrows, 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (!rows || cap <= 0 || n <= 0) return n;
    int k = n < cap ? n : cap;
    std::vector<float4> J1l(k), J1a(k), J2l(k), J2a(k);
    std::vector<float> lam(k), Ad(k);
    std::vector<int> fi(k);
    std::vector<int2> bd(k);
    cudaMemcpyAsync(J1l.data(), ws.r_J1l.p, k * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(J1a.data(), ws.r_J1a.p, k * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(J2l.data(), ws.r_J2l.p, k * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(J2a.data(), ws.r_J2a.p, k * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(lam.data(), ws.r_lambda.p, k * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(Ad.data(), ws.r_Ad.p, k * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(fi.data(), ws.r_findex.p, k * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(bd.data(), ws.r_body.p, k * 8, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int i = 0; i < k; i++) {
        float *o = rows + 20 * i;
        float ad = Ad[i];
        o[0] = J1l[i].x / ad; o[1] = J1l[i].y / ad; o[2] = J1l[i].z / ad;
        o[3] = J1a[i].x / ad; o[4] = J1a[i].y / ad; o[5] = J1a[i].z / ad;
        bool two = bd[i].y >= 0;
        o[6] = two ? J2l[i].x / ad : 0; o[7] = two ? J2l[i].y / ad : 0; o[8] = two ? J2l[i].z / ad : 0;
        o[9] = two ? J2a[i].x / ad : 0; o[10] = two ? J2a[i].y / ad : 0; o[11] = two ? J2a[i].z / ad : 0;
        o[12] = J1l[i].w / ad; o[13] = J1a[i].w / ad; o[14] = J2l[i].w; o[15] = J2a[i].w;
        o[16] = (float)bd[i].x; o[17] = (float)bd[i].y; o[18] = (float)fi[i]; o[19] = lam[i];
    }
    return n;
}

void joint_feedback(Workspace &ws, int ncontacts, int njoints, std::vector<float> &out, cudaStream_t s) {
    const size_t nrec = (size_t)ncontacts + (size_t)njoints;
    out.assign(nrec * 16, 0.f);
    if (nrec == 0) return;
    DBuf &tmp = ws.res_f;
    if (!tmp.ensure(nrec * 64)) {  // feedback left at zero, the error reported
        report_error("joint feedback: device allocation");
        return;
    }
    cudaMemsetAsync(tmp.p, 0, nrec * 64, s);
    k_feedback<<<4 * num_sms(), 256, 0, s>>>(rows_view(ws), &ws.dc->nrows, ws.use_awake ? ws.c_orig.as<int>() : nullptr,
                                             ncontacts, tmp.as<float>());
    count_launch();
    cudaMemcpyAsync(out.data(), tmp.p, nrec * 64, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
}

}  // namespace gb
