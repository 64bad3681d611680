// dWorldStep's constraint solve on the device: one dense mixed LCP per island
// (step.cpp:892-1200 forms A = J M^-1 J^T + diag(cfm), b = rhs; lcp.cpp:836-
// 1160 solves it with Dantzig's principal pivoting), in FP64, one thread block
// per island.
//
// The reference's solver treats friction rows (findex >= 0) after every other
// row: it first solves the problem with the friction rows held at zero, then
// fixes each friction row's bounds at +-|mu * lambda_normal| from that
// solution (0 when the normal multiplier is 0) and continues with all rows
// (lcp.cpp:889-917; the permutation of lcp.cpp:520-533 moves findex rows to
// the end).  With cfm > 0 the matrix is positive definite, and a box-
// constrained LCP with a positive definite matrix has exactly one solution;
// so each of the two phases has a unique answer whatever pivoting sequence
// reaches it.  Here each phase is solved by block principal pivoting
// (Judice and Pires, 1994): every variable is free (w = 0), at its lower
// bound (w >= 0) or at its upper bound (w <= 0); the free set's equations are
// solved by an FP32 Cholesky factorisation with FP64 iterative refinement
// against the FP64 matrix, and the variables that violate their
// conditions all change sets at once while their number keeps falling,
// otherwise only the one with the smallest index (Murty's rule, finite for
// positive definite matrices).  Unbounded rows are always free; a row with
// lo = hi = 0 is fixed at 0.
//
// Memory per island (one device buffer): the FP64 matrix (m^2), per-row
// vectors, and the FP32 factor (m^2); the island's rows reach the kernel as a
// list of row indices.
#include "gbode_internal.h"

namespace gb {

enum : int { LCP_FREE = 0, LCP_LO = 1, LCP_HI = 2, LCP_FIXED = 3 };

struct DantzigArgs {
    Rows Rw;
    float4 *fc;              // per body: M^-1 J^T lambda (linear, angular), zeroed by the body pass
    const int *order;        // island rows, island by island
    const int *start;        // [nisl + 1]
    const long long *doff;   // per island: offset of its FP64 scratch
    const long long *ioff;   // per island: offset of its int scratch
    double *dscr;
    int *iscr;
    int *rloc;               // [row capacity]: row -> index in its island
    DevCounters *dc;
    int max_iter;  // unused (the limit depends on the island's size)
};

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += red[k];
    __syncthreads();
    return s;
}
__device__ __forceinline__ double block_max(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s = fmax(s, red[k]);
    __syncthreads();
    return s;
}

// In-place Cholesky (lower triangle) of the n x n matrix C (row-major, leading
// dimension n), in FP32: FP64 arithmetic runs at a small fraction of FP32's
// rate on this GPU, and the FP64 refinement of the solve below recovers the
// digits.  Blocked right-looking, 32-column panels: the diagonal block is
// factored in shared memory, the panel below it solved row by row, and the
// trailing lower triangle updated tile by tile (32 x 32), one tile per warp
// at a time -- lane a holds row a of the panel tile in registers, the warp's
// partner tile sits in shared memory -- so the trailing matrix is read once
// per panel instead of once per column.  Returns false on a non-positive pivot.
#define CH_TB 32
__device__ bool block_cholesky(float *C, int n, int *s_ok) {
    __shared__ float Dk[CH_TB][CH_TB + 1];
    __shared__ float Tj[8][CH_TB][CH_TB + 1];  // one partner tile per warp (256 threads)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int k0 = 0; k0 < n; k0 += CH_TB) {
        const int kb = min(CH_TB, n - k0);
        // 1. the diagonal block, factored in shared memory
        for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
            const int i = t / kb, j = t % kb;
            Dk[i][j] = C[(size_t)(k0 + i) * n + k0 + j];
        }
        __syncthreads();
        for (int k = 0; k < kb; k++) {
            if (threadIdx.x == 0) {
                const float d = Dk[k][k];
                *s_ok = d > 0.f;
                Dk[k][k] = d > 0.f ? sqrtf(d) : 1.f;
            }
            __syncthreads();
            if (!*s_ok) return false;
            for (int i = k + 1 + threadIdx.x; i < kb; i += blockDim.x) Dk[i][k] /= Dk[k][k];
            __syncthreads();
            for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
                const int i = t / kb, j = t % kb;
                if (i > k && j > k && j <= i) Dk[i][j] -= Dk[i][k] * Dk[j][k];
            }
            __syncthreads();
        }
        for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
            const int i = t / kb, j = t % kb;
            if (j <= i) C[(size_t)(k0 + i) * n + k0 + j] = Dk[i][j];
        }
        // 2. the panel below: L_rk = A_rk L_kk^-T, one row per thread
        const int r0 = k0 + kb;
        for (int r = r0 + threadIdx.x; r < n; r += blockDim.x) {
            float *row = C + (size_t)r * n + k0;
            for (int j = 0; j < kb; j++) {
                float v = row[j];
                for (int m = 0; m < j; m++) v -= row[m] * Dk[j][m];
                row[j] = v / Dk[j][j];
            }
        }
        __syncthreads();
        // 3. the trailing lower triangle, tile pairs (I, J <= I), one per warp
        const int nt = (n - r0 + CH_TB - 1) / CH_TB;
        const int npairs = nt * (nt + 1) / 2;
        for (int p = warp; p < npairs; p += nwarps) {
            int I = (int)((sqrtf(8.f * (float)p + 1.f) - 1.f) * 0.5f);
            while ((I + 1) * (I + 2) / 2 <= p) I++;
            while (I * (I + 1) / 2 > p) I--;
            const int J = p - I * (I + 1) / 2;
            const int i0 = r0 + I * CH_TB, j0 = r0 + J * CH_TB;
            const int ib = min(CH_TB, n - i0), jb = min(CH_TB, n - j0);
            // partner tile rows (j0 + b) of the panel into shared memory
            for (int b = 0; b < jb; b++)
                Tj[warp][b][lane] = lane < kb ? C[(size_t)(j0 + b) * n + k0 + lane] : 0.f;
            __syncwarp();
            if (lane < ib) {
                float ti[CH_TB];
                const float *ri = C + (size_t)(i0 + lane) * n + k0;
#pragma unroll
                for (int m = 0; m < CH_TB; m++) ti[m] = m < kb ? ri[m] : 0.f;
                float *out = C + (size_t)(i0 + lane) * n + j0;
                for (int b = 0; b < jb; b++) {
                    if (j0 + b > i0 + lane) break;  // lower triangle only
                    float acc = 0.f;
#pragma unroll
                    for (int m = 0; m < CH_TB; m++) acc += ti[m] * Tj[warp][b][m];
                    out[b] -= acc;
                }
            }
            __syncwarp();
        }
        __syncthreads();
    }
    return true;
}

// Solve (L L^T) z = z in place, L from block_cholesky.
__device__ void block_chol_solve(const float *C, int n, float *z) {
    for (int k = 0; k < n; k++) {
        if (threadIdx.x == 0) z[k] /= C[(size_t)k * n + k];
        __syncthreads();
        const float zk = z[k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) z[i] -= C[(size_t)i * n + k] * zk;
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; k--) {
        if (threadIdx.x == 0) z[k] /= C[(size_t)k * n + k];
        __syncthreads();
        const float zk = z[k];
        for (int i = threadIdx.x; i < k; i += blockDim.x) z[i] -= C[(size_t)k * n + i] * zk;
        __syncthreads();
    }
}

// One box-constrained LCP phase by block principal pivoting (see the file
// comment).  st/x/lo/hi/A/b live in the island's scratch; returns false when
// the iteration limit is reached or a factorisation fails.
__device__ bool bpp_solve(const double *A, const double *b, const double *lo, const double *hi, double *x,
                          double *w, float *C, double *y, float *z, int *st, int *flist, int m, int max_iter,
                          double *red, int *s_int) {
    int best = 0x7fffffff, budget = 3;
    const double bscale = fmax(1.0, block_max([&] {
        double v = 0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) v = fmax(v, fabs(b[i]));
        return v;
    }(), red));
    for (int iter = 0; iter < max_iter; iter++) {
        // fixed values of the bounded sets; the free list
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (st[i] == LCP_LO) x[i] = lo[i];
            else if (st[i] == LCP_HI) x[i] = hi[i];
            else if (st[i] == LCP_FIXED) x[i] = 0.0;
        }
        if (threadIdx.x == 0) {
            int nf = 0;
            for (int i = 0; i < m; i++)
                if (st[i] == LCP_FREE) flist[nf++] = i;
            s_int[1] = nf;
        }
        __syncthreads();
        const int nf = s_int[1];
        // y_F = b_F - A_F,N x_N; C = A_F,F
        for (int a = threadIdx.x; a < nf; a += blockDim.x) {
            const int i = flist[a];
            double v = b[i];
            for (int j = 0; j < m; j++)
                if (st[j] != LCP_FREE) v -= A[(size_t)i * m + j] * x[j];
            y[a] = v;
        }
        for (long long t = threadIdx.x; t < (long long)nf * nf; t += blockDim.x) {
            const int a = (int)(t / nf), c = (int)(t % nf);
            C[(size_t)a * nf + c] = (float)A[(size_t)flist[a] * m + flist[c]];
        }
        for (int a = threadIdx.x; a < nf; a += blockDim.x) x[flist[a]] = 0.0;
        __syncthreads();
        if (nf > 0) {
            if (!block_cholesky(C, nf, &s_int[2])) return false;
            // x_F = A_FF^-1 y_F by FP32 solves refined against the FP64 matrix
            for (int refine = 0; refine < 4; refine++) {
                for (int a = threadIdx.x; a < nf; a += blockDim.x) {
                    const double *Ai = A + (size_t)flist[a] * m;
                    double r = y[a];
                    for (int c = 0; c < nf; c++) r -= Ai[flist[c]] * x[flist[c]];
                    z[a] = (float)r;
                }
                __syncthreads();
                block_chol_solve(C, nf, z);
                for (int a = threadIdx.x; a < nf; a += blockDim.x) x[flist[a]] += (double)z[a];
                __syncthreads();
            }
        }
        // w = A x - b and the violations
        double xs = 0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            double v = -b[i];
            for (int j = 0; j < m; j++) v += A[(size_t)i * m + j] * x[j];
            w[i] = v;
            xs = fmax(xs, fabs(x[i]));
        }
        const double xscale = fmax(1.0, block_max(xs, red));
        const double tx = 1e-11 * xscale, tw = 1e-11 * bscale;
        int nbad = 0, first = 0x7fffffff;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            bool bad = false;
            if (st[i] == LCP_FREE) bad = x[i] < lo[i] - tx || x[i] > hi[i] + tx;
            else if (st[i] == LCP_LO) bad = w[i] < -tw;
            else if (st[i] == LCP_HI) bad = w[i] > tw;
            if (bad) { nbad++; first = min(first, i); }
        }
        nbad = (int)block_sum((double)nbad, red);
        if (threadIdx.x == 0) s_int[3] = 0x7fffffff;
        __syncthreads();
        atomicMin(&s_int[3], first);
        __syncthreads();
        first = s_int[3];
        if (nbad == 0) return true;
        bool all;
        if (nbad < best) { best = nbad; budget = 3; all = true; }
        else if (budget > 0) { budget--; all = true; }
        else all = false;  // Murty: the smallest violating index only
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (!all && i != first) continue;
            if (st[i] == LCP_FREE) {
                if (x[i] < lo[i] - tx) st[i] = LCP_LO;
                else if (x[i] > hi[i] + tx) st[i] = LCP_HI;
            } else if (st[i] == LCP_LO) {
                if (w[i] < -tw) st[i] = LCP_FREE;
            } else if (st[i] == LCP_HI) {
                if (w[i] > tw) st[i] = LCP_FREE;
            }
        }
        __syncthreads();
    }
    return false;
}

__global__ void __launch_bounds__(256) k_dantzig(DantzigArgs P) {
    __shared__ double red[8];
    __shared__ int s_int[4];
    const int isl = blockIdx.x;
    const int r0 = P.start[isl], m = P.start[isl + 1] - r0;
    if (m <= 0) return;
    const int *R = P.order + r0;
    double *A = P.dscr + P.doff[isl];
    double *b = A + (size_t)m * m;
    double *lo = b + m, *hi = lo + m, *x = hi + m, *w = x + m, *y = w + m, *mu = y + m;
    double *Jm = mu + m;                 // per row: J1 (6), J2 (6), M1 (6), M2 (6)
    float *C = (float *)(Jm + (size_t)m * 24);  // m x m factor
    float *z = C + (size_t)m * m;        // m
    int *st = P.iscr + P.ioff[isl];
    int *flist = st + m, *fi = flist + m, *b1 = fi + m, *b2 = b1 + m;
    const Rows &Rw = P.Rw;
    for (int i = threadIdx.x; i < m; i += blockDim.x) P.rloc[R[i]] = i;
    __syncthreads();
    // unscaled rows (the assembly stores J, rhs and cfm multiplied by Ad)
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int r = R[i];
        const double ad = (double)Rw.Ad[r];
        const float4 j1l = Rw.J1l[r], j1a = Rw.J1a[r], j2l = Rw.J2l[r], j2a = Rw.J2a[r];
        const float4 m1l = Rw.M1l[r], m1a = Rw.M1a[r], m2l = Rw.M2l[r], m2a = Rw.M2a[r];
        const int2 bd = Rw.body[r];
        double *o = Jm + (size_t)i * 24;
        o[0] = j1l.x / ad; o[1] = j1l.y / ad; o[2] = j1l.z / ad; o[3] = j1a.x / ad; o[4] = j1a.y / ad; o[5] = j1a.z / ad;
        if (bd.y >= 0) {
            o[6] = j2l.x / ad; o[7] = j2l.y / ad; o[8] = j2l.z / ad; o[9] = j2a.x / ad; o[10] = j2a.y / ad; o[11] = j2a.z / ad;
        } else {
            for (int q = 6; q < 12; q++) o[q] = 0.0;
        }
        o[12] = m1l.x; o[13] = m1l.y; o[14] = m1l.z; o[15] = m1a.x; o[16] = m1a.y; o[17] = m1a.z;
        o[18] = m2l.x; o[19] = m2l.y; o[20] = m2l.z; o[21] = m2a.x; o[22] = m2a.y; o[23] = m2a.z;
        b[i] = (double)j1l.w / ad;
        mu[i] = (double)j2a.w;  // a friction row's coefficient (its hi before the bounds are fixed)
        lo[i] = (double)j2l.w;
        hi[i] = (double)j2a.w;
        const int f = Rw.findex[r];
        fi[i] = f >= 0 ? P.rloc[f] : -1;
        b1[i] = bd.x;
        b2[i] = bd.y;
        y[i] = (double)j1a.w / ad;  // cfm, moved onto the diagonal below
    }
    __syncthreads();
    // A = J M^-1 J^T + diag(cfm)  (step.cpp:1160-1300)
    for (long long t = threadIdx.x; t < (long long)m * m; t += blockDim.x) {
        const int i = (int)(t / m), j = (int)(t % m);
        const double *Ji = Jm + (size_t)i * 24, *Jj = Jm + (size_t)j * 24;
        double v = 0.0;
        if (b1[i] == b1[j]) for (int q = 0; q < 6; q++) v += Ji[q] * Jj[12 + q];
        if (b2[j] >= 0 && b1[i] == b2[j]) for (int q = 0; q < 6; q++) v += Ji[q] * Jj[18 + q];
        if (b2[i] >= 0 && b2[i] == b1[j]) for (int q = 0; q < 6; q++) v += Ji[6 + q] * Jj[12 + q];
        if (b2[i] >= 0 && b2[i] == b2[j]) for (int q = 0; q < 6; q++) v += Ji[6 + q] * Jj[18 + q];
        if (i == j) v += y[i];
        A[t] = v;
    }
    __syncthreads();
    // phase 1: friction rows held at zero
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        x[i] = 0.0;
        if (fi[i] >= 0) st[i] = LCP_FIXED;
        else if (lo[i] == 0.0 && hi[i] == 0.0) st[i] = LCP_FIXED;
        else st[i] = LCP_FREE;
    }
    __syncthreads();
    const int max_iter = m < 500 ? 64 + 4 * m : 2064;  // flips; Murty's single flips need at most a few per row
    bool ok = bpp_solve(A, b, lo, hi, x, w, C, y, z, st, flist, m, max_iter, red, s_int);
    // phase 2: friction bounds from the normal multipliers, every row
    if (ok) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (fi[i] < 0) continue;
            const double xn = x[fi[i]];
            if (xn == 0.0) { hi[i] = 0.0; lo[i] = 0.0; st[i] = LCP_FIXED; }
            else { hi[i] = fabs(mu[i] * xn); lo[i] = -hi[i]; st[i] = LCP_FREE; }
        }
        __syncthreads();
        ok = bpp_solve(A, b, lo, hi, x, w, C, y, z, st, flist, m, max_iter, red, s_int);
    }
    if (!ok && threadIdx.x == 0) atomicOr(&P.dc->err, ERR_LCP_FAILED);
    // multipliers, and fc = M^-1 J^T lambda accumulated in row order
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const double xi = ok ? fmin(fmax(x[i], lo[i]), hi[i]) : 0.0;
        x[i] = xi;
        Rw.lambda[R[i]] = (float)xi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < m; i++) {
            const float l = (float)x[i];
            if (l == 0.f) continue;
            const double *o = Jm + (size_t)i * 24;
            float4 *f1 = P.fc + 2 * b1[i];
            f1[0].x += l * (float)o[12]; f1[0].y += l * (float)o[13]; f1[0].z += l * (float)o[14];
            f1[1].x += l * (float)o[15]; f1[1].y += l * (float)o[16]; f1[1].z += l * (float)o[17];
            if (b2[i] >= 0) {
                float4 *f2 = P.fc + 2 * b2[i];
                f2[0].x += l * (float)o[18]; f2[0].y += l * (float)o[19]; f2[0].z += l * (float)o[20];
                f2[1].x += l * (float)o[21]; f2[1].y += l * (float)o[22]; f2[1].z += l * (float)o[23];
            }
        }
    }
}

// A batch of dense LCPs given directly (gbodeSolveLCPBatch): problem p's
// matrix at A + p n^2 (row-major), vectors at p n; the first nub variables
// unbounded; findex (optional, per problem) as in the reference's solver.
struct LcpBatchArgs {
    const double *A, *b, *lo, *hi;
    const int *findex;
    double *x, *w;
    double *dscr;  // per problem: n^2 / 2 (FP32 factor) + 6 n doubles
    int *iscr;     // per problem: 3 n
    int n, nub;
    unsigned *err;
};

__global__ void __launch_bounds__(256) k_lcp_batch(LcpBatchArgs P) {
    __shared__ double red[8];
    __shared__ int s_int[4];
    const int n = P.n;
    const size_t pn = (size_t)blockIdx.x * n;
    const double *A = P.A + pn * n;
    const double *b = P.b + pn;
    double *x = P.x + pn, *w = P.w + pn;
    double *D = P.dscr + (size_t)blockIdx.x * ((size_t)n * n / 2 + 1 + 6 * (size_t)n);
    double *lo = D, *hi = lo + n, *y = hi + n, *mu = y + n;
    float *C = (float *)(mu + n);
    float *z = C + (size_t)n * n;
    int *st = P.iscr + (size_t)blockIdx.x * 3 * n, *flist = st + n, *fi = flist + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        lo[i] = i < P.nub ? -INFINITY : P.lo[pn + i];
        hi[i] = i < P.nub ? INFINITY : P.hi[pn + i];
        mu[i] = hi[i];
        fi[i] = P.findex ? P.findex[pn + i] : -1;
        x[i] = 0.0;
        if (fi[i] >= 0 || (lo[i] == 0.0 && hi[i] == 0.0)) st[i] = LCP_FIXED;
        else st[i] = LCP_FREE;
    }
    __syncthreads();
    const int max_iter = n < 500 ? 64 + 4 * n : 2064;
    bool ok = bpp_solve(A, b, lo, hi, x, w, C, y, z, st, flist, n, max_iter, red, s_int);
    bool any_f = false;
    for (int i = 0; i < n; i++) any_f |= fi[i] >= 0;
    if (ok && any_f) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            if (fi[i] < 0) continue;
            const double xn = x[fi[i]];
            if (xn == 0.0) { hi[i] = 0.0; lo[i] = 0.0; st[i] = LCP_FIXED; }
            else { hi[i] = fabs(mu[i] * xn); lo[i] = -hi[i]; st[i] = LCP_FREE; }
        }
        __syncthreads();
        ok = bpp_solve(A, b, lo, hi, x, w, C, y, z, st, flist, n, max_iter, red, s_int);
    }
    if (!ok && threadIdx.x == 0) atomicOr(P.err, ERR_LCP_FAILED);
    // w = A x - b (bpp_solve leaves it for its final x)
    (void)w;
}

bool solve_lcp_batch(int count, int n, const double *A, const double *b, const double *lo, const double *hi,
                     int nub, const int *findex, double *x, double *w, cudaStream_t s) {
    const size_t nn = (size_t)n * n, np = (size_t)count * n;
    DBuf dA, dv, ds, di, derr;
    const size_t vec = np * 8;
    if (!(dA.ensure((size_t)count * nn * 8) && dv.ensure(6 * vec) && ds.ensure((size_t)count * (nn / 2 + 1 + 6 * (size_t)n) * 8) &&
          di.ensure((size_t)count * 3 * n * 4 + 4) && derr.ensure(4))) {
        dA.release(); dv.release(); ds.release(); di.release(); derr.release();
        return false;
    }
    double *vb = dv.as<double>(), *vlo = vb + np, *vhi = vlo + np, *vx = vhi + np, *vw = vx + np;
    int *vf = (int *)(vw + np);
    cudaMemcpyAsync(dA.p, A, (size_t)count * nn * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(vb, b, vec, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(vlo, lo, vec, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(vhi, hi, vec, cudaMemcpyHostToDevice, s);
    if (findex) cudaMemcpyAsync(vf, findex, np * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(derr.p, 0, 4, s);
    LcpBatchArgs P;
    P.A = dA.as<double>(); P.b = vb; P.lo = vlo; P.hi = vhi; P.findex = findex ? vf : nullptr;
    P.x = vx; P.w = vw; P.dscr = ds.as<double>(); P.iscr = di.as<int>(); P.n = n; P.nub = nub;
    P.err = derr.as<unsigned>();
    k_lcp_batch<<<count, 256, 0, s>>>(P);
    count_launch();
    unsigned err = 0;
    cudaMemcpyAsync(x, vx, vec, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(w, vw, vec, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&err, derr.p, 4, cudaMemcpyDeviceToHost, s);
    const bool ok = cudaStreamSynchronize(s) == cudaSuccess && err == 0;
    dA.release(); dv.release(); ds.release(); di.release(); derr.release();
    return ok;
}

bool launch_dantzig(Workspace &ws, const std::vector<int> &order, const std::vector<int> &start, cudaStream_t s) {
    const int nisl = (int)start.size() - 1;
    if (nisl <= 0) return true;
    std::vector<long long> doff(nisl), ioff(nisl);
    long long dt = 0, it = 0;
    for (int i = 0; i < nisl; i++) {
        const long long m = start[i + 1] - start[i];
        if (m > GB_DANTZIG_MAX_ROWS) {
            report_error("dWorldStep: an island has more rows than the dense solver takes");
            return false;
        }
        doff[i] = dt;
        ioff[i] = it;
        dt += m * m + 31 * m + (m * m + m + 1) / 2;  // FP64 matrix and vectors, then the FP32 factor and z
        it += 5 * m;
    }
    const size_t no = order.empty() ? 1 : order.size();
    if (!(ws.i_order.ensure(no * 4) && ws.i_start.ensure((size_t)(nisl + 1) * 4) && ws.d_off.ensure((size_t)nisl * 16) &&
          ws.d_scr.ensure((size_t)(dt > 0 ? dt : 1) * 8) && ws.d_iscr.ensure((size_t)(it > 0 ? it : 1) * 4) &&
          ws.d_rloc.ensure((size_t)(ws.row_cap > 0 ? ws.row_cap : 1) * 4)))
        return false;
    long long *off = ws.d_off.as<long long>();
    if (!order.empty()) cudaMemcpyAsync(ws.i_order.p, order.data(), order.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.i_start.p, start.data(), (size_t)(nisl + 1) * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(off, doff.data(), (size_t)nisl * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(off + nisl, ioff.data(), (size_t)nisl * 8, cudaMemcpyHostToDevice, s);
    DantzigArgs P;
    P.Rw = rows_view_public(ws);
    P.fc = ws.b_fc.as<float4>();
    P.order = ws.i_order.as<int>();
    P.start = ws.i_start.as<int>();
    P.doff = off;
    P.ioff = off + nisl;
    P.dscr = ws.d_scr.as<double>();
    P.iscr = ws.d_iscr.as<int>();
    P.rloc = ws.d_rloc.as<int>();
    P.dc = ws.dc;
    P.max_iter = 0;  // per island: see k_dantzig
    k_dantzig<<<nisl, 256, 0, s>>>(P);
    count_launch();
    // the host vectors above are read by the copies: finish them before return
    return cudaStreamSynchronize(s) == cudaSuccess;
}

}  // namespace gb
