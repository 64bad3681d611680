// Device-side layouts and helpers shared by the gbode kernels.
//
// All kernels are compiled with -fmad=false, -prec-div=true and
// -prec-sqrt=true so that every float expression rounds exactly as the
// reference's dSINGLE build does on the CPU (ODE computes in plain IEEE float
// with separate multiplies and adds); that is what lets contact counts,
// feature codes and reference-order lambdas agree bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {

// ------------------------------------------------------------------ layouts
// Bodies (structure of arrays, one float4 per quantity, capacity nb_cap):
//   pos   xyz, w = inverse mass          q     w x y z (ODE order)
//   R     3 float4 rows per body (3x4 row-major, ODE dMatrix3)
//   lvel  xyz, w = mass                  avel  xyz, w = flags (bit0 gyroscopic)
//   facc, tacc                           accumulated force / torque
//   Ib, invIb   body-frame inertia and its inverse (3 rows each)
//   invIw       world-frame inverse inertia of the current step (3 rows)
//   fc          2 float4 per body: M^-1 J^T lambda (linear, angular)
//   rt          2 float4 per body: -(M^-1 f_ext + v/h) (quickstep.cpp:1644-1690)
struct Bodies {
    float4 *pos, *q, *R, *lvel, *avel, *facc, *tacc, *Ib, *invIb, *invIw, *fc, *rt;
    float4 *damp;  // linear scale, angular scale, squared thresholds (scale 0: no damping)
    float *maxw;   // angular speed cap (infinity: none)
    const int *asleep;  // 1: the body's component sleeps this step (null: sleeping off)
    int n;
};

// Geoms: class, owning body (-1 static), dims (sphere r | box lx ly lz |
// capsule r len | plane a b c d (normalised)), static pose, posed copy.
struct Geoms {
    int *cls, *body;
    float4 *dims, *spos, *sR;  // static pose (sR: 3 rows)
    float4 *gpos, *gR;         // pose of this step (gR: 3 rows)
    float4 *amin, *amax;       // AABB of this step
    int *level;                // hash level, or INT_MAX for the big-box list
    int4 *dblo, *dbhi;         // discretised bounds at the geom's level
    int n;
};

// Contact record (48 B): the dContactGeom fields the joint needs plus the
// attached bodies (before dJointAttach's swap), the surface it uses and the
// (geom pair, slot) key of the warm-start cache.
struct Contact {
    float4 pos_depth;   // pos xyz, depth
    float4 normal;      // xyz
    int b1, b2, surf, slot;
    int g1, g2, pad0, pad1;
};

// dSurfaceParameters + fdir1 (contact.h:55-103), padded to 80 B.
struct Surface {
    int mode;
    float mu, mu2, rho, rho2, rhoN, bounce, bounce_vel, soft_erp, soft_cfm;
    float motion1, motion2, motionN, slip1, slip2;
    float fdir1[3];
    float pad[2];
};

// Constraint rows (structure of arrays, capacity m_cap). J rows are scaled by
// Ad after assembly exactly as quickstep.cpp:2251-2316 does:
//   J1l (xyz, rhs)  J1a (xyz, cfm)  J2l (xyz, lo)  J2a (xyz, hi)
//   M1l (invM J1 linear, w = max|iMJ1|)  M1a  M2l (w = max|iMJ2|)  M2a
//   lambda, findex (global row index or -1), body (b1, b2; b2 = -1 for none),
//   Ad (scale factor, for unscaling in the residual), contact (owner)
struct Rows {
    float4 *J1l, *J1a, *J2l, *J2a, *M1l, *M1a, *M2l, *M2a;
    float *lambda, *Ad;
    int *findex, *contact;
    int2 *body;
    int n_cap;
};

// Error word bits reported back to the host.
enum : unsigned {
    ERR_BARRIER_TIMEOUT = 1u,
    ERR_PAIR_OVERFLOW = 2u,
    ERR_CONTACT_OVERFLOW = 4u,
    ERR_ROW_OVERFLOW = 8u,
    ERR_COLOUR_OVERFLOW = 16u,
    ERR_HASH_OVERFLOW = 32u,
    ERR_CELL_RANGE = 64u,
    ERR_NONFINITE = 128u,
    ERR_STAGE_TIMEOUT = 256u,  // a shared-memory staging copy did not complete in time
    ERR_ISLAND_LIMIT = 512u,   // a union-find merge did not settle within the body count
    ERR_LCP_FAILED = 1024u,    // the dense LCP solve of an island did not finish (its multipliers are zero)
};

#if defined(__CUDACC__)
// ------------------------------------------------------------------ math
// Restatements of include/ode/odemath.h:210-420 with the same operand order.
__device__ __forceinline__ float dot3(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ float dot3v(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ------------------------------------------------------------------ grid barrier
// An arrival-counter barrier for cooperative launches (all blocks
// co-resident).  Every block adds 1 to one counter with release semantics
// (after a block-wide __syncthreads, so the whole block's writes are
// released) and polls it with acquire loads until it reaches the running
// target, gridDim.x more than at the previous barrier; the counter is never
// reset within a launch, so the last arrival is itself the release and no
// block has to write a second word.  Every wait is bounded: after 2^22 polls
// the block records ERR_BARRIER_TIMEOUT in *err and returns false, pollers
// give up when they see that bit, and a block that gave up returns false from
// every later barrier without touching memory, so a kernel whose barrier can
// no longer complete still exits.  `gen` (per block, kept by the caller)
// starts at 0; the counter block must be zeroed before the launch.
struct GridSync {
    unsigned int count;
    unsigned int gen;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool grid_sync(GridSync *gs, unsigned *err, unsigned &gen) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 0;
        if (!(gen & 0x80000000u)) {
            const unsigned target = gen + gridDim.x;
            red_release_add_u32(&gs->count, 1u);
            ok = 1;
            long long polls = 0;
            while ((int)(ld_acquire_u32(&gs->count) - target) < 0) {
                if (++polls > (1ll << 22) || ((polls & 63) == 0 && (ld_acquire_u32(err) & ERR_BARRIER_TIMEOUT))) {
                    atomicOr(err, ERR_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
            gen = ok ? target : (gen | 0x80000000u);
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// The same barrier in two halves: grid_arrive (block-wide __syncthreads, then
// thread 0's release-add) and grid_wait (thread 0 polls, bounded as above;
// then __syncthreads).  Work placed between them -- stores no other block
// reads before a later barrier -- overlaps the wait instead of delaying the
// release.  `target` carries the arrival's count from one half to the other.
__device__ __forceinline__ void grid_arrive(GridSync *gs, unsigned &gen, unsigned &target) {
    __syncthreads();
    if (threadIdx.x == 0 && !(gen & 0x80000000u)) {
        target = gen + gridDim.x;
        red_release_add_u32(&gs->count, 1u);
    }
}
__device__ __forceinline__ bool grid_wait(GridSync *gs, unsigned *err, unsigned &gen, unsigned target) {
    __shared__ int ok_w;
    if (threadIdx.x == 0) {
        int ok = 0;
        if (!(gen & 0x80000000u)) {
            ok = 1;
            long long polls = 0;
            while ((int)(ld_acquire_u32(&gs->count) - target) < 0) {
                if (++polls > (1ll << 22) || ((polls & 63) == 0 && (ld_acquire_u32(err) & ERR_BARRIER_TIMEOUT))) {
                    atomicOr(err, ERR_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
            gen = ok ? target : (gen | 0x80000000u);
        }
        ok_w = ok;
    }
    __syncthreads();
    return ok_w != 0;
}

// Cache-global (L2) loads and stores for data that other SMs rewrite between
// grid barriers (L1 is not coherent across SMs).
__device__ __forceinline__ float4 ldcg4(const float4 *p) { return __ldcg(p); }
__device__ __forceinline__ void stcg4(float4 *p, float4 v) { __stcg(p, v); }
#else
struct GridSync {
    unsigned int count;
    unsigned int gen;
};
#endif

}  // namespace gb
