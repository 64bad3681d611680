// Collision pipeline on the device: geom posing + AABBs, the multi-level
// hash-grid broad phase, the narrow phase and contact compaction.
//
// Broad phase.  The reference's dHashSpace (collision_space.cpp:421-614)
// reports every pair of geoms whose AABBs overlap (after the same-body and
// category filters of collideAABBs, collision_space_internal.h:44-80); its
// cell hierarchy only accelerates the search, and the order of the pairs it
// reports follows its hash-table layout.  This broad phase keeps the
// semantics -- the same set of pairs, with the same level rule (findLevel,
// :329-349: level = frexp exponent of the largest AABB side, clamped below by
// the space's minlevel; AABBs above maxlevel or unbounded go to a separate
// list tested against everything) -- and replaces the sequential search with
// a GPU-friendly one: each geom inserts its <= 8 cells into an open-addressed
// device hash table, then queries its own and every coarser level.  A pair is
// emitted once, by the finer geom (by the lower index at equal levels), in the
// single cell that holds the low corner of the two geoms' discretised overlap,
// so no n*n "tested" bitmap is needed.  Output order is deterministic: pairs
// grouped by first geom, partners ascending.
#include <math.h>

#include "colliders.cuh"
#include "gbode_internal.h"
#include "../../include/gbode.h"

namespace gb {

static constexpr unsigned long long EMPTY_KEY = ~0ull;
static constexpr int BIG_LEVEL = 0x7fffffff;

__device__ __forceinline__ unsigned long long cell_key(int level, int x, int y, int z) {
    return ((unsigned long long)(unsigned)(level + 64) << 57) | ((unsigned long long)((unsigned)x & 0x7FFFFu) << 38) |
           ((unsigned long long)((unsigned)y & 0x7FFFFu) << 19) | (unsigned long long)((unsigned)z & 0x7FFFFu);
}
__device__ __forceinline__ unsigned hash64(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return (unsigned)k;
}

// ------------------------------------------------------------------ pose + AABB
// box.cpp:60-77, sphere.cpp:59-67, capsule.cpp:60-74, plane.cpp:80-105
__global__ void k_pose_aabb(Geoms G, Bodies B, int minlevel, int maxlevel, int *big_list, DevCounters *dc) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G.n) return;
    int cls = G.cls[g], body = G.body[g];
    float4 d = G.dims[g];
    float pos[3], R[12];
    if (body >= 0) {
        float4 p = B.pos[body];
        pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
        for (int r = 0; r < 3; r++) { float4 rr = B.R[3 * body + r]; R[4 * r] = rr.x; R[4 * r + 1] = rr.y; R[4 * r + 2] = rr.z; R[4 * r + 3] = 0; }
    } else {
        float4 p = G.spos[g];
        pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
        for (int r = 0; r < 3; r++) { float4 rr = G.sR[3 * g + r]; R[4 * r] = rr.x; R[4 * r + 1] = rr.y; R[4 * r + 2] = rr.z; R[4 * r + 3] = 0; }
    }
    G.gpos[g] = make_float4(pos[0], pos[1], pos[2], 0.f);
    for (int r = 0; r < 3; r++) G.gR[3 * g + r] = make_float4(R[4 * r], R[4 * r + 1], R[4 * r + 2], 0.f);
    float a[6];
    if (cls == 0) {
        a[0] = pos[0] - d.x; a[1] = pos[0] + d.x; a[2] = pos[1] - d.x; a[3] = pos[1] + d.x; a[4] = pos[2] - d.x; a[5] = pos[2] + d.x;
    } else if (cls == 1) {
        float xr = 0.5f * (fabsf(R[0] * d.x) + fabsf(R[1] * d.y) + fabsf(R[2] * d.z));
        float yr = 0.5f * (fabsf(R[4] * d.x) + fabsf(R[5] * d.y) + fabsf(R[6] * d.z));
        float zr = 0.5f * (fabsf(R[8] * d.x) + fabsf(R[9] * d.y) + fabsf(R[10] * d.z));
        a[0] = pos[0] - xr; a[1] = pos[0] + xr; a[2] = pos[1] - yr; a[3] = pos[1] + yr; a[4] = pos[2] - zr; a[5] = pos[2] + zr;
    } else if (cls == 2) {
        float xr = fabsf(R[2] * d.y) * 0.5f + d.x;
        float yr = fabsf(R[6] * d.y) * 0.5f + d.x;
        float zr = fabsf(R[10] * d.y) * 0.5f + d.x;
        a[0] = pos[0] - xr; a[1] = pos[0] + xr; a[2] = pos[1] - yr; a[3] = pos[1] + yr; a[4] = pos[2] - zr; a[5] = pos[2] + zr;
    } else {
        for (int i = 0; i < 6; i++) a[i] = (i & 1) ? INFINITY : -INFINITY;
        if (cls == 4) {
            if (d.y == 0.0f && d.z == 0.0f) { a[0] = (d.x > 0) ? -INFINITY : -d.w; a[1] = (d.x > 0) ? d.w : INFINITY; }
            else if (d.x == 0.0f && d.z == 0.0f) { a[2] = (d.y > 0) ? -INFINITY : -d.w; a[3] = (d.y > 0) ? d.w : INFINITY; }
            else if (d.x == 0.0f && d.y == 0.0f) { a[4] = (d.z > 0) ? -INFINITY : -d.w; a[5] = (d.z > 0) ? d.w : INFINITY; }
        }
    }
    G.amin[g] = make_float4(a[0], a[2], a[4], 0.f);
    G.amax[g] = make_float4(a[1], a[3], a[5], 0.f);
    // findLevel (collision_space.cpp:329-349) and the level clamp (:451-453)
    int level;
    bool inf = a[0] <= -INFINITY || a[1] >= INFINITY || a[2] <= -INFINITY || a[3] >= INFINITY || a[4] <= -INFINITY ||
               a[5] >= INFINITY;
    if (inf) level = BIG_LEVEL;
    else {
        float q = a[1] - a[0], q2 = a[3] - a[2];
        if (q2 > q) q = q2;
        q2 = a[5] - a[4];
        if (q2 > q) q = q2;
        frexpf(q, &level);
        if (level < minlevel) level = minlevel;
        if (level > maxlevel) level = BIG_LEVEL;
    }
    G.level[g] = level;
    if (level == BIG_LEVEL) {
        int k = atomicAdd(&dc->nbig, 1);
        big_list[k] = g;
    } else {
        atomicMax(&dc->maxlevel, level);
        float csr = ldexpf(1.0f, -level);
        int db[6];
        for (int i = 0; i < 6; i++) {
            float v = floorf(a[i] * csr);
            if (!(v > -262144.0f && v < 262143.0f)) { atomicOr(&dc->err, ERR_CELL_RANGE); v = 0.f; }
            db[i] = (int)v;
        }
        G.dblo[g] = make_int4(db[0], db[2], db[4], 0);
        G.dbhi[g] = make_int4(db[1], db[3], db[5], 0);
    }
}

// ------------------------------------------------------------------ hash grid
__global__ void k_bp_insert(Geoms G, unsigned long long *keys, unsigned mask, int *count, int *entry, DevCounters *dc) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G.n) return;
    int level = G.level[g];
    for (int k = 0; k < 8; k++) entry[8 * g + k] = -1;
    if (level == BIG_LEVEL) return;
    int4 lo = G.dblo[g], hi = G.dbhi[g];
    int k = 0;
    for (int x = lo.x; x <= hi.x; x++)
        for (int y = lo.y; y <= hi.y; y++)
            for (int z = lo.z; z <= hi.z; z++) {
                if (k >= 8) { atomicOr(&dc->err, ERR_CELL_RANGE); return; }
                unsigned long long key = cell_key(level, x, y, z);
                unsigned h = hash64(key) & mask;
                int slot = -1;
                for (unsigned probe = 0; probe <= mask; probe++) {
                    unsigned long long prev = atomicCAS(&keys[h], EMPTY_KEY, key);
                    if (prev == EMPTY_KEY || prev == key) { slot = (int)h; break; }
                    h = (h + 1) & mask;
                }
                if (slot < 0) { atomicOr(&dc->err, ERR_HASH_OVERFLOW); return; }
                atomicAdd(&count[slot], 1);
                entry[8 * g + k++] = slot;
            }
}

__global__ void k_bp_fill(int ng, const int *entry, const int *start, int *fill, int *members) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 8 * ng) return;
    int slot = entry[e];
    if (slot < 0) return;
    int pos = start[slot] + atomicAdd(&fill[slot], 1);
    members[pos] = e >> 3;
}

// The reference hashes a cell as (level*1000 + x*100 + y*10 + zbegin) % size
// with level, x, y as unsigned int and zbegin the int z at which a box starts
// its column (collision_space.cpp:358-361, :497-499, :545-547), summed in
// unsigned long.  When zbegin is negative and the column base is smaller than
// |zbegin| the sum wraps through 2^64, which shifts the bucket by 2^64 mod
// size: a box that starts its column there and one that does not then look in
// different buckets for the same cell and never meet.  column_wraps() tells
// which side of that split a box is on in a given column.
__device__ __forceinline__ bool column_wraps(int level, int x, int y, int zbegin) {
    unsigned long long base = (unsigned long long)(unsigned)level * 1000ull + (unsigned long long)(unsigned)x * 100ull +
                              (unsigned long long)(unsigned)y * 10ull;
    return zbegin < 0 && base < (unsigned long long)(-(long long)zbegin);
}

__device__ __forceinline__ int lookup(const unsigned long long *keys, unsigned mask, unsigned long long key) {
    unsigned h = hash64(key) & mask;
    for (unsigned probe = 0; probe <= mask; probe++) {
        unsigned long long k = keys[h];
        if (k == key) return (int)h;
        if (k == EMPTY_KEY) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}

// collideAABBs (collision_space_internal.h:44-80) without category bits (all set)
__device__ __forceinline__ bool aabb_pair_ok(const Geoms &G, int a, int b) {
    int ba = G.body[a], bb = G.body[b];
    if (ba == bb && ba >= 0) return false;
    float4 l1 = G.amin[a], h1 = G.amax[a], l2 = G.amin[b], h2 = G.amax[b];
    if (l1.x > h2.x || h1.x < l2.x || l1.y > h2.y || h1.y < l2.y || l1.z > h2.z || h1.z < l2.z) return false;
    return true;
}

// pass 0 counts (and keeps each geom's first GB_BP_CACHE partners, in the
// order found), pass 1 writes: a geom whose partners all fit the cache copies
// them, the others search again; then each geom's partners are sorted
// ascending.  Either way the pairs and their order are the same.  (A pass
// takes as long as its slowest geom's search: with 8 cached partners the few
// geoms with more kept pass 1 at 0.30 ms on the 32,768-body pile; with 32 it
// is a copy, 0.02 ms, for 128 bytes a geom.)
#define GB_BP_CACHE 32
template <int PASS>
__global__ void k_bp_pairs(Geoms G, const unsigned long long *keys, unsigned mask, const int *start, const int *count,
                           const int *members, const int *big_list, int *pcount, const int *pstart, int2 *pairs,
                           int pair_cap, DevCounters *dc, int exact, int *cache) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= G.n) return;
    int la = G.level[a];
    int n = 0;
    int base = PASS ? pstart[a] : 0;
    const bool cached = PASS && pcount[a] <= GB_BP_CACHE;
    if (cached) {
        // partners copied from pass 0's cache (no search)
        n = pcount[a];
        for (int i = 0; i < n; i++)
            if (base + i < pair_cap) pairs[base + i] = make_int2(a, cache[(size_t)a * GB_BP_CACHE + i]);
    } else if (la != BIG_LEVEL) {
        int maxlevel = dc->maxlevel;
        int4 lo = G.dblo[a], hi = G.dbhi[a];
        for (int L = la; L <= maxlevel; L++) {
            int sh = L - la;
            int x0 = lo.x >> sh, x1 = hi.x >> sh, y0 = lo.y >> sh, y1 = hi.y >> sh, z0 = lo.z >> sh, z1 = hi.z >> sh;
            for (int x = x0; x <= x1; x++)
                for (int y = y0; y <= y1; y++)
                    for (int z = z0; z <= z1; z++) {
                        int slot = lookup(keys, mask, cell_key(L, x, y, z));
                        if (slot < 0) continue;
                        int s0 = start[slot], s1 = s0 + count[slot];
                        for (int s = s0; s < s1; s++) {
                            int b = members[s];
                            if (b == a) continue;
                            if (L == la && b < a) continue;
                            int4 blo = G.dblo[b], bhi = G.dbhi[b];
                            int cz = max(z0, blo.z);
                            if (cz != z) continue;
                            if (exact) {
                                // every overlapping pair, once: in the low-corner cell of the overlap
                                if (max(x0, blo.x) != x || max(y0, blo.y) != y) continue;
                            } else {
                                // the reference's rule: the pair meets in the first overlap column
                                // (x, then y ascending) where both boxes hash their column alike
                                int fx = 0x7fffffff, fy = 0;
                                for (int cx = max(x0, blo.x); cx <= min(x1, bhi.x) && fx == 0x7fffffff; cx++)
                                    for (int cy = max(y0, blo.y); cy <= min(y1, bhi.y); cy++)
                                        if (column_wraps(L, cx, cy, z0) == column_wraps(L, cx, cy, blo.z)) {
                                            fx = cx; fy = cy;
                                            break;
                                        }
                                if (fx != x || fy != y) continue;
                            }
                            if (!aabb_pair_ok(G, a, b)) continue;
                            if (PASS) {
                                int idx = base + n;
                                if (idx < pair_cap) pairs[idx] = make_int2(a, b);
                            } else if (n < GB_BP_CACHE) {
                                cache[(size_t)a * GB_BP_CACHE + n] = b;
                            }
                            n++;
                        }
                    }
        }
        int nbig = dc->nbig;
        for (int k = 0; k < nbig; k++) {
            int b = big_list[k];
            if (!aabb_pair_ok(G, a, b)) continue;
            if (PASS) {
                int idx = base + n;
                if (idx < pair_cap) pairs[idx] = make_int2(a, b);
            } else if (n < GB_BP_CACHE) {
                cache[(size_t)a * GB_BP_CACHE + n] = b;
            }
            n++;
        }
    } else {
        // big boxes against each other (collision_space.cpp:597-602), once per pair
        int nbig = dc->nbig;
        for (int k = 0; k < nbig; k++) {
            int b = big_list[k];
            if (b <= a || !aabb_pair_ok(G, a, b)) continue;
            if (PASS) {
                int idx = base + n;
                if (idx < pair_cap) pairs[idx] = make_int2(a, b);
            } else if (n < GB_BP_CACHE) {
                cache[(size_t)a * GB_BP_CACHE + n] = b;
            }
            n++;
        }
    }
    if (!PASS) {
        pcount[a] = n;
    } else if (base + n <= pair_cap) {
        // insertion sort of this geom's partners (short lists)
        for (int i = 1; i < n; i++) {
            int2 v = pairs[base + i];
            int j = i - 1;
            while (j >= 0 && pairs[base + j].y > v.y) { pairs[base + j + 1] = pairs[base + j]; j--; }
            pairs[base + j + 1] = v;
        }
    }
}

__global__ void k_bp_finish(DevCounters *dc, int pair_cap) {
    if (dc->npairs > pair_cap) { atomicOr(&dc->err, ERR_PAIR_OVERFLOW); dc->npairs = pair_cap; }
}

// ------------------------------------------------------------------ narrow phase
__device__ __forceinline__ void load_view(const Geoms &G, int g, GeomView &v) {
    v.cls = G.cls[g];
    float4 p = G.gpos[g];
    v.pos[0] = p.x; v.pos[1] = p.y; v.pos[2] = p.z; v.pos[3] = 0;
    for (int r = 0; r < 3; r++) {
        float4 rr = G.gR[3 * g + r];
        v.R[4 * r] = rr.x; v.R[4 * r + 1] = rr.y; v.R[4 * r + 2] = rr.z; v.R[4 * r + 3] = 0;
    }
    float4 d = G.dims[g];
    v.dims[0] = d.x; v.dims[1] = d.y; v.dims[2] = d.z; v.dims[3] = d.w;
}

// One thread per candidate pair: dCollide restated (collision_kernel.cpp:292-338)
// into fixed per-pair slots.
// skip_static: drop pairs of two body-less geoms (a contact joint attached to
// no body never enters the reference's islands); dCollide keeps them.
// Body pairs connected by a ball or hinge joint (open-addressed set of
// min << 32 | max keys; empty: ~0): the fused path skips their geom pairs, as
// an ODE near callback does with dAreConnectedExcluding (demo_boxstack.cpp:140).
__device__ __forceinline__ bool jointed(const unsigned long long *keys, unsigned mask, int a, int b) {
    if (!keys || a < 0 || b < 0) return false;
    const unsigned long long key = ((unsigned long long)(unsigned)min(a, b) << 32) | (unsigned)max(a, b);
    unsigned h = hash64(key) & mask;
    for (unsigned probe = 0; probe <= mask; probe++) {
        const unsigned long long k = keys[h];
        if (k == key) return true;
        if (k == ~0ull) return false;
        h = (h + 1) & mask;
    }
    return false;
}

// Class-sorted batches.  The broad phase emits pairs in hash order, so the
// 32 lanes of a warp would meet several colliders and run them one after
// another.  The pairs are instead visited through a permutation that groups
// them by collider class (class of g1, class of g2; the pairs the narrow phase
// rejects form a 17th group): a warp then takes a batch of 32 pairs of one
// class.  Each pair still writes its own slots, so the contacts, their order
// and every result are as before; the order inside a class is free.
#define GB_PAIR_KEYS 17
__device__ __forceinline__ int class_slot(int c) { return c == dPlaneClass ? 3 : (c >= 0 && c < 3 ? c : 3); }
__device__ __forceinline__ int pair_key(const Geoms &G, int2 pr, int skip_static, const unsigned long long *jkeys,
                                        unsigned jmask) {
    const int a = pr.x, b = pr.y;
    const int ba = G.body[a], bb = G.body[b];
    if (a == b || (ba == bb && ba >= 0) || (skip_static && ba < 0 && bb < 0) || jointed(jkeys, jmask, ba, bb))
        return GB_PAIR_KEYS - 1;
    return class_slot(G.cls[a]) * 4 + class_slot(G.cls[b]);
}

// counts per class key (a shared histogram per block, then the global counters)
__global__ void k_pair_count(Geoms G, const int2 *pairs, const int *npairs_dev, int skip_static,
                             const unsigned long long *jkeys, unsigned jmask, int *kcount) {
    __shared__ int h[GB_PAIR_KEYS];
    const int np = *npairs_dev;
    for (int base = blockIdx.x * blockDim.x; base < np; base += gridDim.x * blockDim.x) {
        if (threadIdx.x < GB_PAIR_KEYS) h[threadIdx.x] = 0;
        __syncthreads();
        const int p = base + threadIdx.x;
        if (p < np) atomicAdd(&h[pair_key(G, pairs[p], skip_static, jkeys, jmask)], 1);
        __syncthreads();
        if (threadIdx.x < GB_PAIR_KEYS && h[threadIdx.x]) atomicAdd(&kcount[threadIdx.x], h[threadIdx.x]);
        __syncthreads();
    }
}

// perm: the pairs grouped by class key (kfill: zeroed positions per key)
__global__ void k_pair_order(Geoms G, const int2 *pairs, const int *npairs_dev, int skip_static,
                             const unsigned long long *jkeys, unsigned jmask, const int *kcount, int *kfill,
                             int *perm) {
    __shared__ int h[GB_PAIR_KEYS], at[GB_PAIR_KEYS], start[GB_PAIR_KEYS];
    const int np = *npairs_dev;
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < GB_PAIR_KEYS; k++) { start[k] = acc; acc += kcount[k]; }
    }
    for (int base = blockIdx.x * blockDim.x; base < np; base += gridDim.x * blockDim.x) {
        if (threadIdx.x < GB_PAIR_KEYS) h[threadIdx.x] = 0;
        __syncthreads();
        const int p = base + threadIdx.x;
        const int key = p < np ? pair_key(G, pairs[p], skip_static, jkeys, jmask) : -1;
        const int rank = key >= 0 ? atomicAdd(&h[key], 1) : 0;
        __syncthreads();
        if (threadIdx.x < GB_PAIR_KEYS && h[threadIdx.x])
            at[threadIdx.x] = start[threadIdx.x] + atomicAdd(&kfill[threadIdx.x], h[threadIdx.x]);
        __syncthreads();
        if (key >= 0) perm[at[key] + rank] = p;
        __syncthreads();
    }
}

__global__ void k_narrow(Geoms G, const int2 *pairs, const int *npairs_dev, int np_host, int maxc, int surf,
                         Contact *slots, int *ccount, int *codes, int skip_static, const unsigned long long *jkeys,
                         unsigned jmask, const int *perm) {
    const int np = npairs_dev ? *npairs_dev : np_host;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const int p = perm ? perm[i] : i;
        int2 pr = pairs[p];
        int a = pr.x, b = pr.y;
        int n = 0, code = -1;
        CPoint c[8];
        const bool both_static = G.body[a] < 0 && G.body[b] < 0;
        if (a != b && !(G.body[a] == G.body[b] && G.body[a] >= 0) && !(skip_static && both_static) &&
            !jointed(jkeys, jmask, G.body[a], G.body[b])) {
            GeomView va, vb;
            load_view(G, a, va);
            load_view(G, b, vb);
            n = collide_pair(va, vb, maxc, c, &code);
        }
        ccount[p] = n;
        if (codes) codes[p] = code;
        int ba = G.body[a], bb = G.body[b];
        for (int i = 0; i < n; i++) {
            Contact k;
            k.pos_depth = make_float4(c[i].pos[0], c[i].pos[1], c[i].pos[2], c[i].depth);
            k.normal = make_float4(c[i].normal[0], c[i].normal[1], c[i].normal[2], 0.f);
            k.b1 = ba; k.b2 = bb; k.surf = surf; k.slot = i;
            k.g1 = a; k.g2 = b; k.pad0 = 0; k.pad1 = 0;
            slots[(size_t)p * 8 + i] = k;
        }
    }
}

__global__ void k_compact(const int *npairs_dev, const int *ccount, const int *cstart, const Contact *slots,
                          Contact *out, int base_count_index, DevCounters *dc, int contact_cap) {
    const int np = *npairs_dev;
    const int base = base_count_index;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        int n = ccount[p], o = base + cstart[p];
        for (int i = 0; i < n; i++) {
            if (o + i < contact_cap) out[o + i] = slots[(size_t)p * 8 + i];
        }
    }
}

__global__ void k_contacts_total(DevCounters *dc, int base, int contact_cap) {
    int total = base + dc->narrow_total;
    if (total > contact_cap) { atomicOr(&dc->err, ERR_CONTACT_OVERFLOW); total = contact_cap; }
    dc->ncontacts = total;
}

// ------------------------------------------------------------------ host side
static int grid_for(int n, int block) { return n <= 0 ? 1 : (n + block - 1) / block; }

static Geoms geoms_view(Workspace &ws, int ng) {
    Geoms G;
    G.cls = ws.g_cls.as<int>(); G.body = ws.g_body.as<int>();
    G.dims = ws.g_dims.as<float4>(); G.spos = ws.g_spos.as<float4>(); G.sR = ws.g_sR.as<float4>();
    G.gpos = ws.g_pos.as<float4>(); G.gR = ws.g_R.as<float4>();
    G.amin = ws.g_amin.as<float4>(); G.amax = ws.g_amax.as<float4>();
    G.level = ws.g_level.as<int>(); G.dblo = ws.g_dblo.as<int4>(); G.dbhi = ws.g_dbhi.as<int4>();
    G.n = ng;
    return G;
}

bool upload_geoms(Workspace &ws, const std::vector<GeomHost> &g, cudaStream_t s) {
    int ng = (int)g.size();
    size_t n = ng > 0 ? ng : 1;
    bool ok = ws.g_cls.ensure(n * 4) && ws.g_body.ensure(n * 4) && ws.g_dims.ensure(n * 16) && ws.g_spos.ensure(n * 16) &&
              ws.g_sR.ensure(n * 48) && ws.g_pos.ensure(n * 16) && ws.g_R.ensure(n * 48) && ws.g_amin.ensure(n * 16) &&
              ws.g_amax.ensure(n * 16) && ws.g_level.ensure(n * 4) && ws.g_dblo.ensure(n * 16) &&
              ws.g_dbhi.ensure(n * 16) && ws.g_big.ensure(n * 4);
    if (!ok) return false;
    std::vector<int> cls(n), body(n);
    std::vector<float> dims(4 * n), spos(4 * n), sR(12 * n);
    for (int i = 0; i < ng; i++) {
        cls[i] = g[i].cls; body[i] = g[i].body;
        for (int k = 0; k < 4; k++) dims[4 * i + k] = g[i].dims[k];
        for (int k = 0; k < 3; k++) spos[4 * i + k] = g[i].pos[k];
        spos[4 * i + 3] = 0;
        for (int k = 0; k < 12; k++) sR[12 * i + k] = g[i].R[k];
    }
    if (ng == 0) return true;
    cudaMemcpyAsync(ws.g_cls.p, cls.data(), 4 * ng, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.g_body.p, body.data(), 4 * ng, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.g_dims.p, dims.data(), 16 * ng, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.g_spos.p, spos.data(), 16 * ng, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ws.g_sR.p, sR.data(), 48 * ng, cudaMemcpyHostToDevice, s);
    // the staging vectors die at return: make the copies complete first
    cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess;
}

__global__ void k_set_surface(Surface v, Surface *dst) { *dst = v; }
void launch_set_surface(Workspace &ws, const Surface &v, cudaStream_t s) {
    k_set_surface<<<1, 1, 0, s>>>(v, ws.surfaces.as<Surface>());
    count_launch();
}

__global__ void k_pose_init(DevCounters *dc) {
    dc->nbig = 0;
    dc->maxlevel = -1000;
}

void launch_pose_aabb(Workspace &ws, const Bodies &b, int ng, int minlevel, int maxlevel, cudaStream_t s) {
    // big-list count and coarsest level in use are rebuilt by the kernel
    k_pose_init<<<1, 1, 0, s>>>(ws.dc);
    k_pose_aabb<<<grid_for(ng, 128), 128, 0, s>>>(geoms_view(ws, ng), b, minlevel, maxlevel, ws.g_big.as<int>(), ws.dc);
    count_launch(2);
}

static unsigned table_mask(int ng) {
    unsigned sz = 1024;
    while (sz < (unsigned)(16 * (ng > 0 ? ng : 1))) sz <<= 1;
    return sz - 1;
}

bool launch_broadphase(Workspace &ws, int ng, int exact, cudaStream_t s) {
    unsigned mask = table_mask(ng);
    size_t tsz = (size_t)mask + 1;
    size_t nge = ng > 0 ? ng : 1;
    if (!(ws.h_keys.ensure(tsz * 8) && ws.h_count.ensure(tsz * 4) && ws.h_start.ensure(tsz * 4) &&
          ws.h_fill.ensure(tsz * 4) && ws.h_members.ensure(nge * 8 * 4) && ws.h_entry.ensure(nge * 8 * 4) &&
          ws.p_count.ensure(nge * 4) && ws.p_start.ensure(nge * 4) && ws.p_cache.ensure(nge * GB_BP_CACHE * 4)))
        return false;
    if (ws.pair_cap < 16 * (int)nge) {
        int cap = 16 * (int)nge;
        if (!ws.pairs.ensure((size_t)cap * 8)) return false;
        ws.pair_cap = cap;
    }
    Geoms G = geoms_view(ws, ng);
    cudaMemsetAsync(ws.h_keys.p, 0xFF, tsz * 8, s);
    cudaMemsetAsync(ws.h_count.p, 0, tsz * 4, s);
    cudaMemsetAsync(ws.h_fill.p, 0, tsz * 4, s);
    k_bp_insert<<<grid_for(ng, 128), 128, 0, s>>>(G, ws.h_keys.as<unsigned long long>(), mask, ws.h_count.as<int>(),
                                                   ws.h_entry.as<int>(), ws.dc);
    scan_exclusive(ws.h_count.as<int>(), ws.h_start.as<int>(), nullptr, (int)tsz, &ws.dc->cells_total, ws, s);
    k_bp_fill<<<grid_for(8 * ng, 256), 256, 0, s>>>(ng, ws.h_entry.as<int>(), ws.h_start.as<int>(), ws.h_fill.as<int>(),
                                                    ws.h_members.as<int>());
    k_bp_pairs<0><<<grid_for(ng, 128), 128, 0, s>>>(G, ws.h_keys.as<unsigned long long>(), mask, ws.h_start.as<int>(),
                                                    ws.h_count.as<int>(), ws.h_members.as<int>(), ws.g_big.as<int>(),
                                                    ws.p_count.as<int>(), nullptr, nullptr, 0, ws.dc, exact,
                                                    ws.p_cache.as<int>());
    scan_exclusive(ws.p_count.as<int>(), ws.p_start.as<int>(), nullptr, ng, &ws.dc->npairs, ws, s);
    k_bp_pairs<1><<<grid_for(ng, 128), 128, 0, s>>>(G, ws.h_keys.as<unsigned long long>(), mask, ws.h_start.as<int>(),
                                                    ws.h_count.as<int>(), ws.h_members.as<int>(), ws.g_big.as<int>(),
                                                    ws.p_count.as<int>(), ws.p_start.as<int>(), ws.pairs.as<int2>(),
                                                    ws.pair_cap, ws.dc, exact, ws.p_cache.as<int>());
    k_bp_finish<<<1, 1, 0, s>>>(ws.dc, ws.pair_cap);
    count_launch(5);
    return cudaGetLastError() == cudaSuccess;
}

static bool ensure_contact_buffers(Workspace &ws, int pair_cap, int extra) {
    size_t slots = (size_t)(pair_cap > 0 ? pair_cap : 1) * 8;
    if (!(ws.c_slots.ensure(slots * sizeof(Contact)) && ws.c_count.ensure((size_t)(pair_cap + 1) * 4) &&
          ws.c_start.ensure((size_t)(pair_cap + 1) * 4) && ws.c_code.ensure((size_t)(pair_cap + 1) * 4)))
        return false;
    int want = 4 * pair_cap + extra;
    if (ws.contact_cap < want) {
        if (!ws.contacts.ensure((size_t)want * sizeof(Contact))) return false;
        ws.contact_cap = want;
    }
    return true;
}

bool launch_narrowphase(Workspace &ws, int maxc, int surf, bool append, cudaStream_t s) {
    if (!ensure_contact_buffers(ws, ws.pair_cap, 0)) return false;
    if (!(ws.n_perm.ensure((size_t)(ws.pair_cap > 0 ? ws.pair_cap : 1) * 4) && ws.n_key.ensure(2 * GB_PAIR_KEYS * 4)))
        return false;
    Geoms G = geoms_view(ws, 0);
    int grid = 4 * num_sms();
    if (maxc > 8) maxc = 8;
    const unsigned long long *jk = ws.njoints > 0 ? ws.j_pairs.as<unsigned long long>() : nullptr;
    int *kcount = ws.n_key.as<int>(), *kfill = kcount + GB_PAIR_KEYS;
    cudaMemsetAsync(kcount, 0, 2 * GB_PAIR_KEYS * 4, s);
    k_pair_count<<<grid, 256, 0, s>>>(G, ws.pairs.as<int2>(), &ws.dc->npairs, 1, jk, ws.j_pair_mask, kcount);
    k_pair_order<<<grid, 256, 0, s>>>(G, ws.pairs.as<int2>(), &ws.dc->npairs, 1, jk, ws.j_pair_mask, kcount, kfill,
                                      ws.n_perm.as<int>());
    k_narrow<<<grid, 128, 0, s>>>(G, ws.pairs.as<int2>(), &ws.dc->npairs, 0, maxc, surf, ws.c_slots.as<Contact>(),
                                  ws.c_count.as<int>(), ws.c_code.as<int>(), 1, jk, ws.j_pair_mask,
                                  ws.n_perm.as<int>());
    count_launch(2);
    scan_exclusive(ws.c_count.as<int>(), ws.c_start.as<int>(), &ws.dc->npairs, ws.pair_cap, &ws.dc->narrow_total, ws, s);
    // the base offset when appending is read on the host only in the compat
    // path; the fused path always starts from an empty contact list
    int base = 0;
    if (append) {
        int nc = 0;
        cudaMemcpyAsync(&nc, &ws.dc->ncontacts, 4, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        base = nc;
    }
    // the capacity the compaction sees (lowered only by the error-path tests)
    const int cap = g_test.contact_cap > 0 && g_test.contact_cap < ws.contact_cap ? g_test.contact_cap : ws.contact_cap;
    k_compact<<<grid, 128, 0, s>>>(&ws.dc->npairs, ws.c_count.as<int>(), ws.c_start.as<int>(), ws.c_slots.as<Contact>(),
                                   ws.contacts.as<Contact>(), base, ws.dc, cap);
    k_contacts_total<<<1, 1, 0, s>>>(ws.dc, base, cap);
    count_launch(3);
    return cudaGetLastError() == cudaSuccess;
}

int narrow_pairs_host(Workspace &ws, const int *pairs, int np, int maxc, std::vector<float> &out, std::vector<int> &counts,
                      cudaStream_t s) {
    if (np <= 0) { out.clear(); counts.clear(); return 0; }
    if (ws.pair_cap < np) {
        if (!ws.pairs.ensure((size_t)np * 8)) return -1;
        ws.pair_cap = np;
    }
    if (!ensure_contact_buffers(ws, ws.pair_cap, 0)) return -1;
    cudaMemcpyAsync(ws.pairs.p, pairs, (size_t)np * 8, cudaMemcpyHostToDevice, s);
    Geoms G = geoms_view(ws, 0);
    if (maxc > 8) maxc = 8;
    k_narrow<<<grid_for(np, 128), 128, 0, s>>>(G, ws.pairs.as<int2>(), nullptr, np, maxc, 0, ws.c_slots.as<Contact>(),
                                               ws.c_count.as<int>(), ws.c_code.as<int>(), 0, nullptr, 0u, nullptr);
    count_launch();
    counts.resize(np);
    std::vector<Contact> slots((size_t)np * 8);
    cudaMemcpyAsync(counts.data(), ws.c_count.p, (size_t)np * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(slots.data(), ws.c_slots.p, (size_t)np * 8 * sizeof(Contact), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    out.assign((size_t)np * 8 * 8, 0.f);
    for (int p = 0; p < np; p++)
        for (int i = 0; i < counts[p]; i++) {
            const Contact &c = slots[(size_t)p * 8 + i];
            float *o = &out[((size_t)p * 8 + i) * 8];
            o[0] = c.pos_depth.x; o[1] = c.pos_depth.y; o[2] = c.pos_depth.z;
            o[3] = c.normal.x; o[4] = c.normal.y; o[5] = c.normal.z;
            o[6] = c.pos_depth.w; o[7] = 0.f;
        }
    return np;
}

}  // namespace gb
