// Two-level coloured SOR sweep (included by solve.cu after k_pgs).
//
// The coloured solver's cost on a large connected pile is the number of grid
// barriers a sweep needs (one per colour, ~1.3 us each on 152 SMs) times the
// sweeps, while the relaxation itself is short.  Here the dynamic bodies are
// split into one spatial part per thread block: SX strips in x, each cut into
// SY parts in y, SX * SY = blocks, every cut placed so that the parts carry
// about the same number of contact ends (a column through the whole pile per
// part).  A constraint group whose bodies lie in one part (the static world
// belongs to every part) is interior to it; the others cross parts.  One sweep
// is then
//   1. the interior phase (repeated `ipasses` times): every block relaxes its
//      part's interior groups, colour by colour under block barriers only,
//      with the rows (80 bytes a row, loaded once per step), their
//      multipliers and the part's body accumulators fc resident in shared
//      memory;
//   2. the part's fc published to global memory, one grid barrier;
//   3. the cross groups in their own global colours, exactly as k_pgs relaxes
//      colours (staged waves, one grid barrier per colour);
//   4. the part's fc read back from global memory.
// Both phases are Gauss-Seidel in a fixed order (no two groups of one colour
// share a body), so a sweep is deterministic.
//
// Neighbour waits (the default; GBODE_SYNC_NEIGHBOURS): a cross group is
// relaxed by the block whose part holds its first body, and a block's steps
// (the interior phase, then each cross colour) conflict only with the steps of
// blocks that touch one of the same bodies -- the part owning a body and the
// owners of the cross groups touching it.  Those blocks are listed once per
// solve; every block counts its finished steps in a global counter (release),
// and before a step that reads bodies a block waits (acquire, bounded) until
// each listed block has finished the previous step.  A block with nothing to
// do in a colour does not wait at all.  Every body's accumulators then see
// the same sequence of updates as under a grid barrier per colour, so the
// result is the same to the bit, while a colour costs only what the blocks
// that work in it need.  The interior and the cross
// groups are coloured independently (k_colour with a class per group).  A
// part whose interior rows, groups or bodies exceed the shared-memory
// capacity gives all its groups to the cross phase, so any world runs; worlds
// of many small islands spread over all blocks keep the one-level k_pgs.
//
// quickstep.cpp:2917-3033 is the row update; the order of the rows inside a
// contact manifold (normal rows first, then the friction pairs) is that of
// relax_triplets.

#define GB_SLAB_NBIN 1024      // histogram bins per axis of the partition
#define GB_SLAB_XCHUNK 128     // cross-phase staging rows per buffer
#define GB_SLAB_ROW_F4 5       // float4 per interior row (80 bytes)
#define GB_SLAB_COLOURS 64     // interior colours (64 + c in the shared colouring)
#define GB_XACC 16             // owner blocks listed per body (cross groups touching it)
#define GB_XADJ_WORDS 8        // words of a block's adjacency bit set (up to 256 blocks)

__device__ __forceinline__ int ord_f(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unord_f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ int slab_bin(float v, int lo_o, int hi_o) {
    const float lo = unord_f(lo_o), hi = unord_f(hi_o);
    const float span = hi - lo;
    int b = span > 0.f ? (int)((v - lo) / span * (float)GB_SLAB_NBIN) : 0;
    return b < 0 ? 0 : (b >= GB_SLAB_NBIN ? GB_SLAB_NBIN - 1 : b);
}

// contact ends per body: the weight the partition balances
__global__ void k_slab_weight(const Contact *C, const int *nc_dev, int *bw, DevCounters *dc) {
    const int nc = *nc_dev;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        dc->slab_box[0] = 0x7fffffff; dc->slab_box[1] = (int)0x80000000;
        dc->slab_box[2] = 0x7fffffff; dc->slab_box[3] = (int)0x80000000;
    }
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Contact k = C[c];
        if (k.b1 >= 0) atomicAdd(&bw[k.b1], 1);
        if (k.b2 >= 0) atomicAdd(&bw[k.b2], 1);
    }
}

// x / y range of the weighted bodies
__global__ void k_slab_range(Bodies B, const int *bw, DevCounters *dc) {
    int x0 = 0x7fffffff, x1 = (int)0x80000000, y0 = 0x7fffffff, y1 = (int)0x80000000;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
        if (bw[b] <= 0) continue;
        const float4 p = B.pos[b];
        x0 = min(x0, ord_f(p.x)); x1 = max(x1, ord_f(p.x));
        y0 = min(y0, ord_f(p.y)); y1 = max(y1, ord_f(p.y));
    }
    x0 = __reduce_min_sync(0xffffffffu, x0); x1 = __reduce_max_sync(0xffffffffu, x1);
    y0 = __reduce_min_sync(0xffffffffu, y0); y1 = __reduce_max_sync(0xffffffffu, y1);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&dc->slab_box[0], x0); atomicMax(&dc->slab_box[1], x1);
        atomicMin(&dc->slab_box[2], y0); atomicMax(&dc->slab_box[3], y1);
    }
}

// hist[0 .. NBIN): weight by x bin; hist[NBIN + strip * NBIN + ybin] (axis 1):
// weight by y bin within each x strip (binpart of the x histogram known)
__global__ void k_slab_hist(Bodies B, const int *bw, const DevCounters *dc, const int *binpart, int *hist, int axis) {
    const int bx0 = dc->slab_box[0], bx1 = dc->slab_box[1], by0 = dc->slab_box[2], by1 = dc->slab_box[3];
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
        const int w = bw[b];
        if (w <= 0) continue;
        const float4 p = B.pos[b];
        const int xb = slab_bin(p.x, bx0, bx1);
        if (axis == 0) atomicAdd(&hist[xb], w);
        else atomicAdd(&hist[GB_SLAB_NBIN + binpart[xb] * GB_SLAB_NBIN + slab_bin(p.y, by0, by1)], w);
    }
}

// One block of GB_SLAB_NBIN threads per histogram row: bin -> part by the
// cumulative weight at the bin's start, floor(parts * before / total).
__global__ void k_slab_cut(const int *hist, int *binpart, int parts) {
    __shared__ int wsum[32];
    const int row = blockIdx.x, t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int v = hist[row * GB_SLAB_NBIN + t];
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += x;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int x = wsum[lane];
        int xi = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        wsum[lane] = xi - x;  // exclusive, per warp
    }
    __syncthreads();
    const long long before = (long long)wsum[wid] + inc - v;
    __shared__ long long total_s;
    if (t == GB_SLAB_NBIN - 1) total_s = before + v;
    __syncthreads();
    const long long total = total_s;
    int p = total > 0 ? (int)(before * parts / total) : 0;
    binpart[row * GB_SLAB_NBIN + t] = p < parts ? p : parts - 1;
}

// part of every weighted body (strip * sy + y part), its index in the part,
// the part's body list (first bcap)
__global__ void k_slab_assign(Bodies B, const int *bw, const DevCounters *dc, const int *binpart, int sy,
                              int *part, int *blocal, int *pbcount, int *pbody, int bcap) {
    const int bx0 = dc->slab_box[0], bx1 = dc->slab_box[1], by0 = dc->slab_box[2], by1 = dc->slab_box[3];
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
        if (bw[b] <= 0) { part[b] = -1; continue; }
        const float4 p = B.pos[b];
        const int strip = binpart[slab_bin(p.x, bx0, bx1)];
        const int q = strip * sy + binpart[GB_SLAB_NBIN + strip * GB_SLAB_NBIN + slab_bin(p.y, by0, by1)];
        const int l = atomicAdd(&pbcount[q], 1);
        part[b] = q;
        blocal[b] = l;
        if (l < bcap) pbody[(size_t)q * bcap + l] = b;
    }
}

// interior (its part) or cross (-1) for every group; interior rows and
// groups counted per part.  Only triplet manifolds (contacts under
// dContactApprox1 with friction) have the compact interior row form.
__global__ void k_slab_classify(const int4 *gdesc, const DevCounters *dc, const int *part, int *gpart, int *prow,
                                int *pgrp) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int4 d = gdesc[e];
        int p = -1;
        if (d.y & GB_DESC_TRIPLETS) {
            const int p0 = part[d.z], p1 = d.w >= 0 ? part[d.w] : p0;
            if (p0 >= 0 && p0 == p1) p = p0;
        }
        gpart[e] = p;
        if (p >= 0) {
            atomicAdd(&prow[p], desc_rows(d));
            atomicAdd(&pgrp[p], 1);
        }
    }
}

// a part over any shared-memory capacity hands all its groups to the cross phase
__global__ void k_slab_demote(const DevCounters *dc, const int *prow, const int *pgrp, const int *pbcount, int rcap,
                              int gcap, int bcap, int *gpart) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int p = gpart[e];
        if (p >= 0 && (prow[p] > rcap || pgrp[p] > gcap || pbcount[p] > bcap)) gpart[e] = -1;
    }
}

__global__ void k_slab_count(const DevCounters *dc, const int *gpart, const int *colour, int *pccount) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int p = gpart[e];
        if (p < 0) continue;
        const int c = colour[e] - 64;
        if (c >= 0 && c < GB_SLAB_COLOURS) atomicAdd(&pccount[p * GB_SLAB_COLOURS + c], 1);
    }
}

// interior groups listed part by part, colour by colour (order within one
// (part, colour) is free: those groups share no body)
__global__ void k_slab_fill(const DevCounters *dc, const int *gpart, const int *colour, const int4 *gdesc,
                            const int *pcstart, int *pcfill, int *ilist, int *irown) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int p = gpart[e];
        if (p < 0) continue;
        const int c = colour[e] - 64;
        if (c < 0 || c >= GB_SLAB_COLOURS) continue;
        const int k = p * GB_SLAB_COLOURS + c;
        const int pos = pcstart[k] + atomicAdd(&pcfill[k], 1);
        ilist[pos] = e;
        irown[pos] = desc_rows(gdesc[e]);
    }
}

// The interior descriptors (first global row, row count and flags, local
// bodies b1 | (b2 + 1) << 16, first row in the part's block of rows) and rows:
//   q0 J1l' (xyz, rhs')   q1 J1a' (xyz, cfm')   q2 J2a' (xyz, hi)
//   q3 M1a (xyz, invm1 / Ad)   q4 M2a (xyz, invm2 / Ad)
// A contact row's second linear Jacobian is the negated first one (J2l' =
// -J1l', exactly), and M^-1 J^T's linear parts are invm * J / Ad, so 80 bytes
// hold the row.  Normal rows have lo = 0; friction rows +-|hi * lambda_normal|.
__global__ void k_slab_pack(Rows Rw, Bodies B, const int *gpart, const int4 *gdesc, const int *ilist,
                            const int *irowoff, const int *irown, const int *pcstart, const int *blocal,
                            int total_slot, int4 *idesc, float4 *ipack, DevCounters *dc) {
    const int total = pcstart[total_slot];
    if (blockIdx.x == 0 && threadIdx.x == 0) dc->slab_rows = total > 0 ? irowoff[total - 1] + irown[total - 1] : 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int e = ilist[i];
        const int4 d = gdesc[e];
        const int p = gpart[e];
        const int off = irowoff[i] - irowoff[pcstart[p * GB_SLAB_COLOURS]];
        const int lb1 = blocal[d.z], lb2 = d.w >= 0 ? blocal[d.w] : -1;
        idesc[i] = make_int4(d.x, d.y, lb1 | ((lb2 + 1) << 16), off);
        const float im1 = B.pos[d.z].w, im2 = d.w >= 0 ? B.pos[d.w].w : 0.f;
        const int n = desc_rows(d);
        for (int k = 0; k < n; k++) {
            const int r = d.x + k;
            const float ad = Rw.Ad[r];
            const float4 m1a = Rw.M1a[r], m2a = Rw.M2a[r];
            float4 *o = ipack + (size_t)(irowoff[i] + k) * GB_SLAB_ROW_F4;
            o[0] = Rw.J1l[r];
            o[1] = Rw.J1a[r];
            o[2] = Rw.J2a[r];
            o[3] = make_float4(m1a.x, m1a.y, m1a.z, im1 / ad);
            o[4] = make_float4(m2a.x, m2a.y, m2a.z, im2 / ad);
        }
    }
}

// ---- neighbour waits: the cross groups per (colour, owner block), the blocks
// touching each body, the block adjacency

// the block that relaxes cross group e: the part of its first body with one
__device__ __forceinline__ int cross_owner(int2 gb, const int *part, int e, int B) {
    const int p1 = gb.x >= 0 ? part[gb.x] : -1, p2 = gb.y >= 0 ? part[gb.y] : -1;
    return p1 >= 0 ? p1 : (p2 >= 0 ? p2 : e % B);
}
__global__ void k_xown_count(const DevCounters *dc, const int *colour, const int2 *gbody, const int *part, int B,
                             int *xcnt) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c >= 0 && c < GB_SLAB_COLOURS) atomicAdd(&xcnt[c * B + cross_owner(gbody[e], part, e, B)], 1);
    }
}
// the cross colours' lists rewritten owner block by owner block: (colour c,
// block b)'s groups take slots xstart[c B + b] .. + xcnt[c B + b] (the
// flattened scan over (colour, block) starts colour c at its list start)
__global__ void k_xown_fill(const DevCounters *dc, const int *colour, const int2 *gbody, const int *part, int B,
                            const int *xstart, int *xfill, int *list) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c < 0 || c >= GB_SLAB_COLOURS) continue;
        const int k = c * B + cross_owner(gbody[e], part, e, B);
        list[xstart[k] + atomicAdd(&xfill[k], 1)] = e;
    }
}
// owner blocks of the cross groups touching each body
__global__ void k_xacc(DevCounters *dc, const int *colour, const int2 *gbody, const int *part, int B, int *accn,
                       int *acc) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c < 0 || c >= GB_SLAB_COLOURS) continue;
        const int2 gb = gbody[e];
        const int o = cross_owner(gb, part, e, B);
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const int x = s ? gb.y : gb.x;
            if (x < 0) continue;
            const int k = atomicAdd(&accn[x], 1);
            if (k < GB_XACC) acc[(size_t)x * GB_XACC + k] = o;
            else dc->slab_nbr_over = 1;
        }
    }
}
// every two blocks touching one body are adjacent
__global__ void k_xadj(const int *accn, const int *acc, const int *part, int nb, unsigned *adj) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < nb; x += gridDim.x * blockDim.x) {
        const int n = min(accn[x], GB_XACC);
        if (n == 0) continue;
        int L[GB_XACC + 1];
        int m = 0;
        if (part[x] >= 0) L[m++] = part[x];
        for (int k = 0; k < n; k++) L[m++] = acc[(size_t)x * GB_XACC + k];
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
                if (L[i] != L[j])
                    atomicOr(&adj[(size_t)L[i] * GB_XADJ_WORDS + (L[j] >> 5)], 1u << (L[j] & 31));
    }
}

// ---- split classes (mass splitting inside a class of merged cross colours)

// A crossing group can be relaxed in a split class if its rows are staged and
// every body it moves is in a part's body list (the part folds the class
// accumulators back into the body at the end of each sweep).
__global__ void k_split_check(DevCounters *dc, const int *colour, const int4 *gdesc, const int2 *gbody,
                              const int *part, const int *blocal, int bcap) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c < 0 || c >= GB_SLAB_COLOURS) continue;
        bool bad = !(gdesc[e].y & GB_DESC_STAGED);
        const int2 gb = gbody[e];
        if (gb.x >= 0 && (part[gb.x] < 0 || blocal[gb.x] >= bcap)) bad = true;
        if (gb.y >= 0 && (part[gb.y] < 0 || blocal[gb.y] >= bcap)) bad = true;
        if (bad) dc->split_off = 1;
    }
}
// Momentum between sweeps needs every body that a crossing group moves in a
// column's body list: each column moves its listed bodies' accumulators on at
// the end of a sweep (interior groups' bodies are listed by construction).
__global__ void k_mom_check(DevCounters *dc, const int *colour, const int2 *gbody, const int *part,
                            const int *blocal, int bcap) {
    const int ng = dc->nmanifolds;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c >= 64 && c < 64 + GB_SLAB_COLOURS) continue;
        const int2 gb = gbody[e];
        bool bad = false;
        if (gb.x >= 0 && (part[gb.x] < 0 || blocal[gb.x] >= bcap)) bad = true;
        if (gb.y >= 0 && (part[gb.y] < 0 || blocal[gb.y] >= bcap)) bad = true;
        if (bad) dc->mom_off = 1;
    }
}
// classes of this solve: k, or 0 (exact colours) if a group cannot be split or
// there are no more colours than classes
__global__ void k_split_classes(DevCounters *dc, int k) {
    dc->split_k = (!dc->split_off && dc->ncolours > k) ? k : 0;
    if (dc->split_k) dc->ncolours = k;
}
__global__ void k_split_remap(const DevCounters *dc, int *colour) {
    const int k = dc->split_k, ng = dc->nmanifolds;
    if (!k) return;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c >= 0 && c < GB_SLAB_COLOURS) colour[e] = c % k;
    }
}
// per body, the classes in which two or more groups touch it (bit c)
__global__ void k_split_mask(const DevCounters *dc, const int *nsplit, int nb, int *smask) {
    const int k = dc->split_k;
    if (!k) return;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int m = 0;
        for (int c = 0; c < k; c++)
            if (nsplit[(size_t)c * nb + b] >= 2) m |= 1 << c;
        smask[b] = m;
    }
}
// groups of each class touching each body
__global__ void k_split_count(const DevCounters *dc, const int *colour, const int2 *gbody, int nb, int *nsplit) {
    const int ng = dc->nmanifolds;
    if (!dc->split_k) return;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ng; e += gridDim.x * blockDim.x) {
        const int c = colour[e];
        if (c < 0 || c >= GB_SLAB_COLOURS) continue;
        const int2 gb = gbody[e];
        if (gb.x >= 0) atomicAdd(&nsplit[(size_t)c * nb + gb.x], 1);
        if (gb.y >= 0) atomicAdd(&nsplit[(size_t)c * nb + gb.y], 1);
    }
}

// Class accumulators: per (body, class c) the fixed-point sum (2^-32 units)
// of the changes that the groups of class c sharing the body made to its
// accumulators fc (linear x y z, angular x y z: 48 bytes; a body's classes
// side by side).  A group alone with a body in its class writes the body's fc
// itself, as the exact colours do.  A group of class k reads the slots of the
// earlier classes that shared its body (bit c of the body's mask) -- up to
// three loads issued together -- and adds its share to slot k; the fold at
// the end of the sweep takes every shared class back into fc.  Integer sums
// do not depend on the order of the additions.
#define GB_FIX_ONE 4294967296.f
__device__ __forceinline__ long long *split_slot(long long *dacc, int stride, int b, int c) {
    return dacc + ((size_t)b * stride + c) * 6;
}
__device__ __forceinline__ void split_add6(long long (&s)[6], const longlong2 *p, bool on) {
    const longlong2 q0 = __ldcg(p), q1 = __ldcg(p + 1), q2 = __ldcg(p + 2);
    if (on) { s[0] += q0.x; s[1] += q0.y; s[2] += q1.x; s[3] += q1.y; s[4] += q2.x; s[5] += q2.y; }
}
// (l, a) += the slots of the classes in `mask`
__device__ __forceinline__ void split_sum(long long *dacc, int stride, int b, int mask, float4 &l, float4 &a) {
    if (!mask) return;
    long long s[6] = {0, 0, 0, 0, 0, 0};
    const int c0 = __ffs(mask) - 1;
    int m = mask & (mask - 1);
    const int c1 = m ? __ffs(m) - 1 : c0;
    const bool h1 = m != 0;
    m &= m - 1;
    const int c2 = m ? __ffs(m) - 1 : c0;
    const bool h2 = m != 0;
    m &= m - 1;
    // three slots' loads before any sum (a missing class re-reads the first)
    const longlong2 *p0 = (const longlong2 *)split_slot(dacc, stride, b, c0);
    const longlong2 *p1 = (const longlong2 *)split_slot(dacc, stride, b, c1);
    const longlong2 *p2 = (const longlong2 *)split_slot(dacc, stride, b, c2);
    const longlong2 x0 = __ldcg(p0), x1 = __ldcg(p0 + 1), x2 = __ldcg(p0 + 2);
    const longlong2 y0 = __ldcg(p1), y1 = __ldcg(p1 + 1), y2 = __ldcg(p1 + 2);
    const longlong2 z0 = __ldcg(p2), z1 = __ldcg(p2 + 1), z2 = __ldcg(p2 + 2);
    s[0] = x0.x; s[1] = x0.y; s[2] = x1.x; s[3] = x1.y; s[4] = x2.x; s[5] = x2.y;
    if (h1) { s[0] += y0.x; s[1] += y0.y; s[2] += y1.x; s[3] += y1.y; s[4] += y2.x; s[5] += y2.y; }
    if (h2) { s[0] += z0.x; s[1] += z0.y; s[2] += z1.x; s[3] += z1.y; s[4] += z2.x; s[5] += z2.y; }
    while (m) {  // a fourth shared class or more
        split_add6(s, (const longlong2 *)split_slot(dacc, stride, b, __ffs(m) - 1), true);
        m &= m - 1;
    }
    const float u = 1.f / GB_FIX_ONE;
    l.x += __ll2float_rn(s[0]) * u; l.y += __ll2float_rn(s[1]) * u; l.z += __ll2float_rn(s[2]) * u;
    a.x += __ll2float_rn(s[3]) * u; a.y += __ll2float_rn(s[4]) * u; a.z += __ll2float_rn(s[5]) * u;
}
__device__ __forceinline__ void split_add1(long long *p, long long q) {
    if (q) atomicAdd((unsigned long long *)p, (unsigned long long)q);
}
// the group's share of the body's change, (local copy - snapshot) / n, into
// the slot of class c
__device__ __forceinline__ void split_add(long long *dacc, int stride, int c, int b, float4 l, float4 a, float4 l0,
                                          float4 a0, float n) {
    const float r = 1.f / n;
    long long *p = split_slot(dacc, stride, b, c);
    split_add1(p + 0, __float2ll_rn((l.x - l0.x) * r * GB_FIX_ONE));
    split_add1(p + 1, __float2ll_rn((l.y - l0.y) * r * GB_FIX_ONE));
    split_add1(p + 2, __float2ll_rn((l.z - l0.z) * r * GB_FIX_ONE));
    split_add1(p + 3, __float2ll_rn((a.x - a0.x) * r * GB_FIX_ONE));
    split_add1(p + 4, __float2ll_rn((a.y - a0.y) * r * GB_FIX_ONE));
    split_add1(p + 5, __float2ll_rn((a.z - a0.z) * r * GB_FIX_ONE));
}

// M^-1 J^T lambda of one group into the bodies' class-0 slot (re-formation of
// fc with split classes, where groups of one class may share a body)
__device__ __forceinline__ void apply_desc_fix(const PgsArgs &A, int4 d, long long *dacc, int stride) {
    const bool two = d.w >= 0;
    float4 f1l = make_float4(0.f, 0.f, 0.f, 0.f), f1a = f1l, f2l = f1l, f2a = f1l;
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
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    split_add(dacc, stride, 0, d.z, f1l, f1a, z, z, 1.f);
    if (two) split_add(dacc, stride, 0, d.w, f2l, f2a, z, z, 1.f);
}

// A staged group of split class `cls`: Jacobi inside the class -- the rows
// (packed for mass splitting) relax against the group's own copies of its
// bodies, which start from the class's snapshot.
__device__ __forceinline__ void relax_split(const PgsArgs &A, int4 d, const float4 *buf, float *lam,
                                            float (&lout)[GB_STAGED_ROWS], long long *dacc, int stride, int cls,
                                            int classes) {
    const int off = desc_chunk_off(d);
    const bool two = d.w >= 0;
    float4 s1l, s1a, s2l = make_float4(0.f, 0.f, 0.f, 0.f), s2a = s2l;
    // the classes sharing each body (bit c) and the bodies' shares n, packed
    // into the group's first row; a prefix slot is read only when an earlier
    // class shared the body
    const int m1 = __float_as_int(buf[swz(off, 4)].w), m2 = __float_as_int(buf[swz(off, 6)].w);
    const float n1 = buf[swz(off, 5)].w, n2 = buf[swz(off, 7)].w;
    const int before = (1 << cls) - 1;
    const float4 b1l = ldcg4(&A.fc[2 * d.z]), b1a = ldcg4(&A.fc[2 * d.z + 1]);
    float4 b2l = s2l, b2a = s2a;
    if (two) { b2l = ldcg4(&A.fc[2 * d.w]); b2a = ldcg4(&A.fc[2 * d.w + 1]); }
    s1l = b1l; s1a = b1a; s2l = b2l; s2a = b2a;
    split_sum(dacc, stride, d.z, m1 & before, s1l, s1a);
    if (two) split_sum(dacc, stride, d.w, m2 & before, s2l, s2a);
    float4 f1l = s1l, f1a = s1a, f2l = s2l, f2a = s2a;
    cp_async_wait_all();
    if (d.y & GB_DESC_TRIPLETS) {
        const int nct = desc_rows(d) / 3;
        triplet_rows(A.passes, nct, off, buf, lam, f1l, f1a, f2l, f2a);
#pragma unroll
        for (int k = 0; k < GB_STAGED_ROWS; k++) lout[k] = k < 3 * nct ? lam[k] : 0.f;
    } else {
        plain_rows(A.passes, desc_rows(d), off, buf, lam, f1l, f1a, f2l, f2a);
#pragma unroll
        for (int k = 0; k < GB_STAGED_ROWS; k++) lout[k] = k < desc_rows(d) ? lam[k] : 0.f;
    }
    // shared: the group's share into the later prefix slots; alone: the
    // body's fc plus the group's change (the slots hold only shared changes)
    if (n1 > 1.5f) {
        split_add(dacc, stride, cls, d.z, f1l, f1a, s1l, s1a, n1);
    } else {
        stcg4(&A.fc[2 * d.z], make_float4(b1l.x + (f1l.x - s1l.x), b1l.y + (f1l.y - s1l.y), b1l.z + (f1l.z - s1l.z), b1l.w));
        stcg4(&A.fc[2 * d.z + 1],
              make_float4(b1a.x + (f1a.x - s1a.x), b1a.y + (f1a.y - s1a.y), b1a.z + (f1a.z - s1a.z), b1a.w));
    }
    if (two) {
        if (n2 > 1.5f) {
            split_add(dacc, stride, cls, d.w, f2l, f2a, s2l, s2a, n2);
        } else {
            stcg4(&A.fc[2 * d.w],
                  make_float4(b2l.x + (f2l.x - s2l.x), b2l.y + (f2l.y - s2l.y), b2l.z + (f2l.z - s2l.z), b2l.w));
            stcg4(&A.fc[2 * d.w + 1],
                  make_float4(b2a.x + (f2a.x - s2a.x), b2a.y + (f2a.y - s2a.y), b2a.z + (f2a.z - s2a.z), b2a.w));
        }
    }
}

// quickstep.cpp:2917-3033 on one 80-byte row (the second body's
// accumulators are zero and unused for a one-body contact)
__device__ __forceinline__ void relax_slab_row(const float4 *row, float &lam, float lo, float hi, float4 &f1l,
                                               float4 &f1a, float4 &f2l, float4 &f2a) {
    const float4 q0 = row[0], q1 = row[1], q2 = row[2];
    const float dx = f1l.x - f2l.x, dy = f1l.y - f2l.y, dz = f1l.z - f2l.z;
    float a = fmaf(dx, q0.x, dy * q0.y);
    float b = fmaf(dz, q0.z, f1a.x * q1.x);
    float c = fmaf(f1a.y, q1.y, f1a.z * q1.z);
    a = fmaf(f2a.x, q2.x, a);
    b = fmaf(f2a.y, q2.y, b);
    c = fmaf(f2a.z, q2.z, c);
    const float old = lam;
    float delta = fmaf(-old, q1.w, q0.w) - ((a + b) + c);
    const float nl = old + delta;
    const float cl = fminf(fmaxf(nl, lo), hi);
    if (cl != nl) delta = cl - old;
    lam = cl;
    const float4 q3 = row[3], q4 = row[4];
    const float d1 = delta * q3.w, d2 = delta * q4.w;
    f1l.x = fmaf(d1, q0.x, f1l.x); f1l.y = fmaf(d1, q0.y, f1l.y); f1l.z = fmaf(d1, q0.z, f1l.z);
    f1a.x = fmaf(delta, q3.x, f1a.x); f1a.y = fmaf(delta, q3.y, f1a.y); f1a.z = fmaf(delta, q3.z, f1a.z);
    f2l.x = fmaf(-d2, q0.x, f2l.x); f2l.y = fmaf(-d2, q0.y, f2l.y); f2l.z = fmaf(-d2, q0.z, f2l.z);
    f2a.x = fmaf(delta, q4.x, f2a.x); f2a.y = fmaf(delta, q4.y, f2a.y); f2a.z = fmaf(delta, q4.z, f2a.z);
}

// one interior triplet manifold, all in shared memory
__device__ __forceinline__ void relax_slab(int4 d, const float4 *rows, float *lam, float4 *fc, int passes) {
    const int nct = desc_rows(d) / 3, off = d.w;
    const int lb1 = d.z & 0xffff, lb2 = (d.z >> 16) - 1;
    float4 f1l = fc[2 * lb1], f1a = fc[2 * lb1 + 1];
    float4 f2l = make_float4(0.f, 0.f, 0.f, 0.f), f2a = f2l;
    if (lb2 >= 0) { f2l = fc[2 * lb2]; f2a = fc[2 * lb2 + 1]; }
    const float4 *R = rows + (size_t)off * GB_SLAB_ROW_F4;
    float *L = lam + off;
#pragma unroll 1
    for (int pass = 0; pass < passes; pass++) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (c >= nct) break;
            relax_slab_row(R + 3 * c * GB_SLAB_ROW_F4, L[3 * c], 0.f, R[3 * c * GB_SLAB_ROW_F4 + 2].w, f1l, f1a, f2l,
                           f2a);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (c >= nct) break;
            const float ln = L[3 * c];
#pragma unroll
            for (int q = 1; q < 3; q++) {
                const float4 *row = R + (3 * c + q) * GB_SLAB_ROW_F4;
                const float hi = fabsf(row[2].w * ln);
                relax_slab_row(row, L[3 * c + q], -hi, hi, f1l, f1a, f2l, f2a);
            }
        }
    }
    fc[2 * lb1] = f1l; fc[2 * lb1 + 1] = f1a;
    if (lb2 >= 0) { fc[2 * lb2] = f2l; fc[2 * lb2 + 1] = f2a; }
}

struct SlabArgs {
    PgsArgs A;
    const int *pcstart;   // [parts * 64 + 1]: interior groups per (part, colour), exclusive scan
    const int *irowoff;   // [interior groups]: first row of each in ipack
    const int *irown;     // [interior groups]: rows of each
    const int4 *idesc;    // [interior groups]
    const float4 *ipack;  // interior rows, 5 float4 each, part by part
    const int *pbody, *pbcount;
    int bcap, rcap, gcap;  // per-part capacities: bodies, interior rows, interior groups
    int chunk_cap;         // cross-phase staging rows per buffer
    int ipasses;           // interior phases per sweep (>= 1)
    // neighbour waits (xspatial: the cross colours' groups are listed owner
    // block by owner block; the waits run unless a body's list overflowed)
    int xspatial;
    const int *xcnt;       // [64 * blocks]: cross groups per (colour, block)
    const unsigned *xadj;  // [blocks * GB_XADJ_WORDS]: adjacency bit sets
    unsigned *xprog;       // [blocks]: steps each block has finished
    // split classes (the cross phase's steps are the classes: k_split_*)
    int split;             // classes asked for (the solve uses dc->split_k: 0 exact colours)
    int dstride;           // classes a body's slots hold in dacc (split, or 1 without split classes)
    long long *dacc;       // [bodies * dstride * 6]: class accumulators (zero between sweeps); class 0 also
                           // re-forms the accumulators from the multipliers
    const int *smask;      // [bodies]: the classes whose groups share the body (bit c)
};

// Shared memory of k_pgs_slab: two cross staging buffers (chunk_cap rows of
// 128 B), the part's interior rows (rcap x 80 B), body accumulators
// ((bcap + 1) x 32 B, the last slot zero), interior descriptors (gcap x
// 16 B), interior multipliers (rcap x 4 B), global body ids (bcap x 4 B).
__host__ __device__ __forceinline__ size_t slab_smem_bytes(int chunk_cap, int rcap, int bcap, int gcap) {
    return (size_t)2 * chunk_cap * 128 + (size_t)rcap * 80 + (size_t)(bcap + 1) * 32 + (size_t)gcap * 16 +
           (size_t)rcap * 4 + (size_t)bcap * 4;
}

template <int T>
__global__ void __launch_bounds__(T, 1) k_pgs_slab(SlabArgs S) {
    const PgsArgs &A = S.A;
    unsigned gen = 0;
    DevCounters *dc = A.dc;
    __shared__ int s_cstart[GB_MAX_COLOURS], s_ccount[GB_MAX_COLOURS], s_wcount[GB_MAX_COLOURS],
        s_wbase[GB_MAX_COLOURS];
    __shared__ int s_icol[GB_SLAB_COLOURS + 1];
    __shared__ int s_nic, s_g0, s_ng, s_row0, s_nrows, s_nb;
    __shared__ unsigned long long s_mbar[4];  // two cross buffers, the interior rows, [3] never armed (poison_stage)
    __shared__ int s_abort;                   // a staging or neighbour wait of this block ran out
    __shared__ float s_lam[T * 13];
    __shared__ int s_nbr[256], s_nn;          // blocks whose steps conflict with this block's
    __shared__ int s_xn[GB_SLAB_COLOURS];     // this block's cross groups per colour
    extern __shared__ float4 pgs_smem[];
    float4 *xbuf = pgs_smem;                                         // 2 x chunk_cap x 8
    float4 *irows = xbuf + (size_t)2 * S.chunk_cap * 8;              // rcap x 5
    float4 *ifc = irows + (size_t)S.rcap * GB_SLAB_ROW_F4;           // (bcap + 1) x 2
    int4 *idesc = (int4 *)(ifc + (size_t)(S.bcap + 1) * 2);          // gcap
    float *ilam = (float *)(idesc + S.gcap);                         // rcap
    int *ibid = (int *)(ilam + S.rcap);                              // bcap
    const int ncol = dc->ncolours;   // cross colours
    const int nicol = dc->nicolours; // interior colours (global)
    const int nrows = dc->nrows;
    const int part = blockIdx.x;
    for (int c = threadIdx.x; c < GB_MAX_COLOURS; c += blockDim.x) {
        s_cstart[c] = A.cstart[c];
        s_ccount[c] = A.ccount[c];
        s_wcount[c] = c < ncol ? A.wcount[c * gridDim.x + blockIdx.x] : 1;
        s_wbase[c] = c < ncol ? A.wbase[c * gridDim.x + blockIdx.x] : 0;
    }
    if (threadIdx.x <= GB_SLAB_COLOURS) {
        const int base = S.pcstart[part * GB_SLAB_COLOURS];
        s_icol[threadIdx.x] = S.pcstart[part * GB_SLAB_COLOURS + threadIdx.x] - base;
    }
    const bool nbr = S.xspatial && !dc->slab_nbr_over;  // the same on every block
    const int nsplit = S.split ? dc->split_k : 0;        // classes of the cross phase (0: exact colours)
    if (blockIdx.x == 0 && threadIdx.x == 0) dc->slab_sync = nbr ? 1 : 0;
    if (threadIdx.x < GB_SLAB_COLOURS)
        s_xn[threadIdx.x] = S.xspatial && threadIdx.x < ncol ? S.xcnt[threadIdx.x * gridDim.x + blockIdx.x] : 1;
    if (threadIdx.x == 0) {
        mbar_init(&s_mbar[0]);
        mbar_init(&s_mbar[1]);
        mbar_init(&s_mbar[2]);
        mbar_init(&s_mbar[3]);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const int g0 = S.pcstart[part * GB_SLAB_COLOURS], g1 = S.pcstart[(part + 1) * GB_SLAB_COLOURS];
        s_g0 = g0;
        s_ng = g1 - g0;
        s_row0 = g1 > g0 ? S.irowoff[g0] : 0;
        s_nrows = g1 > g0 ? S.irowoff[g1 - 1] + S.irown[g1 - 1] - s_row0 : 0;
        s_nb = min(S.pbcount[part], S.bcap);
        int n = 0;
        if (nbr)
            for (int w = 0; w < GB_XADJ_WORDS; w++) {
                unsigned m = S.xadj[(size_t)blockIdx.x * GB_XADJ_WORDS + w];
                while (m) {
                    const int o = w * 32 + __ffs(m) - 1;
                    m &= m - 1;
                    if (o != (int)blockIdx.x && o < (int)gridDim.x) s_nbr[n++] = o;
                }
            }
        s_nn = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int n = 0;
        for (int c = 0; c < GB_SLAB_COLOURS; c++)
            if (s_icol[c + 1] > s_icol[c]) n = c + 1;
        s_nic = n;
    }
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const bool residual_mode = A.target > 0;
    const int itmax = nrows > 0 ? (residual_mode ? A.max_iterations : A.iterations) : 0;
    int it = 0, check = 0, last_reform = 0;
    CheckPlan plan;
    plan.init(A.check_every);
    // momentum between sweeps (k_pgs): the columns move their listed bodies'
    // accumulators on, so every body a crossing group touches must be listed
    float mom = (A.lprev && !dc->mom_off) ? A.momentum : 0.f;
    float *slots = dc->racc;
    // fc = M^-1 J^T lambda over every group (cross colours, then interior colours), from global lambda
    auto form_fc = [&](bool zero) -> bool {
        if (S.dacc) {
            // every group's share goes into its bodies' class-0 integer
            // accumulators (2^-32 units: any order gives the same sums, so no
            // barrier per colour, and a split class's groups may share a
            // body), which then replace (or are added to) fc; the slots are
            // zero here (folded before every check, cleared after each use)
            for (int cc = 0; cc < ncol + nicol; cc++) {
                const int c = cc < ncol ? cc : 64 + (cc - ncol);
                for (int k = tid; k < s_ccount[c]; k += nth)
                    apply_desc_fix(A, __ldg(&A.desc[s_cstart[c] + k]), S.dacc, S.dstride);
            }
            if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
            for (int b = tid; b < A.nb; b += nth) {
                float4 fl = make_float4(0.f, 0.f, 0.f, 0.f), fa = fl;
                if (!zero) { fl = ldcg4(&A.fc[2 * b]); fa = ldcg4(&A.fc[2 * b + 1]); }
                float4 gl = make_float4(0.f, 0.f, 0.f, 0.f), ga = gl;
                split_sum(S.dacc, S.dstride, b, 1, gl, ga);  // the class-0 slot
                longlong2 *p = (longlong2 *)split_slot(S.dacc, S.dstride, b, 0);
                const longlong2 zz = make_longlong2(0, 0);
                __stcg(p, zz); __stcg(p + 1, zz); __stcg(p + 2, zz);
                fl.x += gl.x; fl.y += gl.y; fl.z += gl.z;
                fa.x += ga.x; fa.y += ga.y; fa.z += ga.z;
                stcg4(&A.fc[2 * b], fl);
                stcg4(&A.fc[2 * b + 1], fa);
            }
            return grid_sync(&dc->gsync, &dc->err, gen);
        }
        if (zero) {
            for (int b = tid; b < A.nb; b += nth) {
                stcg4(&A.fc[2 * b], make_float4(0.f, 0.f, 0.f, 0.f));
                stcg4(&A.fc[2 * b + 1], make_float4(0.f, 0.f, 0.f, 0.f));
            }
            if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
        }
        for (int cc = 0; cc < ncol + nicol; cc++) {
            const int c = cc < ncol ? cc : 64 + (cc - ncol);
            for (int k = tid; k < s_ccount[c]; k += nth) apply_desc(A, __ldg(&A.desc[s_cstart[c] + k]));
            if (!grid_sync(&dc->gsync, &dc->err, gen)) return false;
        }
        return true;
    };
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
    // the part's interior rows stream in while the start is formed
    if (threadIdx.x == 0) {
        const unsigned bytes = 80u * (unsigned)min(s_nrows, S.rcap);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&s_mbar[2], bytes);
        if (bytes) bulk_g2s(irows, S.ipack + (size_t)s_row0 * GB_SLAB_ROW_F4, bytes, &s_mbar[2]);
    }
    for (int i = threadIdx.x; i < s_ng && i < S.gcap; i += blockDim.x) idesc[i] = S.idesc[s_g0 + i];
    for (int l = threadIdx.x; l < s_nb; l += blockDim.x) ibid[l] = S.pbody[(size_t)part * S.bcap + l];
    if (threadIdx.x < 2) ifc[2 * S.bcap + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    bool ok = true;
    if (A.learned) {
        float r_mlp = 0.f, r_plain = 0.f;
        ok = form_fc(true) && residual_rel(r_mlp) && swap_alt() && form_fc(true) && residual_rel(r_plain);
        const bool use = ok && r_mlp < r_plain;
        if (ok && use) ok = swap_alt() && form_fc(true);
        if (ok && tid == 0) {
            dc->learn_stats[0] = use ? 1.f : 0.f;
            dc->learn_stats[1] = r_mlp;
            dc->learn_stats[2] = r_plain;
        }
    } else if (A.warm) {
        ok = form_fc(false);
    }
    // the copy of the interior rows ends before the block can exit
    if (threadIdx.x == 0) mbar_wait(&s_mbar[2], 0, &dc->err);
    __syncthreads();
    if (!ok) return;
    // interior multipliers and the part's accumulators into shared memory
    auto load_part = [&](bool with_lambda) {
        for (int l = threadIdx.x; l < s_nb; l += blockDim.x) {
            const int b = ibid[l];
            ifc[2 * l] = ldcg4(&A.fc[2 * b]);
            ifc[2 * l + 1] = ldcg4(&A.fc[2 * b + 1]);
        }
        if (with_lambda)
            for (int i = threadIdx.x; i < s_ng; i += blockDim.x) {
                const int4 d = idesc[i];
                for (int k = 0; k < desc_rows(d); k++) ilam[d.w + k] = __ldcg(&A.Rw.lambda[d.x + k]);
            }
    };
    auto publish_fc = [&]() {
        for (int l = threadIdx.x; l < s_nb; l += blockDim.x) {
            const int b = ibid[l];
            stcg4(&A.fc[2 * b], ifc[2 * l]);
            stcg4(&A.fc[2 * b + 1], ifc[2 * l + 1]);
        }
    };
    // split classes: the part's bodies take their class accumulators back
    // (fc += every class's sum, the sums zeroed) and the part's copies are
    // refreshed; runs when every block touching the bodies is done with the
    // sweep's last class
    auto fold_part = [&]() {
        for (int l = threadIdx.x; l < s_nb; l += blockDim.x) {
            const int b = ibid[l];
            float4 fl, fa;
            const int m = S.smask[b];
            if (m) {
                fl = ldcg4(&A.fc[2 * b]);
                fa = ldcg4(&A.fc[2 * b + 1]);
                split_sum(S.dacc, S.split, b, m, fl, fa);  // fc + every class that shared the body
                const longlong2 z = make_longlong2(0, 0);
                for (int c = 0; c < nsplit; c++)
                    if (m >> c & 1) {
                        longlong2 *p = (longlong2 *)split_slot(S.dacc, S.split, b, c);
                        __stcg(p, z); __stcg(p + 1, z); __stcg(p + 2, z);
                    }
                stcg4(&A.fc[2 * b], fl);
                stcg4(&A.fc[2 * b + 1], fa);
            } else {
                fl = ldcg4(&A.fc[2 * b]);
                fa = ldcg4(&A.fc[2 * b + 1]);
            }
            ifc[2 * l] = fl;
            ifc[2 * l + 1] = fa;
        }
    };
    auto publish_lambda = [&]() {
        for (int i = threadIdx.x; i < s_ng; i += blockDim.x) {
            const int4 d = idesc[i];
            for (int k = 0; k < desc_rows(d); k++) __stcg(&A.Rw.lambda[d.x + k], ilam[d.w + k]);
        }
    };
    load_part(true);
    __syncthreads();
    // The sweep is a sequence of steps: the interior phase (c = -1), then the
    // cross colours' waves.  Buffer q & 1 holds step number q's cross chunk
    // (the interior step copies nothing); its use number q >> 1 is the
    // mbarrier phase to wait for.
    struct Step { int c, w; };
    auto step_after = [&](Step t) -> Step {
        if (t.c < 0) return Step{ncol > 0 ? 0 : -1, 0};
        if (t.w + 1 < s_wcount[t.c]) return Step{t.c, t.w + 1};
        return Step{t.c + 1 < ncol ? t.c + 1 : -1, 0};
    };
    unsigned q = 0;
    unsigned nissued = 0, nwaited = 0;
    int pend_start = 0, pend_rows = 0;
    auto chunk_of = [&](Step t) {
        if (t.c < 0) { pend_start = 0; pend_rows = 0; return; }
        const int wv = s_wbase[t.c] + t.w;
        pend_start = __ldg(&A.chunk_start[wv]);
        pend_rows = __ldg(&A.chunk_rows[wv]);
    };
    auto issue = [&](Step t) {
        const unsigned qq = nissued++;
        unsigned long long *m = &s_mbar[qq & 1];
        const unsigned bytes = 128u * (unsigned)min(pend_rows, S.chunk_cap);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(m, bytes);
        if (bytes) bulk_g2s(xbuf + (qq & 1) * (S.chunk_cap * 8), A.packed + (size_t)pend_start * 8, bytes, m);
        chunk_of(step_after(t));
    };
    auto retire = [&]() {
        const unsigned qq = nwaited++;
        return mbar_wait(&s_mbar[qq & 1], (qq >> 1) & 1, &dc->err);
    };
    auto drain = [&]() {
        cp_async_wait_all();
        if (threadIdx.x == 0)
            while (nwaited < nissued) retire();
    };
    float *my_lam = s_lam + threadIdx.x * 13;
    int4 next = make_int4(0, 0, -1, -1), ahead = next;
    bool has_next = false, staged = false, has_ahead = false;
    auto load_ahead = [&](Step t) {
        if (t.c < 0) { has_ahead = false; return; }
        int k = blockIdx.x + threadIdx.x * (int)gridDim.x;
        if (s_wcount[t.c] == 1 && !S.xspatial) k = k < s_ccount[t.c] ? k : -1;
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
            staged = (next.y & GB_DESC_STAGED) && desc_chunk_off(next) + n <= S.chunk_cap;
            if (staged) {
                for (int k = 0; k < n; k++) cp_async4(&my_lam[k], &A.Rw.lambda[next.x + k]);
                cp_async_commit();
            }
        }
        load_ahead(t_after);
    };
    // neighbour waits: `done` counts this block's finished steps (the same
    // sequence on every block); xprog[b] is block b's count
    unsigned done = 0;
    auto nbr_release = [&]() {
        __syncthreads();  // every thread's stores of the step are issued
        ++done;
        if (threadIdx.x == 0) red_release_add_u32(&S.xprog[blockIdx.x], 1u);
    };
    // before a step that touches bodies: every conflicting block has finished
    // as many steps as this one (bounded like a grid barrier)
    auto nbr_wait = [&](bool work) -> bool {
        if (work)
            for (int i = threadIdx.x; i < s_nn; i += blockDim.x) {
                const unsigned *p = &S.xprog[s_nbr[i]];
                long long polls = 0;
                while ((int)(ld_acquire_u32(p) - done) < 0) {
                    if (++polls > (1ll << 22) ||
                        ((polls & 63) == 0 && (ld_acquire_u32(&dc->err) & ERR_BARRIER_TIMEOUT))) {
                        atomicOr(&dc->err, ERR_BARRIER_TIMEOUT);
                        s_abort = 1;
                        break;
                    }
                    __nanosleep(32);
                }
            }
        __syncthreads();
        return s_abort == 0;
    };
    {
        const Step s0{-1, 0};
        if (threadIdx.x == 0) {
            chunk_of(s0);
            issue(s0);
        }
        load_ahead(s0);
        fetch(step_after(s0));
    }
    // momentum: the part's interior multipliers and listed bodies after a sweep
    // (interior groups are triplet manifolds, at most 12 rows; a thread takes
    // its groups two at a time and issues their previous results' loads together)
    auto interior_momentum = [&](float beta) {
        for (int i = threadIdx.x; i < s_ng; i += 2 * blockDim.x) {
            const int i2 = i + blockDim.x;
            const int4 d = idesc[i];
            const int4 e = i2 < s_ng ? idesc[i2] : make_int4(0, 0, 0, 0);  // rows 0: nothing
            const int n = desc_rows(d), m = desc_rows(e);
            float p[GB_STAGED_ROWS] = {}, q[GB_STAGED_ROWS] = {};
            if (beta > 0.f) {
#pragma unroll
                for (int k = 0; k < GB_STAGED_ROWS; k++) {
                    p[k] = k < n ? __ldcg(&A.lprev[d.x + k]) : 0.f;
                    q[k] = k < m ? __ldcg(&A.lprev[e.x + k]) : 0.f;
                }
            }
#pragma unroll
            for (int k = 0; k < GB_STAGED_ROWS; k++) {
                if (k < n) {
                    const float out = ilam[d.w + k];
                    if (beta > 0.f) ilam[d.w + k] = fmaf(beta, out - p[k], out);
                    __stcg(&A.lprev[d.x + k], out);
                }
                if (k < m) {
                    const float out = ilam[e.w + k];
                    if (beta > 0.f) ilam[e.w + k] = fmaf(beta, out - q[k], out);
                    __stcg(&A.lprev[e.x + k], out);
                }
            }
        }
    };
    // (from_global: the accumulators come from global memory, loaded together
    // with the previous values; otherwise from the part's copies)
    auto part_momentum = [&](float beta, bool from_global) {
        for (int l = threadIdx.x; l < s_nb; l += blockDim.x) {
            const int b = ibid[l];
            float4 fl, fa;
            if (from_global) {
                fl = ldcg4(&A.fc[2 * b]);
                fa = ldcg4(&A.fc[2 * b + 1]);
            } else {
                fl = ifc[2 * l];
                fa = ifc[2 * l + 1];
            }
            body_momentum(A, b, fl, fa, beta);
            ifc[2 * l] = fl;
            ifc[2 * l + 1] = fa;
            if (beta > 0.f) {
                stcg4(&A.fc[2 * b], fl);
                stcg4(&A.fc[2 * b + 1], fa);
            }
        }
    };
    for (; it < itmax;) {
        Step cur{-1, 0};
        const bool check_this = residual_mode && (it + 1 >= plan.next || it + 1 == itmax);
        // plain Gauss-Seidel results for the first sweep, the last and every checked one
        const float beta = (mom > 0.f && it > 0 && it + 1 < itmax && !check_this) ? mom : 0.f;
        for (;;) {
            const Step nxt = step_after(cur), nnx = step_after(nxt);
            const bool interior = cur.c < 0;
            const bool last_wave = interior || cur.w + 1 == s_wcount[cur.c];
            if (threadIdx.x == 0 && !last_wave) issue(nxt);
            float lout[GB_STAGED_ROWS];
            float prev[GB_STAGED_ROWS] = {};
            int nout = 0, xout = 0;
            if (interior) {
                if (s_ng > 0) {  // a part without interior groups leaves its bodies' accumulators alone
                    for (int rep = 0; rep < S.ipasses; rep++)
                        for (int c = 0; c < s_nic; c++) {
                            for (int i = s_icol[c] + threadIdx.x; i < s_icol[c + 1]; i += blockDim.x)
                                relax_slab(idesc[i], irows, ilam, ifc, A.passes);
                            __syncthreads();
                        }
                    publish_fc();
                    if (check_this) publish_lambda();
                }
            } else if (has_next) {
                // momentum: the slot's previous-sweep results, loaded together
                // before the relaxation (in flight while the rows arrive and
                // are relaxed)
#pragma unroll
                for (int k = 0; k < GB_STAGED_ROWS; k++)
                    prev[k] = (beta > 0.f && staged && k < desc_rows(next)) ? __ldcg(&A.lprev[next.x + k]) : 0.f;
                if (!staged) {
                    relax_desc(A, next, beta);
                } else if (A.poison_stage ? mbar_wait(&s_mbar[3], 0, &dc->err, 16)
                                          : mbar_wait(&s_mbar[q & 1], (q >> 1) & 1, &dc->err)) {
                    const float4 *buf = xbuf + (q & 1) * (S.chunk_cap * 8);
                    if (nsplit) relax_split(A, next, buf, my_lam, lout, S.dacc, S.split, cur.c, nsplit);
                    else if (next.y & GB_DESC_TRIPLETS) relax_triplets(A, next, buf, my_lam, lout);
                    else relax_plain(A, next, buf, my_lam, lout);
                    nout = desc_rows(next);
                    xout = next.x;
                } else {
                    s_abort = 1;  // the whole block leaves after the next block barrier
                }
            }
            const bool sweep_end = last_wave && nxt.c < 0;
            if (!last_wave) {
                store_staged(A, xout, lout, nout, beta, prev);
                fetch(nnx);
                __syncthreads();
                if (s_abort) { drain(); return; }
            } else {
                const bool check_next = check_this && sweep_end;
                if (check_next) store_staged(A, xout, lout, nout, beta, prev);
                unsigned target = 0;
                if (nbr) nbr_release();
                else grid_arrive(&dc->gsync, gen, target);
                if (threadIdx.x == 0) issue(nxt);
                if (!check_next) store_staged(A, xout, lout, nout, beta, prev);
                // the interior multipliers move on while the other blocks
                // finish the step (read again only in the next interior phase)
                if (interior && mom > 0.f) interior_momentum(beta);
                fetch(nnx);
                // the next step: a cross colour this block has groups in, or
                // the next sweep's interior phase (its accumulators are read
                // back first).  A residual check reads -- and may re-form --
                // every body's accumulators: all blocks finish the sweep first.
                bool ok;
                if (!nbr) {
                    ok = grid_wait(&dc->gsync, &dc->err, gen, target);
                } else if (check_next) {
                    grid_arrive(&dc->gsync, gen, target);
                    ok = grid_wait(&dc->gsync, &dc->err, gen, target);
                } else {
                    ok = nbr_wait(sweep_end ? ((nsplit || mom > 0.f) ? s_nb > 0 : s_ng > 0) : s_xn[nxt.c] > 0);
                }
                if (!ok || s_abort) { drain(); return; }
            }
            if (threadIdx.x == 0) retire();
            ++q;
            if (sweep_end) break;
            cur = nxt;
        }
        ++it;
        if (check_this && nsplit) {
            // the check reads every body's accumulators: the classes' sums go back first
            if (s_nb > 0) fold_part();
            if (!grid_sync(&dc->gsync, &dc->err, gen)) { drain(); return; }
        }
        if (check_this) {
            // as in k_pgs: re-formed accumulators every reform_every sweeps,
            // and for the check that ends the solve
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
        // every block's cross updates of the part's bodies are out (the last
        // barrier or neighbour wait of the sweep, or the check's barrier):
        // the accumulators come back
        if (nsplit) {
            if (s_nb > 0) fold_part();
            if (mom > 0.f && it < itmax) part_momentum(beta, false);
        } else if (mom > 0.f && it < itmax) {
            part_momentum(beta, true);  // reads the accumulators back as load_part does
        } else if (s_ng > 0) {
            load_part(false);
        }
        __syncthreads();
    }
    // The global accumulators are current here (read back after the last
    // sweep's barrier, or formed at the check that ended the solve); the
    // interior multipliers go out for the integration and the warm-start store.
    publish_lambda();
    drain();
    if (tid == 0) {
        dc->iterations = it;
        dc->mom_final = mom;
    }
}
