// gbodeCollidePairsNoAlloc: the narrow phase for a caller's batch of geom
// pairs, with every temporary it needs in one fixed-size device array that the
// library holds from load to exit, so a call allocates nothing.
//
// Who needs it: a program that manages all of its device memory itself, e.g.
// an engine or a controller that reserves its GPU memory once at start-up and
// must not call cudaMalloc / cudaFree afterwards -- cudaFree synchronises the
// whole device, either call can fail half-way through a frame with a fixed
// deadline, and some hosts run the physics inside a memory budget that the
// library cannot see.  Such a caller passes device buffers it already owns for
// the inputs and outputs; the per-pair contact slots and counts this kernel
// needs in between live in `g_noalloc_scratch` below.
//
// The kernel is the library's narrow phase (k_narrow in collide.cu: one thread
// per pair, dCollide restated from collision_kernel.cpp:292-338) writing into
// the fixed array instead of workspace buffers, followed by a one-block
// exclusive scan of the per-pair counts and a compaction into the caller's
// contact array, all enqueued on the caller's stream.
#include <cstdint>
#include <mutex>

#include "colliders.cuh"
#include "gbode_internal.h"
#include "../../include/gbode.h"

namespace gb {

// Every contact slot is two float4 (pos xyz + depth, normal xyz + 0); each
// pair has 8 slots (the largest contact count of any collider) and one int
// count.  GBODE_NOALLOC_MAX_PAIRS pairs: 8192 * (8 * 32 + 4) B = 2.03 MiB.
static constexpr int NA_SLOTS = 8;
static constexpr size_t NA_SLOT_F4 = (size_t)GBODE_NOALLOC_MAX_PAIRS * NA_SLOTS * 2;
static constexpr size_t NA_COUNT_F4 = (size_t)GBODE_NOALLOC_MAX_PAIRS / 4;

// The scratch itself.  Host code must never hand this name to a kernel: on
// the host it is only a stand-in for the symbol; its device address comes from
// cudaGetSymbolAddress (scratch_ptr below).
static __device__ __align__(256) float4 g_noalloc_scratch[NA_SLOT_F4 + NA_COUNT_F4];

static_assert(GBODE_NOALLOC_MAX_PAIRS % 4 == 0, "count area is a whole number of float4");

__global__ void k_narrow_noalloc(const gbodePairGeom *geoms, int ngeoms, const int2 *pairs, int np, int maxc,
                                 float4 *slots, int *count) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int2 pr = pairs[p];
        int n = 0, code = -1;
        CPoint c[8];
        // dCollide's rejections (collision_kernel.cpp:305-310): a geom with
        // itself, two geoms on one body; pairs naming no geom give nothing
        const bool valid = pr.x >= 0 && pr.y >= 0 && pr.x < ngeoms && pr.y < ngeoms;
        if (valid && pr.x != pr.y && !(geoms[pr.x].body >= 0 && geoms[pr.x].body == geoms[pr.y].body)) {
            GeomView v[2];
            const int ids[2] = {pr.x, pr.y};
            for (int s = 0; s < 2; s++) {
                const gbodePairGeom &g = geoms[ids[s]];
                v[s].cls = g.cls;
                for (int k = 0; k < 3; k++) v[s].pos[k] = g.pos[k];
                v[s].pos[3] = 0.f;
                for (int k = 0; k < 12; k++) v[s].R[k] = (k & 3) == 3 ? 0.f : g.R[k];
                for (int k = 0; k < 4; k++) v[s].dims[k] = g.dims[k];
            }
            n = collide_pair(v[0], v[1], maxc, c, &code);
        }
        count[p] = n;
        for (int i = 0; i < n; i++) {
            slots[((size_t)p * NA_SLOTS + i) * 2] = make_float4(c[i].pos[0], c[i].pos[1], c[i].pos[2], c[i].depth);
            slots[((size_t)p * NA_SLOTS + i) * 2 + 1] = make_float4(c[i].normal[0], c[i].normal[1], c[i].normal[2], 0.f);
        }
    }
}

// One block of 1024 threads: first[p] = sum of count[0..p), first[np] = total.
__global__ void k_scan_noalloc(const int *count, int np, int *first) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < np; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < np ? count[i] : 0;
        int inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            const int x = wsum[lane];
            int xi = x;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, xi, o);
                if (lane >= o) xi += t;
            }
            wsum[lane] = xi - x;
        }
        __syncthreads();
        const int c0 = carry;
        if (i < np) first[i] = c0 + wsum[wid] + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = c0 + wsum[wid] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) first[np] = carry;
}

__global__ void k_compact_noalloc(const float4 *slots, const int *count, const int *first, int np, float *out,
                                  int capacity) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int n = count[p], o = first[p];
        for (int i = 0; i < n && o + i < capacity; i++) {
            const float4 a = slots[((size_t)p * NA_SLOTS + i) * 2], b = slots[((size_t)p * NA_SLOTS + i) * 2 + 1];
            float *d = out + (size_t)(o + i) * 8;
            d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
            d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = 0.f;
        }
    }
}

// Device address of the scratch on the current device, looked up once per
// device (cudaGetSymbolAddress may load the module on that device, so the
// first call on a device does real set-up work).
static float4 *scratch_ptr(const char **why) {
    static std::mutex mu;
    static float4 *addr[64] = {};
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) { *why = "no current CUDA device"; return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) { *why = cudaGetErrorString(e); return nullptr; }
        addr[dev] = (float4 *)p;
    }
    return addr[dev];
}

}  // namespace gb

extern "C" int gbodeCollidePairsNoAlloc(const gbodePairGeom *geoms, int ngeoms, const int *pairs, int npairs, int flags,
                                        float *contacts, int capacity, int *first, void *stream) {
    using namespace gb;
    char msg[192];
    if (npairs < 0 || npairs > GBODE_NOALLOC_MAX_PAIRS) {
        snprintf(msg, sizeof msg, "gbodeCollidePairsNoAlloc: %d pairs, the fixed scratch holds at most %d", npairs,
                 GBODE_NOALLOC_MAX_PAIRS);
        report_error(msg);
        return 0;
    }
    if (ngeoms < 0 || capacity < 0 || (npairs > 0 && (!geoms || !pairs)) || !first || (capacity > 0 && !contacts)) {
        report_error("gbodeCollidePairsNoAlloc: null buffer or negative size");
        return 0;
    }
    // the kernel reads a pair as one 8-byte int2; a misaligned pointer would
    // fault on the device, so it is refused here
    if (((uintptr_t)pairs & 7) != 0) {
        report_error("gbodeCollidePairsNoAlloc: pairs must be 8-byte aligned");
        return 0;
    }
    const char *why = "";
    float4 *scratch = scratch_ptr(&why);
    if (!scratch) {
        snprintf(msg, sizeof msg, "gbodeCollidePairsNoAlloc: cudaGetSymbolAddress failed: %s", why);
        report_error(msg);
        return 0;
    }
    float4 *slots = scratch;
    int *count = (int *)(scratch + NA_SLOT_F4);
    cudaStream_t s = (cudaStream_t)stream;
    int maxc = flags & GB_NUMC_MASK;
    if (maxc > NA_SLOTS) maxc = NA_SLOTS;
    const int grid = npairs > 0 ? (npairs + 127) / 128 : 1;
    // an error left pending on this thread by unrelated earlier work would
    // otherwise be reported (and cleared) as this call's launch failure
    (void)cudaGetLastError();
    // every count[p] and slot this call reads is written by this call first:
    // nothing in the scratch has to start at zero
    if (npairs > 0) {
        k_narrow_noalloc<<<grid, 128, 0, s>>>(geoms, ngeoms, (const int2 *)pairs, npairs, maxc, slots, count);
    }
    k_scan_noalloc<<<1, 1024, 0, s>>>(count, npairs, first);
    if (npairs > 0) k_compact_noalloc<<<grid, 128, 0, s>>>(slots, count, first, npairs, contacts, capacity);
    count_launch(npairs > 0 ? 3 : 1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "gbodeCollidePairsNoAlloc: launch failed: %s", cudaGetErrorString(e));
        report_error(msg);
        return 0;
    }
    return 1;
}
