// Exclusive prefix sums whose length lives in device memory, so a step can
// size its work without a host round trip.  Three launches: per-block scan,
// scan of block totals in one block, add-back.  Deterministic.
#include "gbode_internal.h"

namespace gb {

static constexpr int SCAN_BLOCK = 1024;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ __forceinline__ int block_excl_scan(int v, int *total) {
    __shared__ int wsum[SCAN_BLOCK / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int x = lane < (blockDim.x >> 5) ? wsum[lane] : 0;
        int xi = warp_incl_scan(x);
        if (lane < (blockDim.x >> 5)) wsum[lane] = xi - x;
        if (lane == (blockDim.x >> 5) - 1) *total = xi;
    }
    __syncthreads();
    int r = inc - v + wsum[wid];
    __syncthreads();
    return r;
}

__global__ void k_scan_blocks(const int *in, int *out, const int *n_dev, int n_host, int *block_sums) {
    const int n = n_dev ? *n_dev : n_host;
    const int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if ((int)(blockIdx.x * SCAN_BLOCK) >= n) return;  // whole block idle
    int v = i < n ? in[i] : 0;
    __shared__ int tot;
    int e = block_excl_scan(v, &tot);
    if (i < n) out[i] = e;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int *block_sums, const int *n_dev, int n_host, int *total_dev) {
    const int n = n_dev ? *n_dev : n_host;
    const int nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    __shared__ int carry_s;
    __shared__ int tot;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += SCAN_BLOCK) {
        int i = base + threadIdx.x;
        int v = i < nb ? block_sums[i] : 0;
        int e = block_excl_scan(v, &tot);
        int carry = carry_s;
        if (i < nb) block_sums[i] = e + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_dev) *total_dev = carry_s;
}

__global__ void k_scan_add(int *out, const int *n_dev, int n_host, const int *block_sums) {
    const int n = n_dev ? *n_dev : n_host;
    const int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

// One block, no scratch: the same exclusive scan in SCAN_BLOCK-element
// tiles with a carry (used when the scratch of the fast path cannot grow).
__global__ void k_scan_single(const int *in, int *out, const int *n_dev, int n_host, int *total_dev) {
    const int n = n_dev ? *n_dev : n_host;
    __shared__ int carry_s;
    __shared__ int tot;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n; base += SCAN_BLOCK) {
        const int i = base + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        const int e = block_excl_scan(v, &tot);
        const int carry = carry_s;
        if (i < n) out[i] = e + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_dev) *total_dev = carry_s;
}

void scan_exclusive(const int *in, int *out, const int *n_dev, int n_cap, int *total_dev, Workspace &ws,
                    cudaStream_t s) {
    int nblocks = (n_cap + SCAN_BLOCK - 1) / SCAN_BLOCK;
    if (nblocks < 1) nblocks = 1;
    if (!ws.scan_tmp.ensure(sizeof(int) * (size_t)(nblocks + 1))) {
        k_scan_single<<<1, SCAN_BLOCK, 0, s>>>(in, out, n_dev, n_cap, total_dev);
        count_launch();
        return;
    }
    int *sums = ws.scan_tmp.as<int>();
    k_scan_blocks<<<nblocks, SCAN_BLOCK, 0, s>>>(in, out, n_dev, n_cap, sums);
    k_scan_sums<<<1, SCAN_BLOCK, 0, s>>>(sums, n_dev, n_cap, total_dev);
    k_scan_add<<<nblocks, SCAN_BLOCK, 0, s>>>(out, n_dev, n_cap, sums);
    count_launch(3);
}

}  // namespace gb
