// Learned warm start: a small MLP that predicts a contact's three multipliers
// (normal + two friction) from twelve local features, as the start of the
// coloured SOR sweeps.
//
//   x (12 raw features) -> standardise -> 128 SiLU -> 128 SiLU -> 128 SiLU -> 3
//
// Parameters (FP32 master copy, this order; GB_MLP_NPARAMS floats):
//   mean[12] std[12] W1[128][12] b1[128] W2[128][128] b2[128]
//   W3[128][128] b3[128] W4[3][128] b4[3]
// Outputs are multipliers in units of the contact's weight scale s (the
// features kernel's m_eff * |g|); targets are the multipliers the plain solver
// reaches after 200 sweeps, in the same units.
//
// Training: one kernel computes the mean-squared-error loss and its gradient
// for a mini-batch (forward and backward through all four layers, FP32, 32
// rows per block in shared memory, weight gradients reduced with atomics),
// one kernel applies Adam.  Inference: a tensor-core kernel (tcgen05.mma,
// kind::f16 with BF16 operands and FP32 accumulators in tensor memory), 128
// contacts per tile, the four layers chained through shared memory.
#include <math.h>
#include <stdint.h>
#include <cuda_bf16.h>

#include <vector>

#include "../../include/gbode.h"
#include "gbode_internal.h"

namespace gb {

static constexpr int NI = GB_MLP_IN, NH = GB_MLP_HIDDEN, NO = GB_MLP_OUT;
static constexpr int OFF_MEAN = 0, OFF_STD = NI, OFF_W1 = 2 * NI, OFF_B1 = OFF_W1 + NH * NI;
static constexpr int OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NH;
static constexpr int OFF_W4 = OFF_B3 + NH, OFF_B4 = OFF_W4 + NO * NH, NPARAMS = OFF_B4 + NO;
static_assert(NPARAMS == GB_MLP_NPARAMS, "parameter layout");

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// ------------------------------------------------------------------ training (FP32)
static constexpr int TR_ROWS = 32;     // rows per block
static constexpr int TR_THREADS = 256;

// out[r][j] = sum_k in[r][k] * W[j][k] + b[j] for TR_ROWS rows; in and out in
// shared memory (row strides lin, lout); W (N x K) staged transposed in wt.
__device__ void tr_dense(const float *in, int lin, int K, const float *W, const float *b, int N, float *out, int lout,
                         float *wt) {
    for (int i = threadIdx.x; i < N * K; i += blockDim.x) {
        const int j = i / K, k = i - j * K;
        wt[k * (NH + 1) + j] = W[i];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TR_ROWS * N; i += blockDim.x) {
        const int r = i / N, j = i - r * N;
        float acc = b[j];
        for (int k = 0; k < K; k++) acc = fmaf(in[r * lin + k], wt[k * (NH + 1) + j], acc);
        out[r * lout + j] = acc;
    }
    __syncthreads();
}

// Backward through one layer: given dZ (TR_ROWS x N, shared), the layer's input
// A (TR_ROWS x K, shared; already activated), accumulate dW (N x K) and db
// into global gradients and, if dA is given, dA = dZ W (TR_ROWS x K).
__device__ void tr_dense_back(const float *dZ, int ldz, const float *A, int lda, int K, const float *W, int N,
                              float *gW, float *gb, float *dA, int ldda) {
    for (int i = threadIdx.x; i < N * K; i += blockDim.x) {
        const int j = i / K, k = i - j * K;
        float acc = 0.f;
        for (int r = 0; r < TR_ROWS; r++) acc = fmaf(dZ[r * ldz + j], A[r * lda + k], acc);
        atomicAdd(&gW[i], acc);
    }
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        float acc = 0.f;
        for (int r = 0; r < TR_ROWS; r++) acc += dZ[r * ldz + j];
        atomicAdd(&gb[j], acc);
    }
    if (dA) {
        for (int i = threadIdx.x; i < TR_ROWS * K; i += blockDim.x) {
            const int r = i / K, k = i - r * K;
            float acc = 0.f;
            for (int j = 0; j < N; j++) acc = fmaf(dZ[r * ldz + j], W[j * K + k], acc);
            dA[r * ldda + k] = acc;
        }
    }
    __syncthreads();
}

// Loss 1/(3n) sum (y_pred - y)^2 over the rows idx[0..n) of (X, Y); gradient
// into grad (zeroed by the caller), loss into *loss (atomic).
__global__ void __launch_bounds__(TR_THREADS) k_mlp_loss_grad(const float *P, const float *X, const float *Y,
                                                              const int *idx, int n, float inv_count, float *grad,
                                                              float *loss) {
    extern __shared__ float sm[];
    const int LD = NH + 1;
    float *x0 = sm;                       // TR_ROWS x NI (standardised input)
    float *z1 = x0 + TR_ROWS * NI;        // TR_ROWS x LD  pre-activations
    float *z2 = z1 + TR_ROWS * LD;
    float *z3 = z2 + TR_ROWS * LD;
    float *a = z3 + TR_ROWS * LD;         // TR_ROWS x LD  scratch activation
    float *d = a + TR_ROWS * LD;          // TR_ROWS x LD  gradient
    float *o = d + TR_ROWS * LD;          // TR_ROWS x 4   outputs
    float *wt = o + TR_ROWS * 4;          // NH x LD       transposed weights
    const int r0 = blockIdx.x * TR_ROWS;
    for (int i = threadIdx.x; i < TR_ROWS * NI; i += blockDim.x) {
        const int r = i / NI, k = i - r * NI;
        float v = 0.f;
        if (r0 + r < n) {
            const int row = idx ? idx[r0 + r] : r0 + r;
            v = (X[(size_t)row * NI + k] - P[OFF_MEAN + k]) / P[OFF_STD + k];
        }
        x0[i] = v;
    }
    __syncthreads();
    auto act = [&](const float *z) {
        for (int i = threadIdx.x; i < TR_ROWS * NH; i += blockDim.x) {
            const int r = i / NH, j = i - r * NH;
            a[r * LD + j] = silu(z[r * LD + j]);
        }
        __syncthreads();
    };
    tr_dense(x0, NI, NI, P + OFF_W1, P + OFF_B1, NH, z1, LD, wt);
    act(z1);
    tr_dense(a, LD, NH, P + OFF_W2, P + OFF_B2, NH, z2, LD, wt);
    act(z2);
    tr_dense(a, LD, NH, P + OFF_W3, P + OFF_B3, NH, z3, LD, wt);
    act(z3);
    tr_dense(a, LD, NH, P + OFF_W4, P + OFF_B4, NO, o, 4, wt);
    // output gradient (rows past n contribute nothing)
    float lsum = 0.f;
    for (int i = threadIdx.x; i < TR_ROWS * NO; i += blockDim.x) {
        const int r = i / NO, j = i - r * NO;
        float g = 0.f;
        if (r0 + r < n) {
            const int row = idx ? idx[r0 + r] : r0 + r;
            const float e = o[r * 4 + j] - Y[(size_t)row * NO + j];
            lsum += e * e;
            g = 2.f * e * inv_count;
        }
        d[r * LD + j] = g;
    }
    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum * inv_count);
    __syncthreads();
    // layer 4: input a = silu(z3)
    float *gW4 = grad + OFF_W4, *gb4 = grad + OFF_B4;
    float *dA = wt;  // reuse the weight buffer as dA (TR_ROWS x LD)
    tr_dense_back(d, LD, a, LD, NH, P + OFF_W4, NO, gW4, gb4, dA, LD);
    auto back_hidden = [&](const float *z, const float *A_in, int lda, int K, const float *W, float *gW, float *gb,
                           bool want_dA) {
        for (int i = threadIdx.x; i < TR_ROWS * NH; i += blockDim.x) {
            const int r = i / NH, j = i - r * NH;
            d[r * LD + j] = dA[r * LD + j] * silu_grad(z[r * LD + j]);
        }
        __syncthreads();
        tr_dense_back(d, LD, A_in, lda, K, W, NH, gW, gb, want_dA ? dA : nullptr, LD);
    };
    // layer 3: input silu(z2)
    act(z2);
    back_hidden(z3, a, LD, NH, P + OFF_W3, grad + OFF_W3, grad + OFF_B3, true);
    act(z1);
    back_hidden(z2, a, LD, NH, P + OFF_W2, grad + OFF_W2, grad + OFF_B2, true);
    back_hidden(z1, x0, NI, NI, P + OFF_W1, grad + OFF_W1, grad + OFF_B1, false);
}

static size_t loss_grad_smem() {
    const int LD = NH + 1;
    return sizeof(float) * ((size_t)TR_ROWS * NI + 5 * (size_t)TR_ROWS * LD + TR_ROWS * 4 + (size_t)NH * LD);
}

// Adam on the trainable parameters (the standardisation is fixed)
__global__ void k_adam(float *P, const float *g, float *m, float *v, int t, float lr, float b1, float b2, float eps) {
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    for (int i = OFF_W1 + blockIdx.x * blockDim.x + threadIdx.x; i < NPARAMS; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// ------------------------------------------------------------------ inference (tcgen05, BF16)
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, element (r, k) of an R x K matrix
// at (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2 with
// SBO = K / 8 * 128.  One tcgen05.mma consumes a K slice of 16 (two core
// matrices along K: LBO = 128 B).
static constexpr int IN_K = 16;  // input features padded to one MMA K step
static constexpr int OUT_N = 16; // outputs padded to the smallest N
static constexpr int TILE_M = 128;
static constexpr int INF_THREADS = 128;

__host__ __device__ __forceinline__ int kmajor_off(int r, int k, int K) {
    return (r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// BF16 operands in the layout above, one buffer: W1 (128 x 16), W2, W3
// (128 x 128), W4 (16 x 128), then FP32 biases b1 b2 b3 (128 each), b4 (16)
// and the standardisation mean/std (16 each).
static constexpr int WB_W1 = 0, WB_W2 = WB_W1 + NH * IN_K * 2, WB_W3 = WB_W2 + NH * NH * 2,
                     WB_W4 = WB_W3 + NH * NH * 2, WB_F32 = WB_W4 + OUT_N * NH * 2;
static constexpr int WB_B1 = 0, WB_B2 = NH, WB_B3 = 2 * NH, WB_B4 = 3 * NH, WB_MEAN = 3 * NH + OUT_N,
                     WB_STD = WB_MEAN + 16, WB_NF32 = WB_STD + 16;
static constexpr int WB_BYTES = WB_F32 + WB_NF32 * 4;  // 75,456 B

__global__ void k_mlp_pack(const float *P, unsigned char *wb) {
    __nv_bfloat16 *w1 = (__nv_bfloat16 *)(wb + WB_W1), *w2 = (__nv_bfloat16 *)(wb + WB_W2),
                  *w3 = (__nv_bfloat16 *)(wb + WB_W3), *w4 = (__nv_bfloat16 *)(wb + WB_W4);
    float *f = (float *)(wb + WB_F32);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int i = tid; i < NH * IN_K; i += nth) {
        const int j = i / IN_K, k = i % IN_K;
        w1[kmajor_off(j, k, IN_K) / 2] = __float2bfloat16_rn(k < NI ? P[OFF_W1 + j * NI + k] : 0.f);
    }
    for (int i = tid; i < NH * NH; i += nth) {
        const int j = i / NH, k = i % NH;
        w2[kmajor_off(j, k, NH) / 2] = __float2bfloat16_rn(P[OFF_W2 + i]);
        w3[kmajor_off(j, k, NH) / 2] = __float2bfloat16_rn(P[OFF_W3 + i]);
    }
    for (int i = tid; i < OUT_N * NH; i += nth) {
        const int j = i / NH, k = i % NH;
        w4[kmajor_off(j, k, NH) / 2] = __float2bfloat16_rn(j < NO ? P[OFF_W4 + j * NH + k] : 0.f);
    }
    for (int i = tid; i < NH; i += nth) {
        f[WB_B1 + i] = P[OFF_B1 + i];
        f[WB_B2 + i] = P[OFF_B2 + i];
        f[WB_B3 + i] = P[OFF_B3 + i];
    }
    for (int i = tid; i < 16; i += nth) {
        f[WB_B4 + i] = i < NO ? P[OFF_B4 + i] : 0.f;
        f[WB_MEAN + i] = i < NI ? P[OFF_MEAN + i] : 0.f;
        f[WB_STD + i] = i < NI ? P[OFF_STD + i] : 1.f;
    }
}

__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor (tcgen05): start, LBO, SBO in 16-byte
// units, bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(const void *p, unsigned lbo, unsigned sbo) {
    unsigned long long d = 0;
    d |= (unsigned long long)((su32(p) >> 4) & 0x3FFF);
    d |= (unsigned long long)((lbo >> 4) & 0x3FFF) << 16;
    d |= (unsigned long long)((sbo >> 4) & 0x3FFF) << 32;
    d |= 1ull << 46;
    return d;
}
// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, N, M
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc,
                                         int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned long long *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(mbar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void async_smem_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init1(unsigned long long *m) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(m)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *m, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 32 consecutive FP32 columns of this thread's TMEM lane (row)
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float *v) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Inference: y[n][3] = MLP(x[n][12]) in units of the weight scale.  Persistent
// blocks of 128 threads, one 128-contact tile at a time; thread t owns row t
// of the tile (its TMEM lane).  Every mbarrier wait is bounded; on a timeout
// the block records ERR_STAGE_TIMEOUT, frees its tensor memory and returns.
__global__ void __launch_bounds__(INF_THREADS, 1) k_mlp_infer(const unsigned char *wb_g, const float *X, int n_host,
                                                              const int *n_dev, float *Y, unsigned *err) {
    const int n = n_dev ? *n_dev : n_host;
    extern __shared__ __align__(128) unsigned char ism[];
    unsigned char *w1 = ism + WB_W1, *w2 = ism + WB_W2, *w3 = ism + WB_W3, *w4 = ism + WB_W4;
    const float *f = (const float *)(ism + WB_F32);
    unsigned char *act = ism + WB_BYTES;  // TILE_M x NH BF16 activations (also the 128 x 16 input)
    __shared__ unsigned long long mbar;
    __shared__ unsigned tmem_base;
    __shared__ int abort_s;
    const int t = threadIdx.x, warp = t >> 5;
    // stage the weights (16-byte copies)
    for (int i = t; i < WB_BYTES / 16; i += blockDim.x) ((int4 *)ism)[i] = ((const int4 *)wb_g)[i];
    if (t == 0) {
        mbar_init1(&mbar);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abort_s = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base)),
                     "r"(NH)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    async_smem_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base;
    const unsigned lane_addr = tmem + ((unsigned)(warp * 32) << 16);
    unsigned phase = 0;
    const unsigned id_hidden = idesc_bf16(TILE_M, NH), id_out = idesc_bf16(TILE_M, OUT_N);

    // one layer: D(TMEM) = act(K) x W^T, issued by thread 0, completion awaited by all
    auto run_layer = [&](const unsigned char *wsm, int K, unsigned idesc) -> bool {
        async_smem_fence();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            const unsigned sbo = (unsigned)(K / 8) * 128u;
            for (int k0 = 0; k0 < K; k0 += 16) {
                const unsigned long long a = smem_desc(act + k0 * 16, 128, sbo);
                const unsigned long long b = smem_desc(wsm + k0 * 16, 128, sbo);
                mma_bf16(tmem, a, b, idesc, k0 > 0);
            }
            mma_commit(&mbar);
        }
        long long tries = 0;
        bool ok = true;
        while (!mbar_test(&mbar, phase)) {
            if (++tries > (1ll << 20)) { ok = false; break; }
        }
        if (!ok) {
            atomicOr(err, ERR_STAGE_TIMEOUT);
            abort_s = 1;
        }
        phase ^= 1u;
        tc_fence_after();
        __syncthreads();
        return abort_s == 0;
    };
    // epilogue of a hidden layer: this thread's row, bias + SiLU, BF16, into act
    auto hidden_epilogue = [&](const float *bias) {
        float v[32];
        for (int c0 = 0; c0 < NH; c0 += 32) {
            tmem_ld32(lane_addr + c0, v);
#pragma unroll
            for (int i = 0; i < 32; i += 2) {
                const float a0 = silu(v[i] + bias[c0 + i]), a1 = silu(v[i + 1] + bias[c0 + i + 1]);
                *(__nv_bfloat162 *)(act + kmajor_off(t, c0 + i, NH)) = __floats2bfloat162_rn(a0, a1);
            }
        }
    };
    const int ntiles = (n + TILE_M - 1) / TILE_M;
    bool alive = true;
    for (int tile = blockIdx.x; tile < ntiles && alive; tile += gridDim.x) {
        const int row = tile * TILE_M + t;
        // input: standardised features, padded to 16 with zeros
        {
            float x[IN_K];
#pragma unroll
            for (int k = 0; k < IN_K; k++) {
                const float raw = (row < n && k < NI) ? X[(size_t)row * NI + k] : 0.f;
                x[k] = k < NI ? (raw - f[WB_MEAN + k]) / f[WB_STD + k] : 0.f;
            }
#pragma unroll
            for (int k = 0; k < IN_K; k += 2)
                *(__nv_bfloat162 *)(act + kmajor_off(t, k, IN_K)) = __floats2bfloat162_rn(x[k], x[k + 1]);
        }
        if (!(alive = run_layer(w1, IN_K, id_hidden))) break;
        tc_fence_before();
        __syncthreads();  // every thread has read its input row before act is overwritten
        hidden_epilogue(f + WB_B1);
        if (!(alive = run_layer(w2, NH, id_hidden))) break;
        hidden_epilogue(f + WB_B2);
        if (!(alive = run_layer(w3, NH, id_hidden))) break;
        hidden_epilogue(f + WB_B3);
        if (!(alive = run_layer(w4, NH, id_out))) break;
        {
            float v[32];
            tmem_ld32(lane_addr, v);
            if (row < n)
                for (int j = 0; j < NO; j++) Y[(size_t)row * NO + j] = v[j] + f[WB_B4 + j];
        }
        tc_fence_before();
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NH) : "memory");
}

static size_t infer_smem() { return (size_t)WB_BYTES + (size_t)TILE_M * NH * 2; }

// ------------------------------------------------------------------ host side
bool mlp_pack(const float *P_dev, unsigned char *wb_dev, cudaStream_t s) {
    k_mlp_pack<<<64, 256, 0, s>>>(P_dev, wb_dev);
    count_launch();
    return cudaGetLastError() == cudaSuccess;
}

bool mlp_infer(const unsigned char *wb_dev, const float *X, int n, const int *n_dev, float *Y, unsigned *err,
               cudaStream_t s) {
    static bool attr = false;
    const size_t smem = infer_smem();
    if (!attr) {
        if (cudaFuncSetAttribute((const void *)k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return false;
        attr = true;
    }
    int grid = num_sms();
    if (!n_dev) {
        if (n <= 0) return true;
        const int tiles = (n + TILE_M - 1) / TILE_M;
        if (grid > tiles) grid = tiles;
    }
    k_mlp_infer<<<grid, INF_THREADS, smem, s>>>(wb_dev, X, n, n_dev, Y, err);
    count_launch();
    return cudaGetLastError() == cudaSuccess;
}

size_t mlp_wb_bytes() { return WB_BYTES; }

}  // namespace gb

// ------------------------------------------------------------------ C ABI
using namespace gb;

namespace {
struct DevArray {
    void *p = nullptr;
    ~DevArray() { if (p) cudaFree(p); }
    bool alloc(size_t bytes) { return cudaMalloc(&p, bytes > 0 ? bytes : 16) == cudaSuccess; }
    template <class T> T *as() const { return (T *)p; }
};
bool upload(DevArray &d, const void *h, size_t bytes) {
    return d.alloc(bytes) && cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
}
}  // namespace

extern "C" int gbodeMlpParamCount(void) { return NPARAMS; }

extern "C" int gbodeMlpLossGrad(const float *params, const float *X, const float *Y, int n, float *grad, float *loss) {
    if (!params || !X || !Y || !grad || !loss || n <= 0) { report_error("gbodeMlpLossGrad: bad argument"); return 0; }
    DevArray P, dX, dY, dG, dL;
    if (!(upload(P, params, NPARAMS * 4) && upload(dX, X, (size_t)n * NI * 4) && upload(dY, Y, (size_t)n * NO * 4) &&
          dG.alloc(NPARAMS * 4) && dL.alloc(4))) {
        report_error("gbodeMlpLossGrad: device allocation");
        return 0;
    }
    cudaMemset(dG.p, 0, NPARAMS * 4);
    cudaMemset(dL.p, 0, 4);
    const size_t smem = loss_grad_smem();
    cudaFuncSetAttribute((const void *)k_mlp_loss_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mlp_loss_grad<<<(n + TR_ROWS - 1) / TR_ROWS, TR_THREADS, smem>>>(P.as<float>(), dX.as<float>(), dY.as<float>(),
                                                                       nullptr, n, 1.f / (3.f * n), dG.as<float>(),
                                                                       dL.as<float>());
    count_launch();
    if (cudaMemcpy(grad, dG.p, NPARAMS * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(loss, dL.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
        report_error("gbodeMlpLossGrad: kernel failed");
        return 0;
    }
    return 1;
}

extern "C" int gbodeMlpTrain(const float *X, const float *Y, int n, int epochs, int batch, float lr, unsigned seed,
                             float *params, float *loss_per_epoch) {
    if (!X || !Y || !params || n <= 0 || epochs <= 0 || batch <= 0) {
        report_error("gbodeMlpTrain: bad argument");
        return 0;
    }
    DevArray P, dX, dY, dG, dM, dV, dL, dIdx;
    if (!(upload(P, params, NPARAMS * 4) && upload(dX, X, (size_t)n * NI * 4) && upload(dY, Y, (size_t)n * NO * 4) &&
          dG.alloc(NPARAMS * 4) && dM.alloc(NPARAMS * 4) && dV.alloc(NPARAMS * 4) && dL.alloc(4) &&
          dIdx.alloc((size_t)n * 4))) {
        report_error("gbodeMlpTrain: device allocation");
        return 0;
    }
    cudaMemset(dM.p, 0, NPARAMS * 4);
    cudaMemset(dV.p, 0, NPARAMS * 4);
    const size_t smem = loss_grad_smem();
    cudaFuncSetAttribute((const void *)k_mlp_loss_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd = [&]() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; };
    int step = 0;
    for (int e = 0; e < epochs; e++) {
        for (int i = n - 1; i > 0; i--) { const int j = (int)(rnd() % (unsigned long long)(i + 1)); std::swap(idx[i], idx[j]); }
        cudaMemcpy(dIdx.p, idx.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
        cudaMemset(dL.p, 0, 4);
        const int nb = (n + batch - 1) / batch;
        for (int b = 0; b < nb; b++) {
            const int b0 = b * batch, bn = b0 + batch <= n ? batch : n - b0;
            cudaMemsetAsync(dG.p, 0, NPARAMS * 4);
            // the loss accumulates the per-batch means; divided by nb below
            k_mlp_loss_grad<<<(bn + TR_ROWS - 1) / TR_ROWS, TR_THREADS, smem>>>(
                P.as<float>(), dX.as<float>(), dY.as<float>(), dIdx.as<int>() + b0, bn, 1.f / (3.f * bn),
                dG.as<float>(), dL.as<float>());
            k_adam<<<64, 256>>>(P.as<float>(), dG.as<float>(), dM.as<float>(), dV.as<float>(), ++step, lr, 0.9f, 0.999f,
                                1e-8f);
            count_launch(2);
        }
        float l = 0.f;
        if (cudaMemcpy(&l, dL.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
            report_error("gbodeMlpTrain: kernel failed");
            return 0;
        }
        if (loss_per_epoch) loss_per_epoch[e] = l / nb;
    }
    if (cudaMemcpy(params, P.p, NPARAMS * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
        report_error("gbodeMlpTrain: kernel failed");
        return 0;
    }
    return 1;
}

extern "C" int gbodeMlpPredict(const float *params, const float *X, int n, float *Y) {
    if (!params || !X || !Y || n <= 0) { report_error("gbodeMlpPredict: bad argument"); return 0; }
    DevArray P, WB, dX, dY, dE;
    if (!(upload(P, params, NPARAMS * 4) && WB.alloc(WB_BYTES) && upload(dX, X, (size_t)n * NI * 4) &&
          dY.alloc((size_t)n * NO * 4) && dE.alloc(4))) {
        report_error("gbodeMlpPredict: device allocation");
        return 0;
    }
    cudaMemset(dE.p, 0, 4);
    if (!mlp_pack(P.as<float>(), WB.as<unsigned char>(), 0) ||
        !mlp_infer(WB.as<unsigned char>(), dX.as<float>(), n, nullptr, dY.as<float>(), dE.as<unsigned>(), 0)) {
        report_error("gbodeMlpPredict: launch failed");
        return 0;
    }
    unsigned e = 0;
    if (cudaMemcpy(Y, dY.p, (size_t)n * NO * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&e, dE.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess || e) {
        report_error("gbodeMlpPredict: kernel failed");
        return 0;
    }
    return 1;
}
