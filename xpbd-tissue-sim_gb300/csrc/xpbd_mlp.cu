// Per-tet warm-start MLP (14 -> 64 -> 64 -> 64 -> 2, SiLU) on the 5th-gen
// tensor cores: BF16 operands in shared memory, FP32 accumulators in tensor
// memory (tcgen05.mma / tcgen05.commit / tcgen05.ld), training by hand-written
// forward, backward and Adam kernels.
//
// Operand layout (shared memory, no swizzle, K-major canonical): an R x K BF16
// tile is a grid of 8-row x 16-byte core matrices; core (r/8, k/8) starts at
// (r/8) * SBO + (k/8) * LBO with LBO = 128 B, SBO = (K/8) * 128 B, and element
// (r, k) sits at (r%8) * 16 + (k%8) * 2 inside it. D = A * B^T with A (M x K)
// and B (N x K) both K-major; one MMA covers K = 16, so a K-step advances both
// descriptors' start addresses by 2 core matrices (256 B).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xpbd_kernels.cuh"

namespace xg {

namespace {

constexpr int kRows = 128;  // tets per tile (MMA M)
constexpr int kHid = 64;
constexpr int kIn = 16;     // 14 features, zero padded
constexpr int kOutPad = 16; // 2 outputs padded to the smallest N for M = 128
constexpr unsigned kLimit = 1u << 22;

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned kmaj_off(int r, int k, int K) {
    return (unsigned)((r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint64_t smem_desc(const void* base, int K) {
    const uint64_t addr = su32(base);
    const uint64_t lbo = 128, sbo = (uint64_t)(K >> 3) * 128;
    return ((addr & 0x3FFFFull) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D F32, A/B BF16, both K-major, M = 128
__device__ __forceinline__ uint32_t idesc_bf16(int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);
}

__device__ __forceinline__ void umma(unsigned tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::
            "r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

// D (tmem columns from tmem_d) = A (128 x K) * B (N x K)^T, accumulating onto
// D when acc; issued by one thread.
__device__ __forceinline__ void mma_tile(unsigned tmem_d, const void* A, const void* B, int K, int N, bool acc) {
    const uint32_t id = idesc_bf16(N);
    for (int s = 0; s < K / 16; s++)
        umma(tmem_d, smem_desc((const char*)A + 256 * s, K), smem_desc((const char*)B + 256 * s, K), id,
             (s > 0 || acc) ? 1 : 0);
}

__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void async_smem_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool bar_wait(unsigned long long* bar, unsigned parity) {
    for (unsigned i = 0; i < kLimit; i++) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_alloc(unsigned* dst, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (warp w reads lanes 32w..32w+31)
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float* v) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// SiLU through sigmoid(z) = (1 + tanh(z / 2)) / 2 with the one-instruction
// PTX tanh.approx: one MUFU operation per activation instead of two (an
// exponential and a reciprocal). The epilogue of a 1.3M-row launch does 192
// activations per row, and the MUFU rate, not the tensor pipe, bounds it. The
// approximation's relative error (about 2^-11) is below the BF16 rounding
// that every activation then takes.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid_f(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu_f(float z) { return z * sigmoid_f(z); }
__device__ __forceinline__ float dsilu_f(float z) {
    const float s = sigmoid_f(z);
    return s * (1.f + z * (1.f - s));
}

// 8 consecutive K values of row r as one 16-byte store into a K-major tile
__device__ __forceinline__ void st_row8(char* tile, int r, int k0, int K, const float* v) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(tile + kmaj_off(r, k0, K)) = *reinterpret_cast<const uint4*>(h);
}

__device__ __forceinline__ void st_one(char* tile, int r, int k, int K, float v) {
    *reinterpret_cast<__nv_bfloat16*>(tile + kmaj_off(r, k, K)) = __float2bfloat16_rn(v);
}

// warp sum of v added to a shared-memory accumulator by lane 0
__device__ __forceinline__ void warp_add(float* dst, float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, v);
}

// zero a byte range of shared memory cooperatively
__device__ __forceinline__ void zero_smem(char* p, int bytes) {
    for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16) *reinterpret_cast<uint4*>(p + i) = make_uint4(0, 0, 0, 0);
}

__device__ __forceinline__ void copy_smem(char* dst, const char* src, int bytes) {
    for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16)
        *reinterpret_cast<uint4*>(dst + i) = __ldg(reinterpret_cast<const uint4*>(src + i));
}

constexpr int kW1Bytes = kHid * kIn * 2;       // 64 x 16
constexpr int kW2Bytes = kHid * kHid * 2;      // 64 x 64
constexpr int kW4Bytes = kOutPad * kHid * 2;   // 16 x 64
constexpr int kA0Bytes = kRows * kIn * 2;      // 128 x 16
constexpr int kABytes = kRows * kHid * 2;      // 128 x 64

// ---- forward: persistent CTAs, one 128-tet tile at a time ----
// Smem: W1 | W2 | W3 | W4 | A0 | A  (+ biases, barrier, tmem address). The
// weights and biases are staged once per CTA; each tile's input rows are
// loaded into registers while the previous tile is computed. Eight warps:
// warp w reads tensor-memory lanes 32 (w % 4) .. +31 (its rows) and runs the
// epilogue of hidden columns 32 (w / 4) .. +31.
constexpr int kFwdSmem = kW1Bytes + 2 * kW2Bytes + kW4Bytes + kA0Bytes + kABytes;
constexpr int kFwdThreads = 2 * kRows;

template <bool TRAIN>
__global__ void __launch_bounds__(kFwdThreads) k_mlp_forward(const __nv_bfloat16* __restrict__ X, int n, MlpNet net,
                                                       float* __restrict__ out, MlpCache cache,
                                                       unsigned long long* __restrict__ err) {
    extern __shared__ __align__(128) char smem[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ unsigned s_tmem;
    __shared__ __align__(16) float s_b[3 * kHid + 2];
    char* W1 = smem;
    char* W2 = W1 + kW1Bytes;
    char* W3 = W2 + kW2Bytes;
    char* W4 = W3 + kW2Bytes;
    char* A0 = W4 + kW4Bytes;
    char* A = A0 + kA0Bytes;
    const int warp = threadIdx.x >> 5;
    const int t = (warp & 3) * 32 + (threadIdx.x & 31);  // row within the tile
    const int half = warp >> 2;                           // hidden columns 32 half .. +31
    const int ntiles = (n + kRows - 1) / kRows;
    copy_smem(W1, (const char*)net.w1, kW1Bytes);
    copy_smem(W2, (const char*)net.w2, kW2Bytes);
    copy_smem(W3, (const char*)net.w3, kW2Bytes);
    copy_smem(W4, (const char*)net.w4, kW4Bytes);
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
        s_b[i] = __ldg(net.b1 + i);
        s_b[kHid + i] = __ldg(net.b2 + i);
        s_b[2 * kHid + i] = __ldg(net.b3 + i);
    }
    if (threadIdx.x < 2) s_b[3 * kHid + threadIdx.x] = __ldg(net.b4 + threadIdx.x);
    if (threadIdx.x == 0) bar_init(&bar);
    if (warp == 0) tmem_alloc(&s_tmem, 64);
    tc_before();
    __syncthreads();
    tc_after();
    const unsigned tmem = s_tmem;
    const unsigned my_lane = tmem + ((unsigned)(32 * (warp & 3)) << 16);
    unsigned phase = 0;
    bool ok = true;
    // this thread's input row of the first tile
    uint4 xa = make_uint4(0, 0, 0, 0), xb = make_uint4(0, 0, 0, 0);
    {
        const int row = blockIdx.x * kRows + t;
        if (half == 0 && blockIdx.x < ntiles && row < n) {
            xa = __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * kIn));
            xb = __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * kIn + 8));
        }
    }
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int row = tile * kRows + t;
        const bool live = row < n;
        if (half == 0) {
            *reinterpret_cast<uint4*>(A0 + kmaj_off(t, 0, kIn)) = xa;
            *reinterpret_cast<uint4*>(A0 + kmaj_off(t, 8, kIn)) = xb;
        }
        // next tile's row: in flight while this tile is computed
        {
            const int nrow = (tile + gridDim.x) * kRows + t;
            xa = make_uint4(0, 0, 0, 0);
            xb = make_uint4(0, 0, 0, 0);
            if (half == 0 && tile + (int)gridDim.x < ntiles && nrow < n) {
                xa = __ldg(reinterpret_cast<const uint4*>(X + (size_t)nrow * kIn));
                xb = __ldg(reinterpret_cast<const uint4*>(X + (size_t)nrow * kIn + 8));
            }
        }
        async_smem_fence();
        tc_before();
        __syncthreads();
        tc_after();
#pragma unroll
        for (int layer = 0; layer < 4; layer++) {
            const int K = layer == 0 ? kIn : kHid;
            const int N = layer == 3 ? kOutPad : kHid;
            const char* Wl = layer == 0 ? W1 : (layer == 1 ? W2 : (layer == 2 ? W3 : W4));
            if (threadIdx.x == 0) {
                mma_tile(tmem, layer == 0 ? A0 : A, Wl, K, N, false);
                umma_commit(&bar);
            }
            // every thread polls; the block agrees on the outcome
            ok = __syncthreads_and(bar_wait(&bar, phase)) != 0;
            phase ^= 1u;
            tc_after();
            if (!ok) break;
            if (layer < 3) {
                const float* bl = s_b + layer * kHid;
#pragma unroll
                for (int c = 32 * half; c < 32 * half + 32; c += 16) {
                    float v[16];
                    tmem_ld16(my_lane + c, v);
                    float a[16];
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const float z = v[i] + bl[c + i];
                        a[i] = silu_f(z);
                        if (TRAIN && live) cache.z[layer][(size_t)row * kHid + c + i] = z;
                    }
                    st_row8(A, t, c, kHid, a);
                    st_row8(A, t, c + 8, kHid, a + 8);
                    if (TRAIN && live) {
                        // the BF16 activation the next layer consumes
                        *reinterpret_cast<uint4*>(cache.a[layer] + (size_t)row * kHid + c) =
                            *reinterpret_cast<const uint4*>(A + kmaj_off(t, c, kHid));
                        *reinterpret_cast<uint4*>(cache.a[layer] + (size_t)row * kHid + c + 8) =
                            *reinterpret_cast<const uint4*>(A + kmaj_off(t, c + 8, kHid));
                    }
                }
                async_smem_fence();
                tc_before();
                __syncthreads();
                tc_after();
            } else if (half == 0) {
                float v[16];
                tmem_ld16(my_lane, v);
                if (live) {
                    *reinterpret_cast<float2*>(out + 2 * (size_t)row) =
                        make_float2(v[0] + s_b[3 * kHid], v[1] + s_b[3 * kHid + 1]);
                }
                // the next tile's first MMA overwrites these columns
                tc_before();
            }
        }
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicAdd(err, 1ull);
        // let any MMA still in flight land before the tensor memory is freed
        bar_wait(&bar, 0);
        bar_wait(&bar, 1);
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

// ---- backward: `tiles` consecutive 128-row tiles per CTA ----
// Smem: W3t | W2t | Td (128x64) | TdT (128x128) | TaT (64x128)
constexpr int kTdTBytes = kRows * kRows * 2;
constexpr int kTaTBytes = kHid * kRows * 2;
constexpr int kBwdSmem = 2 * kW2Bytes + kABytes + kTdTBytes + kTaTBytes;

__global__ void __launch_bounds__(kRows) k_mlp_backward(const __nv_bfloat16* __restrict__ X, const float* __restrict__ Y,
                                                        int n, int tiles, float inv_batch, MlpNet net, MlpCache cache,
                                                        const float* __restrict__ out, float* __restrict__ grad,
                                                        unsigned long long* __restrict__ err) {
    extern __shared__ __align__(128) char smem[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ unsigned s_tmem;
    __shared__ float s_g4[kOutPad * kHid];  // dW4 (2 x 64 used)
    __shared__ float s_gb[3 * kHid + 2];    // db1, db2, db3, db4
    char* W3t = smem;
    char* W2t = W3t + kW2Bytes;
    char* Td = W2t + kW2Bytes;
    char* TdT = Td + kABytes;
    char* TaT = TdT + kTdTBytes;
    const int t = threadIdx.x, warp = t >> 5;
    copy_smem(W3t, (const char*)net.w3t, kW2Bytes);
    copy_smem(W2t, (const char*)net.w2t, kW2Bytes);
    zero_smem(TdT, kTdTBytes);  // rows 64..127 (the M padding) stay zero
    for (int i = t; i < kOutPad * kHid; i += kRows) s_g4[i] = 0.f;
    for (int i = t; i < 3 * kHid + 2; i += kRows) s_gb[i] = 0.f;
    if (t == 0) bar_init(&bar);
    if (warp == 0) tmem_alloc(&s_tmem, 256);
    async_smem_fence();
    tc_before();
    __syncthreads();
    tc_after();
    const unsigned tmem = s_tmem;
    const unsigned my_lane = tmem + ((unsigned)(32 * warp) << 16);
    // columns: [0,64) dA scratch, [64,128) dW3, [128,192) dW2, [192,208) dW1
    unsigned phase = 0;
    bool ok = true;
    for (int tile = 0; tile < tiles && ok; tile++) {
        const int row = (blockIdx.x * tiles + tile) * kRows + t;
        const bool live = row < n;
        // output layer (2 wide) on the CUDA cores
        float d4[2] = {0.f, 0.f};
        if (live) {
            d4[0] = 2.f * (out[2 * (size_t)row] - Y[2 * (size_t)row]) * inv_batch;
            d4[1] = 2.f * (out[2 * (size_t)row + 1] - Y[2 * (size_t)row + 1]) * inv_batch;
        }
        warp_add(&s_gb[3 * kHid], d4[0]);
        warp_add(&s_gb[3 * kHid + 1], d4[1]);
        float d[kHid];
#pragma unroll
        for (int i = 0; i < kHid; i++) {
            const float a3 = live ? __bfloat162float(cache.a[2][(size_t)row * kHid + i]) : 0.f;
            warp_add(&s_g4[i], d4[0] * a3);
            warp_add(&s_g4[kHid + i], d4[1] * a3);
            const float da3 = d4[0] * __ldg(net.w4f + i) + d4[1] * __ldg(net.w4f + kHid + i);
            d[i] = live ? da3 * dsilu_f(cache.z[2][(size_t)row * kHid + i]) : 0.f;
        }
        // layers 3, 2, 1: dA = D W (tensor cores), dW += D^T A (tensor cores)
        for (int layer = 2; layer >= 0 && ok; layer--) {
#pragma unroll
            for (int i = 0; i < kHid; i++) warp_add(&s_gb[layer * kHid + i], d[i]);
#pragma unroll
            for (int c = 0; c < kHid; c += 8) st_row8(Td, t, c, kHid, d + c);
#pragma unroll
            for (int i = 0; i < kHid; i++) st_one(TdT, i, t, kRows, d[i]);
            const int in_w = layer == 0 ? kIn : kHid;
            if (layer > 0) {
                for (int i = 0; i < kHid; i++) {
                    const float a = live ? __bfloat162float(cache.a[layer - 1][(size_t)row * kHid + i]) : 0.f;
                    st_one(TaT, i, t, kRows, a);
                }
            } else {
                for (int i = 0; i < kIn; i++) {
                    const float a = live ? __bfloat162float(X[(size_t)row * kIn + i]) : 0.f;
                    st_one(TaT, i, t, kRows, a);
                }
            }
            async_smem_fence();
            tc_before();
            __syncthreads();
            tc_after();
            if (t == 0) {
                const unsigned col = layer == 2 ? 64u : (layer == 1 ? 128u : 192u);
                mma_tile(tmem + col, TdT, TaT, kRows, in_w, tile > 0);
                if (layer > 0) mma_tile(tmem, Td, layer == 2 ? W3t : W2t, kHid, kHid, false);
                umma_commit(&bar);
            }
            ok = __syncthreads_and(bar_wait(&bar, phase)) != 0;
            phase ^= 1u;
            tc_after();
            if (!ok) break;
            if (layer > 0) {
#pragma unroll
                for (int c = 0; c < kHid; c += 16) {
                    float v[16];
                    tmem_ld16(my_lane + c, v);
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        d[c + i] = live ? v[i] * dsilu_f(cache.z[layer - 1][(size_t)row * kHid + c + i]) : 0.f;
                }
            }
            tc_before();
            __syncthreads();  // smem tiles are rewritten next
            tc_after();
        }
    }
    if (ok) {
        // weight gradients out of tensor memory: rows j < 64 live in lanes 0..63
        if (warp < 2) {
            const int j = t;
            for (int c = 0; c < kHid; c += 16) {
                float v[16];
                tmem_ld16(my_lane + 64 + c, v);
                for (int i = 0; i < 16; i++) atomicAdd(grad + kOffW3 + j * kHid + c + i, v[i]);
                tmem_ld16(my_lane + 128 + c, v);
                for (int i = 0; i < 16; i++) atomicAdd(grad + kOffW2 + j * kHid + c + i, v[i]);
            }
            float v[16];
            tmem_ld16(my_lane + 192, v);
            for (int i = 0; i < kIn; i++) atomicAdd(grad + kOffW1 + j * kIn + i, v[i]);
        }
        __syncthreads();
        for (int i = t; i < 2 * kHid; i += kRows) atomicAdd(grad + kOffW4 + i, s_g4[i]);
        for (int i = t; i < kHid; i += kRows) {
            atomicAdd(grad + kOffB1 + i, s_gb[i]);
            atomicAdd(grad + kOffB2 + i, s_gb[kHid + i]);
            atomicAdd(grad + kOffB3 + i, s_gb[2 * kHid + i]);
        }
        if (t < 2) atomicAdd(grad + kOffB4 + t, s_gb[3 * kHid + t]);
    } else {
        if (t == 0) atomicAdd(err, 1ull);
        bar_wait(&bar, 0);
        bar_wait(&bar, 1);
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// ---- Adam on the FP32 master parameters, then the BF16 operand packing ----
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Pack the FP32 parameters (W_k row-major out x in) into the BF16 K-major
// operand tiles: W1 (64x16), W2, W3 (64x64), W4 (16x64, rows 2.. zero), the
// transposes W2t, W3t for the backward pass, and W4 as FP32.
__global__ void k_mlp_pack(const float* __restrict__ p, MlpNet net) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    auto put = [](__nv_bfloat16* tile, int r, int k, int K, float v) {
        *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(tile) + kmaj_off(r, k, K)) = __float2bfloat16_rn(v);
    };
    if (i < kHid * kIn) {
        const int r = i / kIn, k = i % kIn;
        put(net.w1, r, k, kIn, p[kOffW1 + i]);
    }
    if (i < kHid * kHid) {
        const int r = i / kHid, k = i % kHid;
        put(net.w2, r, k, kHid, p[kOffW2 + i]);
        put(net.w3, r, k, kHid, p[kOffW3 + i]);
        put(net.w2t, k, r, kHid, p[kOffW2 + i]);
        put(net.w3t, k, r, kHid, p[kOffW3 + i]);
    }
    if (i < kOutPad * kHid) {
        const int r = i / kHid, k = i % kHid;
        put(net.w4, r, k, kHid, r < 2 ? p[kOffW4 + i] : 0.f);
        if (r < 2) net.w4f[i] = __bfloat162float(__float2bfloat16_rn(p[kOffW4 + i]));
    }
}

// sum over rows of ||out - Y||^2 (FP64 accumulation)
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ Y, int n, double* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const double a = (double)out[2 * (size_t)i] - Y[2 * (size_t)i];
        const double b = (double)out[2 * (size_t)i + 1] - Y[2 * (size_t)i + 1];
        v = a * a + b * b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(acc, v);
}

inline int nb(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

int mlp_forward_smem() { return kFwdSmem; }
int mlp_backward_smem() { return kBwdSmem; }

cudaError_t mlp_prepare_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem);
    return e;
}

void launch_mlp_pack(cudaStream_t s, const float* params, const MlpNet& net) {
    k_mlp_pack<<<nb(kHid * kHid, 256), 256, 0, s>>>(params, net);
}

void launch_mlp_forward(cudaStream_t s, const __nv_bfloat16* X, int n, const MlpNet& net, float* out,
                        const MlpCache* cache, unsigned long long* err) {
    if (n <= 0) return;
    // persistent: 5 CTAs per SM (shared memory's limit; 64 tensor-memory columns each),
    // weights staged once each; co-resident CTAs overlap one another's MMA waits with
    // their epilogues (0.104 ms with 4 per SM, 0.099 with 5, 1.31M rows)
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    const int grid = std::min(nb(n, kRows), 5 * sms);
    if (cache)
        k_mlp_forward<true><<<grid, kFwdThreads, kFwdSmem, s>>>(X, n, net, out, *cache, err);
    else
        k_mlp_forward<false><<<grid, kFwdThreads, kFwdSmem, s>>>(X, n, net, out, MlpCache{}, err);
}

void launch_mlp_backward(cudaStream_t s, const __nv_bfloat16* X, const float* Y, int n, const MlpNet& net,
                         const MlpCache& cache, const float* out, float* grad, unsigned long long* err) {
    if (n <= 0) return;
    const int tiles_total = nb(n, kRows);
    const int tiles = tiles_total >= 8 * 148 ? 8 : 1;
    k_mlp_backward<<<nb(tiles_total, tiles), kRows, kBwdSmem, s>>>(X, Y, n, tiles, 1.f / (float)n, net, cache, out,
                                                                  grad, err);
}

void launch_mse(cudaStream_t s, const float* out, const float* Y, int n, double* acc) {
    if (n > 0) k_mse<<<nb(n, 256), 256, 0, s>>>(out, Y, n, acc);
}

void launch_adam(cudaStream_t s, float* p, const float* g, float* m, float* v, int n, float lr, int step) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<nb(n, 256), 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace xg
