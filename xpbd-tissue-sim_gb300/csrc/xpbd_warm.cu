// C ABI of the learned warm start (declared in include/xpbd_gpu.h): the
// per-tet network's parameters, forward / loss-gradient / Adam entry points on
// host buffers, online training on substeps the solver records, and the
// warm-start mode of xpbd_update. The reference has no learned component; the
// network's place in the substep is after XPBDMeshObject_::_movePositionsInertially
// (XPBDMeshObject.cpp:449-456) and before the solver iterations
// (XPBDSolver.hpp:71-96).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/xpbd_gpu.h"
#include "xpbd_ctx.cuh"
#include "xpbd_kernels.cuh"

using namespace xg;

static_assert(XPBD_MLP_PARAMS == kMlpParams, "parameter count of the header and the kernels");
static_assert(XPBD_MLP_INPUTS == kMlpIn, "feature row width of the header and the kernels");

namespace {

constexpr int kTileElems = 64 * 16 + 4 * 64 * 64 + 16 * 64;  // W1 | W2 | W3 | W4 | W2t | W3t

// round-to-nearest-even FP32 -> BF16 bits (NaN kept quiet)
uint16_t to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

float from_bf16(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int ensure_mlp(xpbd_ctx* c) {
    if (c->mlp_p.p) return XPBD_OK;
    XPBD_CU(c, mlp_prepare_kernels());
    XPBD_CU(c, c->mlp_p.alloc(kMlpParams));
    XPBD_CU(c, c->mlp_m.alloc(kMlpParams));
    XPBD_CU(c, c->mlp_v.alloc(kMlpParams));
    XPBD_CU(c, c->mlp_g.alloc(kMlpParams));
    XPBD_CU(c, c->mlp_w4f.alloc(2 * kMlpHid));
    XPBD_CU(c, c->mlp_tiles.alloc(kTileElems));
    XPBD_CU(c, cudaMemset(c->mlp_tiles.p, 0, sizeof(__nv_bfloat16) * kTileElems));
    c->graph_dirty = true;  // captured substeps hold no network yet
    return XPBD_OK;
}

// upload FP32 parameters, reset the Adam moments, pack the operand tiles
int set_params(xpbd_ctx* c, const float* p) {
    int st = ensure_mlp(c);
    if (st) return st;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    XPBD_CU(c, cudaMemcpy(c->mlp_p.p, p, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemset(c->mlp_m.p, 0, sizeof(float) * kMlpParams));
    XPBD_CU(c, cudaMemset(c->mlp_v.p, 0, sizeof(float) * kMlpParams));
    XPBD_CU(c, cudaMemset(c->mlp_g.p, 0, sizeof(float) * kMlpParams));
    c->adam_t = 0;
    launch_mlp_pack(c->stream, c->mlp_p.p, c->net());
    XPBD_CU(c, cudaGetLastError());
    c->mlp_ready = true;
    return XPBD_OK;
}

int ensure_step_buffers(xpbd_ctx* c) {
    if (!c->feat.p) {
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        XPBD_CU(c, c->feat.alloc((size_t)kMlpIn * c->T));
        XPBD_CU(c, c->pred.alloc(2 * (size_t)c->T));
        XPBD_CU(c, c->target.alloc(2 * (size_t)c->T));
        XPBD_CU(c, c->x_pred.alloc(c->V));
        c->graph_dirty = true;
    }
    return XPBD_OK;
}

int ensure_cache(xpbd_ctx* c, int rows) {
    if (c->cache_rows >= rows) return XPBD_OK;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    c->cache_z.release();
    c->cache_a.release();
    c->cache_out.release();
    XPBD_CU(c, c->cache_z.alloc(3 * (size_t)kMlpHid * rows));
    XPBD_CU(c, c->cache_a.alloc(3 * (size_t)kMlpHid * rows));
    XPBD_CU(c, c->cache_out.alloc(2 * (size_t)rows));
    c->cache_rows = rows;
    return XPBD_OK;
}

MlpCache cache_of(xpbd_ctx* c) {
    const size_t r = (size_t)c->cache_rows * kMlpHid;
    return MlpCache{{c->cache_z.p, c->cache_z.p + r, c->cache_z.p + 2 * r},
                    {c->cache_a.p, c->cache_a.p + r, c->cache_a.p + 2 * r}};
}

// one forward (training) + loss + backward on device rows [X, Y) of n rows;
// the gradient of the mean loss replaces mlp_g, the summed squared error is
// added to c->mse
void enqueue_loss_grad(xpbd_ctx* c, const __nv_bfloat16* X, const float* Y, int n) {
    const MlpCache cache = cache_of(c);
    const MlpNet net = c->net();
    unsigned long long* err = &c->flags.p->timeouts;
    launch_mlp_forward(c->stream, X, n, net, c->cache_out.p, &cache, err);
    launch_mse(c->stream, c->cache_out.p, Y, n, c->mse.p);
    cudaMemsetAsync(c->mlp_g.p, 0, sizeof(float) * kMlpParams, c->stream);
    launch_mlp_backward(c->stream, X, Y, n, net, cache, c->cache_out.p, c->mlp_g.p, err);
    c->launches += 3;
}

void enqueue_adam(xpbd_ctx* c, float lr) {
    c->adam_t++;
    launch_adam(c->stream, c->mlp_p.p, c->mlp_g.p, c->mlp_m.p, c->mlp_v.p, kMlpParams, lr, c->adam_t);
    launch_mlp_pack(c->stream, c->mlp_p.p, c->net());
    c->launches += 2;
}

// host FP32 rows (n x 16) -> a fresh device BF16 buffer
int upload_features(xpbd_ctx* c, const float* X, int64_t n, DevBuf<__nv_bfloat16>& d) {
    std::vector<uint16_t> h((size_t)n * kMlpIn);
    for (size_t i = 0; i < h.size(); i++) h[i] = to_bf16(X[i]);
    XPBD_CU(c, d.alloc(h.size()));
    XPBD_CU(c, cudaMemcpy(d.p, h.data(), sizeof(uint16_t) * h.size(), cudaMemcpyHostToDevice));
    return XPBD_OK;
}

struct Tmp {
    DevBuf<__nv_bfloat16> X;
    DevBuf<float> Y, out;
    ~Tmp() {
        X.release();
        Y.release();
        out.release();
    }
};

int check_timeouts(xpbd_ctx* c) {
    Flags f{};
    XPBD_CU(c, cudaMemcpy(&f, c->flags.p, sizeof f, cudaMemcpyDeviceToHost));
    if (f.timeouts) return fail(c, XPBD_ERR_TIMEOUT, "%llu blocks gave up waiting on the tensor cores", f.timeouts);
    return XPBD_OK;
}

}  // namespace

extern "C" {

int xpbd_mlp_init(xpbd_ctx* c, uint64_t seed) {
    if (!c) return XPBD_ERR_INVALID;
    // He-normal weights (std sqrt(2 / fan_in), fan_in of W1 = 14 real inputs),
    // zero biases, W4 scaled by 0.1, W1's two padding columns zero.
    // Normals: splitmix64 uniforms through Box-Muller.
    uint64_t s = seed;
    auto next = [&s]() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() { return std::sqrt(-2.0 * std::log(next())) * std::cos(6.283185307179586 * next()); };
    std::vector<float> p(kMlpParams, 0.f);
    for (int r = 0; r < kMlpHid; r++)
        for (int k = 0; k < 14; k++) p[kOffW1 + r * kMlpIn + k] = (float)(normal() * std::sqrt(2.0 / 14));
    for (int i = 0; i < kMlpHid * kMlpHid; i++) p[kOffW2 + i] = (float)(normal() * std::sqrt(2.0 / kMlpHid));
    for (int i = 0; i < kMlpHid * kMlpHid; i++) p[kOffW3 + i] = (float)(normal() * std::sqrt(2.0 / kMlpHid));
    for (int i = 0; i < 2 * kMlpHid; i++) p[kOffW4 + i] = (float)(0.1 * normal() * std::sqrt(2.0 / kMlpHid));
    return set_params(c, p.data());
}

int xpbd_mlp_set_params(xpbd_ctx* c, const float* params, int64_t n) {
    if (!c || !params || n != kMlpParams) return XPBD_ERR_INVALID;
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(params[i])) return fail(c, XPBD_ERR_INVALID, "parameter %lld is not finite", (long long)i);
    return set_params(c, params);
}

int xpbd_mlp_get_params(xpbd_ctx* c, float* params, int64_t n) {
    if (!c || !params || n != kMlpParams) return XPBD_ERR_INVALID;
    if (!c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    XPBD_CU(c, cudaMemcpy(params, c->mlp_p.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    return XPBD_OK;
}

int xpbd_mlp_forward(xpbd_ctx* c, const float* X, int64_t n, float* out) {
    if (!c || !X || !out || n <= 0 || n > (1 << 28)) return XPBD_ERR_INVALID;
    if (!c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    Tmp t;
    int st = upload_features(c, X, n, t.X);
    if (st) return st;
    XPBD_CU(c, t.out.alloc(2 * (size_t)n));
    launch_mlp_forward(c->stream, t.X.p, (int)n, c->net(), t.out.p, nullptr, &c->flags.p->timeouts);
    c->launches++;
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    st = check_timeouts(c);
    if (st) return st;
    XPBD_CU(c, cudaMemcpy(out, t.out.p, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToHost));
    return XPBD_OK;
}

int xpbd_mlp_loss_grad(xpbd_ctx* c, const float* X, const float* Y, int64_t n, double* loss, float* grad) {
    if (!c || !X || !Y || n <= 0 || n > (1 << 24)) return XPBD_ERR_INVALID;
    if (!c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    int st = ensure_cache(c, (int)n);
    if (st) return st;
    Tmp t;
    st = upload_features(c, X, n, t.X);
    if (st) return st;
    XPBD_CU(c, t.Y.alloc(2 * (size_t)n));
    XPBD_CU(c, cudaMemcpy(t.Y.p, Y, sizeof(float) * 2 * (size_t)n, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemsetAsync(c->mse.p, 0, sizeof(double), c->stream));
    enqueue_loss_grad(c, t.X.p, t.Y.p, (int)n);
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    st = check_timeouts(c);
    if (st) return st;
    if (loss) {
        double v = 0;
        XPBD_CU(c, cudaMemcpy(&v, c->mse.p, sizeof v, cudaMemcpyDeviceToHost));
        *loss = v / (double)n;
    }
    if (grad) XPBD_CU(c, cudaMemcpy(grad, c->mlp_g.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    return XPBD_OK;
}

int xpbd_mlp_adam_step(xpbd_ctx* c, const float* grad, float lr) {
    if (!c || !(lr > 0.f) || !std::isfinite(lr)) return XPBD_ERR_INVALID;
    if (!c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    if (grad)
        XPBD_CU(c, cudaMemcpyAsync(c->mlp_g.p, grad, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c->stream));
    enqueue_adam(c, lr);
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}

int xpbd_mlp_record(xpbd_ctx* c, int32_t on) {
    if (!c || (on != 0 && on != 1)) return XPBD_ERR_INVALID;
    if (on) {
        int st = ensure_step_buffers(c);
        if (st) return st;
    }
    if ((on != 0) != c->record) c->graph_dirty = true;
    c->record = on != 0;
    c->recorded = false;
    return XPBD_OK;
}

int xpbd_mlp_get_samples(xpbd_ctx* c, float* X, float* Y) {
    if (!c || (!X && !Y)) return XPBD_ERR_INVALID;
    if (!c->recorded) return fail(c, XPBD_ERR_STATE, "no substep recorded");
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    const size_t T = (size_t)c->T;
    if (X) {
        std::vector<uint16_t> h(T * kMlpIn);
        XPBD_CU(c, cudaMemcpy(h.data(), c->feat.p, sizeof(uint16_t) * h.size(), cudaMemcpyDeviceToHost));
        for (size_t s = 0; s < T; s++) {
            const size_t t = (size_t)c->tet_of_slot[s];
            for (int k = 0; k < kMlpIn; k++) X[t * kMlpIn + k] = from_bf16(h[s * kMlpIn + k]);
        }
    }
    if (Y) {
        std::vector<float> h(2 * T);
        XPBD_CU(c, cudaMemcpy(h.data(), c->target.p, sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
        for (size_t s = 0; s < T; s++) {
            const size_t t = (size_t)c->tet_of_slot[s];
            Y[2 * t] = h[2 * s];
            Y[2 * t + 1] = h[2 * s + 1];
        }
    }
    return XPBD_OK;
}

int xpbd_mlp_train(xpbd_ctx* c, int32_t epochs, int32_t batch, float lr, double* loss) {
    if (!c || epochs <= 0 || batch < 128 || batch > (1 << 22) || !(lr > 0.f) || !std::isfinite(lr))
        return XPBD_ERR_INVALID;
    if (!c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    if (!c->recorded) return fail(c, XPBD_ERR_STATE, "no substep recorded");
    const int T = c->T;
    const int B = std::min(batch, T);
    int st = ensure_cache(c, B);
    if (st) return st;
    const int nchunks = (T + B - 1) / B;
    std::vector<int> order(nchunks);
    uint64_t rng = 0x2545f4914f6cdd1dull ^ (uint64_t)c->adam_t;
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < nchunks; i++) order[i] = i;
        for (int i = nchunks - 1; i > 0; i--) {  // Fisher-Yates on an xorshift stream
            rng ^= rng << 13;
            rng ^= rng >> 7;
            rng ^= rng << 17;
            std::swap(order[i], order[(int)(rng % (uint64_t)(i + 1))]);
        }
        XPBD_CU(c, cudaMemsetAsync(c->mse.p, 0, sizeof(double), c->stream));
        for (int i = 0; i < nchunks; i++) {
            const int s0 = order[i] * B;
            const int n = std::min(B, T - s0);
            enqueue_loss_grad(c, c->feat.p + (size_t)s0 * kMlpIn, c->target.p + 2 * (size_t)s0, n);
            enqueue_adam(c, lr);
        }
    }
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    st = check_timeouts(c);
    if (st) return st;
    if (loss) {
        double v = 0;
        XPBD_CU(c, cudaMemcpy(&v, c->mse.p, sizeof v, cudaMemcpyDeviceToHost));
        *loss = v / (double)T;
    }
    return XPBD_OK;
}

int xpbd_set_warm_start(xpbd_ctx* c, int32_t mode) {
    if (!c || mode < XPBD_WARM_NONE || mode > XPBD_WARM_MLP) return XPBD_ERR_INVALID;
    if (mode == XPBD_WARM_MLP && !c->mlp_ready) return fail(c, XPBD_ERR_STATE, "network not initialised");
    if (mode != XPBD_WARM_NONE) {
        int st = ensure_step_buffers(c);
        if (st) return st;
    }
    if (mode != c->warm_mode) c->graph_dirty = true;
    c->warm_mode = mode;
    return XPBD_OK;
}

int xpbd_warm_start_stats(xpbd_ctx* c, int64_t* kept, int64_t* rejected) {
    if (!c || !kept || !rejected) return XPBD_ERR_INVALID;
    unsigned long long h[2] = {0, 0};
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    XPBD_CU(c, cudaMemcpy(h, c->warm_stats.p, sizeof h, cudaMemcpyDeviceToHost));
    *kept = (int64_t)h[0];
    *rejected = (int64_t)h[1];
    return XPBD_OK;
}

}  // extern "C"
