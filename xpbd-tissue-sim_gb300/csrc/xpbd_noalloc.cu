// xpbd_residual_noalloc: the constraint residual at the current state
// without allocating device or pinned host memory (declared in
// include/xpbd_gpu.h). xpbd_residual keeps its per-block partial sums in
// context buffers that it grows on demand (cudaMalloc / cudaMallocHost on the
// first call and when the row count grows); this entry point instead uses one
// fixed scratch array in the library's own device image.
//
// Scratch: kScratchDoubles doubles (128 KiB + 16 B) in a file-scope __device__
// array, one per device. Layout per call: [0, nb) the per-block partials of
// k_residual (nb = ceil(T / block)), [nb] a padding slot the reduction also
// reads, [nb + 1] the reduced sum of squares. The call clears [0, nb + 2)
// before the kernels run, so nothing has to start at zero.
//
// The scratch is shared by every context on a device: calls that overlap in
// time (two host threads, or two contexts whose streams run concurrently)
// race on it. Serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/xpbd_gpu.h"
#include "xpbd_ctx.cuh"
#include "xpbd_kernels.cuh"

using namespace xg;

namespace {

constexpr int kScratchBlocks = 16384;                  // partial sums: up to 16384 residual blocks
constexpr int kScratchDoubles = kScratchBlocks + 2;    // + padding slot + result
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_residual_scratch[kScratchDoubles];

// device address of g_residual_scratch, resolved once per device
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// cudaGetSymbolAddress with `dev` current (restoring the caller's device)
int scratch_for_device(xpbd_ctx* c, int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(c, XPBD_ERR_CAPACITY, "device ordinal %d >= %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        int cur = -1;
        XPBD_CU(c, cudaGetDevice(&cur));
        if (cur != dev) XPBD_CU(c, cudaSetDevice(dev));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_residual_scratch);
        if (cur != dev) cudaSetDevice(cur);
        if (e != cudaSuccess) return cuda_check(c, e, "cudaGetSymbolAddress(g_residual_scratch)");
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return XPBD_OK;
}

}  // namespace

extern "C" int xpbd_residual_noalloc(xpbd_ctx* c, double* abs_norm) {
    if (!c || !abs_norm) return XPBD_ERR_INVALID;
    const int nb = residual_blocks(c->T, c->block);
    if (nb > kScratchBlocks)
        return fail(c, XPBD_ERR_CAPACITY,
                    "xpbd_residual_noalloc: %d tets at block size %d need %d partial sums; the fixed scratch holds "
                    "%d (at most %lld tets at this block size)",
                    c->T, c->block, nb, kScratchBlocks, (long long)kScratchBlocks * c->block);
    int dev = -1;
    XPBD_CU(c, cudaStreamGetDevice(c->stream, &dev));
    double* scratch = nullptr;
    int st = scratch_for_device(c, dev, &scratch);
    if (st) return st;
    XPBD_CU(c, cudaMemsetAsync(scratch, 0, sizeof(double) * (size_t)(nb + 2), c->stream));
    {
        Scope s(c, K_RESIDUAL);
        launch_residual(c->L(), c->block, c->tets(), c->T, c->x.p,
                        c->prm.constraint_type == XPBD_CONSTRAINT_SEPARATE, c->perm.p, nullptr,
                        ResidualSink{scratch, 0, nb + 1, 0}, nullptr, (float)(c->prm.dt * c->prm.dt));
    }
    {
        Scope s(c, K_REDUCE);
        launch_reduce_rows(c->L(), scratch, 1, nb + 1, scratch + nb + 1);
    }
    XPBD_CU(c, cudaGetLastError());
    double v = 0.0;
    XPBD_CU(c, cudaMemcpyAsync(&v, scratch + nb + 1, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    *abs_norm = std::sqrt(v);
    return XPBD_OK;
}
