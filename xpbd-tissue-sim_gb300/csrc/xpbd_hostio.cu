// Position transfers between the caller's host arrays and the device: the
// conversion kernels read and write the host array directly when the GPU
// addresses pageable host memory.
#include "xpbd_device.cuh"

namespace xg {

namespace {

// ---- host arrays the device addresses directly (coherent pageable memory
// on a Grace-Blackwell system): 3 values per vertex, converted here ----
// A block moves its 256 vertices' 3 x 256 values through shared memory, so the
// host side is read and written in whole 16-byte pieces covering full cache
// lines (when the block's run of the array is 16-byte aligned).
constexpr int kHostIoThreads = 256;

template <typename H>
__global__ void __launch_bounds__(kHostIoThreads) k_xyz_from_host(float4* __restrict__ x, const H* __restrict__ h,
                                                                  int V, bool keep_w) {
    __shared__ __align__(16) H buf[3 * kHostIoThreads];
    const int tid = threadIdx.x, v0 = blockIdx.x * kHostIoThreads;
    const int n = min(kHostIoThreads, V - v0), nv = 3 * n;
    const H* src = h + 3 * (size_t)v0;
    constexpr int kPer16 = 16 / (int)sizeof(H);
    if (((uintptr_t)src & 15) == 0) {
        for (int i = tid; i < nv / kPer16; i += kHostIoThreads)
            reinterpret_cast<uint4*>(buf)[i] = __ldcv(reinterpret_cast<const uint4*>(src) + i);
        for (int i = nv / kPer16 * kPer16 + tid; i < nv; i += kHostIoThreads) buf[i] = src[i];
    } else {
        for (int i = tid; i < nv; i += kHostIoThreads) buf[i] = src[i];
    }
    __syncthreads();
    if (tid < n) {
        const int i = v0 + tid;
        const float w = keep_w ? x[i].w : 0.f;  // inverse mass and fixed sign stay
        x[i] = make_float4((float)buf[3 * tid], (float)buf[3 * tid + 1], (float)buf[3 * tid + 2], w);
    }
}

template <typename H>
__global__ void __launch_bounds__(kHostIoThreads) k_xyz_to_host(H* __restrict__ h, const float4* __restrict__ x,
                                                                int V) {
    __shared__ __align__(16) H buf[3 * kHostIoThreads];
    const int tid = threadIdx.x, v0 = blockIdx.x * kHostIoThreads;
    const int n = min(kHostIoThreads, V - v0), nv = 3 * n;
    if (tid < n) {
        const float4 p = x[v0 + tid];
        buf[3 * tid] = (H)p.x;
        buf[3 * tid + 1] = (H)p.y;
        buf[3 * tid + 2] = (H)p.z;
    }
    __syncthreads();
    H* dst = h + 3 * (size_t)v0;
    constexpr int kPer16 = 16 / (int)sizeof(H);
    if (((uintptr_t)dst & 15) == 0) {
        for (int i = tid; i < nv / kPer16; i += kHostIoThreads)
            reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(buf)[i];
        for (int i = nv / kPer16 * kPer16 + tid; i < nv; i += kHostIoThreads) dst[i] = buf[i];
    } else {
        for (int i = tid; i < nv; i += kHostIoThreads) dst[i] = buf[i];
    }
}

}  // namespace

void launch_xyz_from_host(cudaStream_t s, float4* x, const double* h, int V, bool keep_w) {
    if (V > 0) k_xyz_from_host<double><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(x, h, V, keep_w);
}
void launch_xyz_from_host(cudaStream_t s, float4* x, const float* h, int V, bool keep_w) {
    if (V > 0) k_xyz_from_host<float><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(x, h, V, keep_w);
}
void launch_xyz_to_host(cudaStream_t s, double* h, const float4* x, int V) {
    if (V > 0) k_xyz_to_host<double><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(h, x, V);
}
void launch_xyz_to_host(cudaStream_t s, float* h, const float4* x, int V) {
    if (V > 0) k_xyz_to_host<float><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(h, x, V);
}

}  // namespace xg
