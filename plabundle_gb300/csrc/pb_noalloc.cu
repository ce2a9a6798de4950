// pb_noalloc.cu -- allocation-free robust objective of caller-owned device arrays.
//
// pb_gpu_objective_noalloc is the per-observation cost kernel of the LM line search
// (k_cost_batch / k_cost_final: FP64 projection, robust loss, per-block partial sums reduced in a
// fixed order) for callers that own their device buffers and may not allocate.  Its per-block
// partials live in one file-scope device array of fixed size instead of context memory, so a
// call launches two kernels, copies three numbers back and allocates nothing.
//
// Limits and rules (also stated in include/pb_gpu.h):
//   - at most PB_NOALLOC_MAX_OBS observations (one 256-thread block per 256 observations, one
//     partial per block); larger inputs are rejected before any launch;
//   - every element of the scratch array that the final kernel reads is written by the first
//     kernel of the same call, so nothing has to start at zero;
//   - the array is shared by all callers on a device: calls that overlap in time on one device
//     race; callers serialise them (one stream, or host-side ordering);
//   - the array's device address is resolved with cudaGetSymbolAddress on the first call on each
//     device (that call may load the module), so that first call should come before any stream
//     capture; the address is kept for the life of the process (not valid across a
//     cudaDeviceReset);
//   - an error already pending on the calling thread is left for its owner: the call returns
//     PB_ERR_CUDA without launching, and every status it reads afterwards is its own.
#include <cuda_runtime.h>

#include <mutex>

#include "pb_device.cuh"

namespace pb {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = static_cast<int>(PB_NOALLOC_MAX_OBS / kNoAllocThreads);
constexpr int kNoAllocMaxDevices = 64;

// [0, B): cost partials; [B, 2B): invalid projections; [2B, 3B): index errors; [3B, 3B + 3): totals
// (B = 16384 blocks: 384 KB per device)
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocMaxBlocks + 3];

namespace {

__global__ void __launch_bounds__(kNoAllocThreads)
    k_objective_part(const double* __restrict__ cameras, int n_cameras, const double* __restrict__ points,
                     int n_points, const int* __restrict__ obs_camera, const int* __restrict__ obs_point,
                     const double* __restrict__ obs_u, const double* __restrict__ obs_v,
                     const double* __restrict__ obs_w, long long n_obs, int loss, double scale,
                     double* __restrict__ scratch) {
    __shared__ double s_red[3][kNoAllocThreads / 32];
    const long long o = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    double cost = 0.0, bad = 0.0, oob = 0.0;
    if (o < n_obs) {
        const int cam = obs_camera[o], pt = obs_point[o];
        if (cam < 0 || cam >= n_cameras || pt < 0 || pt >= n_points) {
            oob = 1.0;  // the access is skipped; the host reports PB_ERR_BOUNDS
        } else {
            DCam c;
            load_cam(cameras + static_cast<size_t>(cam) * kCamStride, c);
            const double* X = points + static_cast<size_t>(pt) * 3;
            Proj p;
            double cst = 0.0, rw;
            bool good = project64(c, X[0], X[1], X[2], p);
            if (good) {
                const double r0 = p.px - obs_u[o], r1 = p.py - obs_v[o];
                good = robust_loss(obs_w[o] * (r0 * r0 + r1 * r1), loss, scale, cst, rw) && isfinite(cst);
            }
            if (good) cost = cst;
            else bad = 1.0;
        }
    }
    const double v[3] = {warp_sum(cost), warp_sum(bad), warp_sum(oob)};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) s_red[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) t += s_red[threadIdx.x][w];
        scratch[static_cast<size_t>(threadIdx.x) * kNoAllocMaxBlocks + blockIdx.x] = t;
    }
}

// Fixed-order sums of the block partials into scratch[3B .. 3B + 2].
__global__ void __launch_bounds__(kNoAllocThreads) k_objective_final(int nblocks, double* __restrict__ scratch) {
    __shared__ double s_red[3][kNoAllocThreads];
    for (int k = 0; k < 3; ++k) {
        double t = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) t += scratch[static_cast<size_t>(k) * kNoAllocMaxBlocks + b];
        s_red[k][threadIdx.x] = t;
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 3; ++k) s_red[k][threadIdx.x] += s_red[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) scratch[3 * static_cast<size_t>(kNoAllocMaxBlocks) + threadIdx.x] = s_red[threadIdx.x][0];
}

// Device address of the scratch array on the current device, resolved once per device.
double* noalloc_scratch() {
    static std::mutex mu;
    static double* addr[kNoAllocMaxDevices] = {nullptr};
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
        addr[dev] = static_cast<double*>(p);
    }
    return addr[dev];
}

}  // namespace

}  // namespace pb

extern "C" pb_status pb_gpu_objective_noalloc(const double* cameras, int32_t n_cameras, const double* points,
                                              int32_t n_points, const int32_t* obs_camera, const int32_t* obs_point,
                                              const double* obs_u, const double* obs_v, const double* obs_w,
                                              int64_t n_obs, int32_t robust_loss, double robust_loss_scale,
                                              void* stream, double* cost, int64_t* invalid_projections) {
    using namespace pb;
    if (!cost || n_obs < 0 || n_cameras < 0 || n_points < 0) return PB_ERR_INVALID_ARGUMENT;
    if (robust_loss < 0 || robust_loss > 2 || (robust_loss != 0 && !(robust_loss_scale > 0.0)))
        return PB_ERR_INVALID_ARGUMENT;
    if (n_obs > static_cast<int64_t>(PB_NOALLOC_MAX_OBS)) return PB_ERR_BOUNDS;
    if (n_obs > 0 && (!cameras || !points || !obs_camera || !obs_point || !obs_u || !obs_v || !obs_w))
        return PB_ERR_INVALID_ARGUMENT;
    if (n_obs == 0) {
        *cost = 0.0;
        if (invalid_projections) *invalid_projections = 0;
        return PB_OK;
    }
    // an error pending from earlier work on this thread is not this call's: leave it in place
    if (cudaPeekAtLastError() != cudaSuccess) return PB_ERR_CUDA;
    double* scratch = noalloc_scratch();
    if (!scratch) return PB_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblocks = static_cast<int>((n_obs + kNoAllocThreads - 1) / kNoAllocThreads);
    k_objective_part<<<nblocks, kNoAllocThreads, 0, st>>>(cameras, n_cameras, points, n_points, obs_camera, obs_point,
                                                          obs_u, obs_v, obs_w, static_cast<long long>(n_obs),
                                                          robust_loss, robust_loss_scale, scratch);
    if (cudaGetLastError() != cudaSuccess) return PB_ERR_CUDA;
    k_objective_final<<<1, kNoAllocThreads, 0, st>>>(nblocks, scratch);
    if (cudaGetLastError() != cudaSuccess) return PB_ERR_CUDA;
    double totals[3] = {0.0, 0.0, 0.0};
    if (cudaMemcpyAsync(totals, scratch + 3 * static_cast<size_t>(kNoAllocMaxBlocks), sizeof totals,
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PB_ERR_CUDA;
    if (totals[2] != 0.0) return PB_ERR_BOUNDS;
    *cost = totals[0];
    if (invalid_projections) *invalid_projections = static_cast<int64_t>(totals[1]);
    return PB_OK;
}
