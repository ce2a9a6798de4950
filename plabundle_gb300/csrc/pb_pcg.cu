// pb_pcg.cu -- block-Jacobi preconditioned conjugate gradients on the reduced camera system.
//
// The reduced matrix is an arrowhead: a block-sparse part over 6x6 pose blocks (CSR, both
// triangles) bordered by the dense columns of the shared intrinsics (B: 6*ncb x nb, C: nb x nb).
// One cooperative persistent kernel runs the whole solve: warp-per-block-row SpMV, the border
// products, the dot products and the vector updates, separated by three grid barriers per
// iteration.  Partial dot products are summed in a fixed order, so the solve is deterministic.
// The preconditioner blocks (6x6 poses, ni x ni per calibration group) are factored in FP64.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace cg = cooperative_groups;

namespace pb {

namespace {
constexpr int kPcgThreads = 256;
constexpr int kPcgWarps = kPcgThreads / 32;
constexpr int kPartStride = 2 + kMaxNB;  // per-block partials: [dot, dot2, border products]

// In-place FP64 Cholesky inverse of a small SPD matrix (n <= 9); false if not positive definite.
__device__ bool spd_inverse(double* A, int n, double* inv) {
    double L[kMaxNI * kMaxNI > 36 ? kMaxNI * kMaxNI : 36];
    for (int i = 0; i < n * n; ++i) L[i] = 0.0;
    for (int j = 0; j < n; ++j) {
        double d = A[j * n + j];
        for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
        if (!(d > 0.0) || !isfinite(d)) return false;
        d = sqrt(d);
        L[j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double v = A[i * n + j];
            for (int k = 0; k < j; ++k) v -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = v / d;
        }
    }
    // Li = L^-1 (lower), stored in A
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    for (int j = 0; j < n; ++j) {
        A[j * n + j] = 1.0 / L[j * n + j];
        for (int i = j + 1; i < n; ++i) {
            double v = 0.0;
            for (int k = j; k < i; ++k) v -= L[i * n + k] * A[k * n + j];
            A[i * n + j] = v / L[i * n + i];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double v = 0.0;
            for (int k = (i > j ? i : j); k < n; ++k) v += A[k * n + i] * A[k * n + j];
            inv[i * n + j] = v;
        }
    return true;
}
}  // namespace

template <typename T>
__global__ void k_precond(PcgSystem<T> sys, int* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < sys.ncb) {
        double A[36], inv[36];
        const T* blk = sys.vals + static_cast<size_t>(sys.diag_pos[t]) * 36;
        for (int i = 0; i < 36; ++i) A[i] = static_cast<double>(blk[i]);
        if (!spd_inverse(A, 6, inv)) {
            atomicOr(status, 2);
            for (int i = 0; i < 36; ++i) inv[i] = (i % 7 == 0) ? 1.0 : 0.0;
        }
        for (int i = 0; i < 36; ++i) sys.Dinv[static_cast<size_t>(t) * 36 + i] = static_cast<T>(inv[i]);
    } else if (t < sys.ncb + sys.ng) {
        const int g = t - sys.ncb, ni = sys.ni;
        double A[kMaxNI * kMaxNI], inv[kMaxNI * kMaxNI];
        for (int i = 0; i < ni; ++i)
            for (int j = 0; j < ni; ++j) A[i * ni + j] = static_cast<double>(sys.Cm[(g * ni + i) * sys.nb + g * ni + j]);
        if (!spd_inverse(A, ni, inv)) {
            atomicOr(status, 2);
            for (int i = 0; i < ni * ni; ++i) inv[i] = (i % (ni + 1) == 0) ? 1.0 : 0.0;
        }
        for (int i = 0; i < ni * ni; ++i) sys.Cinv[static_cast<size_t>(g) * ni * ni + i] = static_cast<T>(inv[i]);
    }
}

// Sum of per-block partial `slot` over the grid in a fixed order (every block obtains the same
// value).  A lane's loads are issued back to back (no dependent chain through L2), then summed in
// block order.
__device__ __forceinline__ double grid_total(const double* part, int slot, int nblocks) {
    constexpr int kPerLane = 16;  // up to 512 blocks
    const int lane = threadIdx.x & 31;
    double v = 0.0;
    if (nblocks <= 32 * kPerLane) {
        double t[kPerLane];
#pragma unroll
        for (int m = 0; m < kPerLane; ++m) {
            const int b = lane + 32 * m;
            t[m] = b < nblocks ? part[static_cast<size_t>(b) * kPartStride + slot] : 0.0;
        }
#pragma unroll
        for (int m = 0; m < kPerLane; ++m) v += t[m];
    } else {
        for (int b = lane; b < nblocks; b += 32) v += part[static_cast<size_t>(b) * kPartStride + slot];
    }
    return warp_sum(v);
}

template <typename T>
__device__ __forceinline__ void block_store(double* s_red, double v, int slot, double* part, int nslots_written) {
    (void)nslots_written;
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) s_red[(threadIdx.x >> 5) * kPartStride + slot] = v;
}

template <typename T>
__global__ void __launch_bounds__(kPcgThreads) k_pcg(PcgSystem<T> sys, const T* __restrict__ b, T* __restrict__ x,
                                                     T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
                                                     T* __restrict__ q, double* __restrict__ partA,
                                                     double* __restrict__ partB, PcgResult* __restrict__ res,
                                                     double abs_tol, double rel_tol, int max_iter) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double s_red[kPcgWarps * kPartStride];
    __shared__ double s_tot[kPartStride];
    __shared__ T s_pb[kMaxNB], s_qb[kMaxNB], s_rb[kMaxNB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // warp-major row order: consecutive block rows go to different blocks (SMs)
    const int gw = warp * gridDim.x + blockIdx.x, tw = gridDim.x * kPcgWarps;
    const int ncb = sys.ncb, nb = sys.nb, n6 = 6 * ncb, ng = sys.ng, ni = sys.ni;
    const int nblk = gridDim.x;

    auto block_reduce = [&](double* part, int nslots) {
        __syncthreads();
        for (int s = threadIdx.x; s < nslots; s += blockDim.x) {
            double v = 0.0;
            for (int w = 0; w < kPcgWarps; ++w) v += s_red[w * kPartStride + s];
            part[static_cast<size_t>(blockIdx.x) * kPartStride + s] = v;
        }
    };
    auto totals = [&](const double* part, int nslots) {
        // slots spread over the warps; results broadcast through shared memory
        __syncthreads();
        for (int s = warp; s < nslots; s += kPcgWarps) {
            const double v = grid_total(part, s, nblk);
            if (lane == 0) s_tot[s] = v;
        }
        __syncthreads();
    };
    for (int i = threadIdx.x; i < kPcgWarps * kPartStride; i += blockDim.x) s_red[i] = 0.0;
    __syncthreads();

    // ---- initialisation: x = 0, r = b, z = M^-1 r, p = z
    double a_rz = 0.0, a_rr = 0.0, a_bb = 0.0;
    for (int i = gw; i < ncb; i += tw) {
        const T bv = lane < 6 ? b[6 * i + lane] : T(0);
        T zv = T(0);
        const T* Di = sys.Dinv + static_cast<size_t>(i) * 36;
        for (int c = 0; c < 6; ++c) {
            const T rc = __shfl_sync(0xffffffffu, bv, c);
            if (lane < 6) zv += Di[lane * 6 + c] * rc;
        }
        if (lane < 6) {
            x[6 * i + lane] = T(0);
            r[6 * i + lane] = bv;
            z[6 * i + lane] = zv;
            p[6 * i + lane] = zv;
            a_rz += static_cast<double>(bv) * static_cast<double>(zv);
            a_rr += static_cast<double>(bv) * static_cast<double>(bv);
            a_bb += static_cast<double>(bv) * static_cast<double>(bv);
        }
    }
    if (blockIdx.x == 0 && nb > 0) {
        if (threadIdx.x < nb) s_rb[threadIdx.x] = b[n6 + threadIdx.x];
        __syncthreads();
        if (threadIdx.x < nb) {
            const int g = threadIdx.x / ni, a = threadIdx.x - g * ni;
            T zv = T(0);
            for (int c = 0; c < ni; ++c) zv += sys.Cinv[(g * ni + a) * ni + c] * s_rb[g * ni + c];
            const T bv = s_rb[threadIdx.x];
            x[n6 + threadIdx.x] = T(0);
            r[n6 + threadIdx.x] = bv;
            z[n6 + threadIdx.x] = zv;
            p[n6 + threadIdx.x] = zv;
            a_rz += static_cast<double>(bv) * static_cast<double>(zv);
            a_rr += static_cast<double>(bv) * static_cast<double>(bv);
            a_bb += static_cast<double>(bv) * static_cast<double>(bv);
        }
    }
    {
        const double v0 = warp_sum(a_rz), v1 = warp_sum(a_rr), v2 = warp_sum(a_bb);
        if (lane == 0) {
            s_red[warp * kPartStride + 0] = v0;
            s_red[warp * kPartStride + 1] = v1;
            s_red[warp * kPartStride + 2] = v2;
        }
    }
    block_reduce(partB, 3);
    grid.sync();
    totals(partB, 3);
    double rz = s_tot[0];
    const double bnorm = sqrt(s_tot[2]);
    double rnorm = sqrt(s_tot[1]);
    const double tol = fmax(rel_tol * bnorm, abs_tol);
    int it = 0, status = 0;
    bool converged = rnorm <= tol;
    (void)ng;

    while (!converged && it < max_iter) {
        // ---- q = A p  (pose rows), partial p.q and B^T p
        __syncthreads();
        for (int c = threadIdx.x; c < nb; c += blockDim.x) s_pb[c] = p[n6 + c];
        for (int i = threadIdx.x; i < kPcgWarps * kPartStride; i += blockDim.x) s_red[i] = 0.0;
        __syncthreads();
        double a_pq = 0.0;
        double a_bt[2] = {0.0, 0.0};  // border columns lane, lane + 32
        for (int i = gw; i < ncb; i += tw) {
            T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            for (int e = sys.row_ptr[i] + lane; e < sys.row_ptr[i + 1]; e += 32) {
                const int j = sys.col_idx[e];
                const T* A = sys.vals + static_cast<size_t>(e) * 36;
                T pj[6];
#pragma unroll
                for (int c = 0; c < 6; ++c) pj[c] = p[6 * j + c];
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                    T s = acc[a];
#pragma unroll
                    for (int c = 0; c < 6; ++c) s += A[a * 6 + c] * pj[c];
                    acc[a] = s;
                }
            }
            const T* Bi = sys.border + static_cast<size_t>(i) * 6 * nb;
            for (int c = lane; c < nb; c += 32) {
                const T pb = s_pb[c];
#pragma unroll
                for (int a = 0; a < 6; ++a) acc[a] += Bi[a * nb + c] * pb;
            }
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                T v = acc[a];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                acc[a] = v;
            }
            T pi[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) pi[a] = p[6 * i + a];
            if (lane < 6) {
                T qv = acc[0];
#pragma unroll
                for (int a = 1; a < 6; ++a)
                    if (lane == a) qv = acc[a];
                q[6 * i + lane] = qv;
                a_pq += static_cast<double>(pi[lane]) * static_cast<double>(qv);
            }
            for (int c = lane, k = 0; c < nb; c += 32, ++k) {
                T s = T(0);
#pragma unroll
                for (int a = 0; a < 6; ++a) s += Bi[a * nb + c] * pi[a];
                a_bt[k] += static_cast<double>(s);
            }
        }
        {
            const double v = warp_sum(a_pq);
            if (lane == 0) s_red[warp * kPartStride + 0] = v;
            for (int c = lane, k = 0; c < nb; c += 32, ++k) s_red[warp * kPartStride + 2 + c] = a_bt[k];
        }
        block_reduce(partA, 2 + nb);
        grid.sync();
        totals(partA, 2 + nb);
        // border rows: q_b = B^T p + C p_b (every block computes them)
        if (threadIdx.x < nb) {
            double v = s_tot[2 + threadIdx.x];
            for (int d = 0; d < nb; ++d)
                v += static_cast<double>(sys.Cm[threadIdx.x * nb + d]) * static_cast<double>(s_pb[d]);
            s_qb[threadIdx.x] = static_cast<T>(v);
        }
        __syncthreads();
        double pq = s_tot[0];
        for (int c = 0; c < nb; ++c) pq += static_cast<double>(s_pb[c]) * static_cast<double>(s_qb[c]);
        if (!(pq > 0.0) || !isfinite(pq)) {
            status = 1;
            break;
        }
        const double alpha = rz / pq;
        const T ta = static_cast<T>(alpha);
        // ---- x += alpha p, r -= alpha q, z = M^-1 r
        for (int i = threadIdx.x; i < kPcgWarps * kPartStride; i += blockDim.x) s_red[i] = 0.0;
        __syncthreads();
        double a_rz2 = 0.0, a_rr2 = 0.0;
        for (int i = gw; i < ncb; i += tw) {
            T rv = T(0);
            if (lane < 6) {
                const int k = 6 * i + lane;
                x[k] += ta * p[k];
                rv = r[k] - ta * q[k];
                r[k] = rv;
            }
            T zv = T(0);
            const T* Di = sys.Dinv + static_cast<size_t>(i) * 36;
            for (int c = 0; c < 6; ++c) {
                const T rc = __shfl_sync(0xffffffffu, rv, c);
                if (lane < 6) zv += Di[lane * 6 + c] * rc;
            }
            if (lane < 6) {
                z[6 * i + lane] = zv;
                a_rz2 += static_cast<double>(rv) * static_cast<double>(zv);
                a_rr2 += static_cast<double>(rv) * static_cast<double>(rv);
            }
        }
        if (blockIdx.x == 0 && nb > 0) {
            if (threadIdx.x < nb) {
                const int k = n6 + threadIdx.x;
                x[k] += ta * s_pb[threadIdx.x];
                s_rb[threadIdx.x] = r[k] - ta * s_qb[threadIdx.x];
                r[k] = s_rb[threadIdx.x];
            }
            __syncthreads();
            if (threadIdx.x < nb) {
                const int g = threadIdx.x / ni, a = threadIdx.x - g * ni;
                T zv = T(0);
                for (int c = 0; c < ni; ++c) zv += sys.Cinv[(g * ni + a) * ni + c] * s_rb[g * ni + c];
                z[n6 + threadIdx.x] = zv;
                a_rz2 += static_cast<double>(s_rb[threadIdx.x]) * static_cast<double>(zv);
                a_rr2 += static_cast<double>(s_rb[threadIdx.x]) * static_cast<double>(s_rb[threadIdx.x]);
            }
        }
        {
            const double v0 = warp_sum(a_rz2), v1 = warp_sum(a_rr2);
            if (lane == 0) {
                s_red[warp * kPartStride + 0] = v0;
                s_red[warp * kPartStride + 1] = v1;
            }
        }
        block_reduce(partB, 2);
        grid.sync();
        totals(partB, 2);
        const double rz_new = s_tot[0];
        rnorm = sqrt(s_tot[1]);
        ++it;
        if (!isfinite(rnorm)) {
            status = 1;
            break;
        }
        if (rnorm <= tol) {
            converged = true;
            break;
        }
        const T beta = static_cast<T>(rz_new / rz);
        rz = rz_new;
        for (int i = gw; i < ncb; i += tw)
            if (lane < 6) {
                const int k = 6 * i + lane;
                p[k] = z[k] + beta * p[k];
            }
        if (blockIdx.x == 0)
            for (int c = threadIdx.x; c < nb; c += blockDim.x) p[n6 + c] = z[n6 + c] + beta * p[n6 + c];
        grid.sync();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        res->iterations = it;
        res->converged = converged ? 1 : 0;
        res->status = status;
        res->rnorm = rnorm;
        res->bnorm = bnorm;
    }
}

template <typename T>
int pcg_precondition(const PcgSystem<T>& sys, int* d_status, cudaStream_t st) {
    const int n = sys.ncb + sys.ng;
    if (n == 0) return 0;
    k_precond<T><<<(n + 127) / 128, 128, 0, st>>>(sys, d_status);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

template <typename T>
int pcg_grid_size(int ncb) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg<T>, kPcgThreads, 0);
    const int want = std::max(1, (ncb + kPcgWarps - 1) / kPcgWarps);
    return std::max(1, std::min(want, sms * std::max(1, per_sm)));
}

template <typename T>
int pcg_solve(const PcgSystem<T>& sys, const T* b, T* x, T* work, double* partials, PcgResult* d_result,
              double abs_tol, double rel_tol, int max_iter, int grid, cudaStream_t st) {
    const int n = 6 * sys.ncb + sys.nb;
    T* r = work;
    T* z = work + n;
    T* p = work + 2 * n;
    T* q = work + 3 * n;
    double* partA = partials;
    double* partB = partials + static_cast<size_t>(grid) * kPartStride;
    PcgSystem<T> s = sys;
    void* args[] = {&s, &b, &x, &r, &z, &p, &q, &partA, &partB, &d_result, &abs_tol, &rel_tol, &max_iter};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_pcg<T>), dim3(grid),
                                                      dim3(kPcgThreads), args, 0, st);
    return e == cudaSuccess ? 0 : 1;
}

// ---- FP64 residual r = b - A x over the stored matrix (iterative refinement)
template <typename T>
__global__ void k_res_rows(PcgSystem<T> sys, const double* __restrict__ b, const double* __restrict__ x,
                           double* __restrict__ r, double* __restrict__ part) {
    __shared__ double s_bt[kPcgWarps][kMaxNB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * kPcgWarps + warp;
    const int nb = sys.nb, n6 = 6 * sys.ncb;
    for (int c = lane; c < kMaxNB; c += 32) s_bt[warp][c] = 0.0;
    if (i < sys.ncb) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int e = sys.row_ptr[i] + lane; e < sys.row_ptr[i + 1]; e += 32) {
            const int j = sys.col_idx[e];
            const T* A = sys.vals + static_cast<size_t>(e) * 36;
            for (int a = 0; a < 6; ++a)
                for (int c = 0; c < 6; ++c) acc[a] = fma(static_cast<double>(A[a * 6 + c]), x[6 * j + c], acc[a]);
        }
        const T* Bi = sys.border + static_cast<size_t>(i) * 6 * nb;
        for (int c = lane; c < nb; c += 32)
            for (int a = 0; a < 6; ++a) acc[a] = fma(static_cast<double>(Bi[a * nb + c]), x[n6 + c], acc[a]);
        for (int a = 0; a < 6; ++a) acc[a] = warp_sum(acc[a]);
        if (lane < 6) {
            double v = acc[0];
            for (int a = 1; a < 6; ++a)
                if (lane == a) v = acc[a];
            r[6 * i + lane] = b[6 * i + lane] - v;
        }
        for (int c = lane; c < nb; c += 32) {
            double s = 0.0;
            for (int a = 0; a < 6; ++a) s = fma(static_cast<double>(Bi[a * nb + c]), x[6 * i + a], s);
            s_bt[warp][c] = s;
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nb; c += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < kPcgWarps; ++w) s += s_bt[w][c];
        part[static_cast<size_t>(blockIdx.x) * kMaxNB + c] = s;
    }
}

template <typename T>
__global__ void k_res_border(PcgSystem<T> sys, const double* __restrict__ b, const double* __restrict__ x,
                             double* __restrict__ r, const double* __restrict__ part, int nblk, double* __restrict__ out) {
    __shared__ double s_rr[256], s_bb[256];
    const int nb = sys.nb, n6 = 6 * sys.ncb, n = n6 + nb;
    if (threadIdx.x < nb) {
        double v = 0.0;
        for (int k = 0; k < nblk; ++k) v += part[static_cast<size_t>(k) * kMaxNB + threadIdx.x];
        for (int d = 0; d < nb; ++d) v = fma(static_cast<double>(sys.Cm[threadIdx.x * nb + d]), x[n6 + d], v);
        r[n6 + threadIdx.x] = b[n6 + threadIdx.x] - v;
    }
    __syncthreads();
    double rr = 0.0, bb = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rr += r[i] * r[i];
        bb += b[i] * b[i];
    }
    s_rr[threadIdx.x] = rr;
    s_bb[threadIdx.x] = bb;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            s_rr[threadIdx.x] += s_rr[threadIdx.x + s];
            s_bb[threadIdx.x] += s_bb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sqrt(s_rr[0]);
        out[1] = sqrt(s_bb[0]);
    }
}

template <typename T>
void residual64(const PcgSystem<T>& sys, const double* b64, const double* x64, double* r64, double* out,
                cudaStream_t st) {
    const int nblk = std::max(1, (sys.ncb + kPcgWarps - 1) / kPcgWarps);
    double* part = out + 2;
    k_res_rows<T><<<nblk, kPcgThreads, 0, st>>>(sys, b64, x64, r64, part);
    k_res_border<T><<<1, 256, 0, st>>>(sys, b64, x64, r64, part, nblk, out);
}

__global__ void k_to_double_f(const float* in, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<double>(in[i]);
}
__global__ void k_to_double_d(const double* in, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}
__global__ void k_to_float(const double* in, float* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<float>(in[i]);
}
__global__ void k_axpy64(double* x, const float* d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += static_cast<double>(d[i]);
}

void to_double(const float* in, double* out, int n, cudaStream_t st) {
    if (n > 0) k_to_double_f<<<(n + 255) / 256, 256, 0, st>>>(in, out, n);
}
void to_double(const double* in, double* out, int n, cudaStream_t st) {
    if (n > 0) k_to_double_d<<<(n + 255) / 256, 256, 0, st>>>(in, out, n);
}
void to_float(const double* in, float* out, int n, cudaStream_t st) {
    if (n > 0) k_to_float<<<(n + 255) / 256, 256, 0, st>>>(in, out, n);
}
void axpy64(double* x, const float* d, int n, cudaStream_t st) {
    if (n > 0) k_axpy64<<<(n + 255) / 256, 256, 0, st>>>(x, d, n);
}

template int pcg_precondition<float>(const PcgSystem<float>&, int*, cudaStream_t);
template int pcg_precondition<double>(const PcgSystem<double>&, int*, cudaStream_t);
template int pcg_grid_size<float>(int);
template int pcg_grid_size<double>(int);
template int pcg_solve<float>(const PcgSystem<float>&, const float*, float*, float*, double*, PcgResult*, double,
                              double, int, int, cudaStream_t);
template int pcg_solve<double>(const PcgSystem<double>&, const double*, double*, double*, double*, PcgResult*, double,
                               double, int, int, cudaStream_t);
template void residual64<float>(const PcgSystem<float>&, const double*, const double*, double*, double*, cudaStream_t);
template void residual64<double>(const PcgSystem<double>&, const double*, const double*, double*, double*,
                                 cudaStream_t);

}  // namespace pb
