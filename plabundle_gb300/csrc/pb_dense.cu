// pb_dense.cu -- dense Cholesky preconditioner and FP64 conjugate gradients for the reduced system.
//
// The reduced camera system of the online Schur path is small (6 x cameras + refined intrinsics)
// but badly conditioned: the focal-length / altitude mode of a nadir block gives a normalised
// condition number near 1e7, where block-Jacobi PCG needs thousands of iterations.  Here the
// Jacobi-scaled matrix Sn = D^-1/2 S D^-1/2 is factored densely (Sn + shift I = L L^T, blocked
// right-looking Cholesky on 64x64 tiles), L is inverted (X = L^-1), and M^-1 = D^-1/2 X^T X D^-1/2
// preconditions conjugate gradients whose matrix-vector products use the FP64 reduced matrix.
// On the mixed path the factor and inverse are FP32 with a small shift that keeps the FP32
// factorisation positive definite; the FP64 CG recovers the FP64 solution (it plays the role of
// iterative refinement).  On the FP64 path the factor is FP64 and CG converges in one or two
// iterations.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

namespace {
constexpr int TS = 64;        // tile size
constexpr int TP = TS + 1;    // padded shared-memory row

__device__ __forceinline__ int tri_row(int idx) {
    // i such that i (i + 1) / 2 <= idx < (i + 1) (i + 2) / 2
    int i = static_cast<int>((sqrtf(8.0f * static_cast<float>(idx) + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= idx) ++i;
    while (i * (i + 1) / 2 > idx) --i;
    return i;
}
}  // namespace

// d_i = 1 / sqrt(S_ii) of the FP64 reduced matrix (pose diagonal blocks, intrinsic block).
__global__ void k_dense_scale(PcgSystem<double> sys, double* __restrict__ dscale, int* __restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n6 = 6 * sys.ncb, n = n6 + sys.nb;
    if (i >= n) return;
    double d;
    if (i < n6) {
        const int b = i / 6, a = i - b * 6;
        d = sys.vals[static_cast<size_t>(sys.diag_pos[b]) * 36 + a * 7];
    } else {
        const int c = i - n6;
        d = sys.Cm[c * sys.nb + c];
    }
    if (!(d > 0.0) || !isfinite(d)) {
        atomicOr(status, 1);
        d = 1.0;
    }
    dscale[i] = 1.0 / sqrt(d);
}

// Scatter of the scaled reduced matrix into a dense row-major np x np array (both triangles).
template <typename T>
__global__ void k_dense_fill(PcgSystem<double> sys, const double* __restrict__ dscale, T* __restrict__ A, int np) {
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int n6 = 6 * sys.ncb, nb = sys.nb;
    const long long nblk = static_cast<long long>(sys.row_ptr[sys.ncb]) * 36;
    const long long nbor = static_cast<long long>(n6) * nb;
    if (idx < nblk) {
        const int e = static_cast<int>(idx / 36), r = static_cast<int>(idx - static_cast<long long>(e) * 36);
        int lo = 0, hi = sys.ncb;  // block row of CSR entry e
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sys.row_ptr[mid] <= e) lo = mid;
            else hi = mid;
        }
        const int row = 6 * lo + r / 6, col = 6 * sys.col_idx[e] + r % 6;
        A[static_cast<size_t>(row) * np + col] = static_cast<T>(sys.vals[idx] * dscale[row] * dscale[col]);
    } else if (idx < nblk + nbor) {
        const long long k = idx - nblk;
        const int row = static_cast<int>(k / nb), c = static_cast<int>(k - static_cast<long long>(row) * nb);
        const T v = static_cast<T>(sys.border[k] * dscale[row] * dscale[n6 + c]);
        A[static_cast<size_t>(row) * np + n6 + c] = v;
        A[static_cast<size_t>(n6 + c) * np + row] = v;
    } else if (idx < nblk + nbor + static_cast<long long>(nb) * nb) {
        const int k = static_cast<int>(idx - nblk - nbor), a = k / nb, b = k - a * nb;
        A[static_cast<size_t>(n6 + a) * np + n6 + b] = static_cast<T>(sys.Cm[k] * dscale[n6 + a] * dscale[n6 + b]);
    }
}

// Diagonal shift of the scaled matrix (1 + shift) and identity on the padding.
template <typename T>
__global__ void k_dense_diag(T* __restrict__ A, int n, int np, double shift) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    T* d = A + static_cast<size_t>(i) * np + i;
    *d = i < n ? static_cast<T>(static_cast<double>(*d) + shift) : T(1);
}

// Cholesky of the diagonal tile k (one CTA).  A non-positive pivot sets status bit 2 and is
// replaced by 1 so that the remaining steps stay finite; the caller retries with a larger shift.
template <typename T>
__global__ void __launch_bounds__(256) k_potrf_diag(T* __restrict__ A, int np, int k, int* __restrict__ status) {
    __shared__ T s[TS * TP];
    T* tile = A + static_cast<size_t>(k) * TS * np + static_cast<size_t>(k) * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) s[(e / TS) * TP + e % TS] = tile[static_cast<size_t>(e / TS) * np + e % TS];
    __syncthreads();
    for (int j = 0; j < TS; ++j) {
        if (threadIdx.x == 0) {
            T d = s[j * TP + j];
            if (!(d > T(0)) || !isfinite(static_cast<double>(d))) {
                atomicOr(status, 2);
                d = T(1);
            }
            s[j * TP + j] = sqrt(d);
        }
        __syncthreads();
        const T inv = T(1) / s[j * TP + j];
        for (int i = j + 1 + threadIdx.x; i < TS; i += blockDim.x) s[i * TP + j] *= inv;
        __syncthreads();
        const int m = TS - 1 - j;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = j + 1 + e / m, l = j + 1 + e % m;
            if (l <= i) s[i * TP + l] -= s[i * TP + j] * s[l * TP + j];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) {
        const int r = e / TS, c = e % TS;
        tile[static_cast<size_t>(r) * np + c] = c <= r ? s[r * TP + c] : T(0);
    }
}

// A_ik <- A_ik L_kk^-T for every tile below the diagonal tile k (one CTA of 64 threads per tile,
// one row per thread).
template <typename T>
__global__ void __launch_bounds__(64) k_trsm_col(T* __restrict__ A, int np, int k) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sL = reinterpret_cast<T*>(smem_raw);
    T* sX = sL + TS * TP;
    const int i = k + 1 + blockIdx.x;
    const T* L = A + static_cast<size_t>(k) * TS * np + static_cast<size_t>(k) * TS;
    T* X = A + static_cast<size_t>(i) * TS * np + static_cast<size_t>(k) * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) {
        sL[(e / TS) * TP + e % TS] = L[static_cast<size_t>(e / TS) * np + e % TS];
        sX[(e / TS) * TP + e % TS] = X[static_cast<size_t>(e / TS) * np + e % TS];
    }
    __syncthreads();
    const int r = threadIdx.x;
    for (int c = 0; c < TS; ++c) {
        T v = sX[r * TP + c];
        for (int m = 0; m < c; ++m) v -= sX[r * TP + m] * sL[c * TP + m];
        sX[r * TP + c] = v / sL[c * TP + c];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) X[static_cast<size_t>(e / TS) * np + e % TS] = sX[(e / TS) * TP + e % TS];
}

// C (64x64) += A (64x64) * B (64x64): sA holds A row-major [r][k], sB holds B k-major [k][c];
// 256 threads, thread (ty, tx) owns rows ty + 16 m and columns tx + 16 m'.
template <typename T>
__device__ __forceinline__ void tile_mma(const T* __restrict__ sA, const T* __restrict__ sB, T acc[4][4]) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll 8
    for (int kk = 0; kk < TS; ++kk) {
        T a[4], b[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            a[m] = sA[(ty + 16 * m) * TP + kk];
            b[m] = sB[kk * TP + tx + 16 * m];
        }
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][q] += a[m] * b[q];
    }
}

// Loads a global 64x64 tile (row stride np) into shared memory, row-major or transposed.
template <typename T, bool TRANSPOSE>
__device__ __forceinline__ void tile_load(const T* __restrict__ g, int np, T* __restrict__ s) {
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) {
        const int r = e / TS, c = e % TS;
        const T v = g[static_cast<size_t>(r) * np + c];
        if (TRANSPOSE) s[c * TP + r] = v;
        else s[r * TP + c] = v;
    }
}

// Trailing update of the right-looking Cholesky: A_ij -= A_ik A_jk^T for k < j <= i.
template <typename T>
__global__ void __launch_bounds__(256) k_syrk_update(T* __restrict__ A, int np, int k) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);
    T* sB = sA + TS * TP;
    const int t = tri_row(blockIdx.x);
    const int i = k + 1 + t, j = k + 1 + (blockIdx.x - t * (t + 1) / 2);
    tile_load<T, false>(A + static_cast<size_t>(i) * TS * np + static_cast<size_t>(k) * TS, np, sA);
    tile_load<T, true>(A + static_cast<size_t>(j) * TS * np + static_cast<size_t>(k) * TS, np, sB);
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
    tile_mma<T>(sA, sB, acc);
    T* C = A + static_cast<size_t>(i) * TS * np + static_cast<size_t>(j) * TS;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) C[static_cast<size_t>(ty + 16 * m) * np + tx + 16 * q] -= acc[m][q];
}

// Inverses of all diagonal tiles of L (lower triangular), one CTA of 64 threads per tile,
// thread c solves L x = e_c.
template <typename T>
__global__ void __launch_bounds__(64) k_tile_inverse(const T* __restrict__ A, int np, T* __restrict__ Dinv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sL = reinterpret_cast<T*>(smem_raw);
    T* sX = sL + TS * TP;
    const int k = blockIdx.x;
    tile_load<T, false>(A + static_cast<size_t>(k) * TS * np + static_cast<size_t>(k) * TS, np, sL);
    __syncthreads();
    const int c = threadIdx.x;
    for (int r = 0; r < TS; ++r) {
        T v = r == c ? T(1) : T(0);
        if (r >= c)
            for (int m = c; m < r; ++m) v -= sL[r * TP + m] * sX[m * TP + c];
        sX[r * TP + c] = r >= c ? v / sL[r * TP + r] : T(0);
    }
    __syncthreads();
    T* out = Dinv + static_cast<size_t>(k) * TS * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) out[e] = sX[(e / TS) * TP + e % TS];
}

// X <- identity (the right-hand side of L X = I).
template <typename T>
__global__ void k_identity(T* __restrict__ X, int np) {
    const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e < static_cast<long long>(np) * np) X[e] = (e / np == e % np) ? T(1) : T(0);
}

// Row step k of X = L^-1 (right-looking forward substitution with identity right-hand side):
// X_kc <- Dinv_k X_kc for every tile column c <= k.
template <typename T>
__global__ void __launch_bounds__(256) k_trtri_row(T* __restrict__ X, int np, const T* __restrict__ Dinv, int k) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);
    T* sB = sA + TS * TP;
    const int c = blockIdx.x;
    const T* D = Dinv + static_cast<size_t>(k) * TS * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) sA[(e / TS) * TP + e % TS] = D[e];
    T* Xt = X + static_cast<size_t>(k) * TS * np + static_cast<size_t>(c) * TS;
    tile_load<T, false>(Xt, np, sB);
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
    tile_mma<T>(sA, sB, acc);
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) Xt[static_cast<size_t>(ty + 16 * m) * np + tx + 16 * q] = acc[m][q];
}

// X_ic -= L_ik X_kc for i > k, c <= k.
template <typename T>
__global__ void __launch_bounds__(256) k_trtri_update(const T* __restrict__ A, T* __restrict__ X, int np, int k) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);
    T* sB = sA + TS * TP;
    const int ncol = k + 1;
    const int i = k + 1 + blockIdx.x / ncol, c = blockIdx.x % ncol;
    tile_load<T, false>(A + static_cast<size_t>(i) * TS * np + static_cast<size_t>(k) * TS, np, sA);
    tile_load<T, false>(X + static_cast<size_t>(k) * TS * np + static_cast<size_t>(c) * TS, np, sB);
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
    tile_mma<T>(sA, sB, acc);
    T* Ct = X + static_cast<size_t>(i) * TS * np + static_cast<size_t>(c) * TS;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) Ct[static_cast<size_t>(ty + 16 * m) * np + tx + 16 * q] -= acc[m][q];
}

// XT = X^T restricted to the lower triangle of X (tile transposes through shared memory).
template <typename T>
__global__ void __launch_bounds__(256) k_transpose_lower(const T* __restrict__ X, T* __restrict__ XT, int np) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s = reinterpret_cast<T*>(smem_raw);
    const int t = tri_row(blockIdx.x);
    const int i = t, j = blockIdx.x - t * (t + 1) / 2;  // tile (i, j), j <= i
    tile_load<T, true>(X + static_cast<size_t>(i) * TS * np + static_cast<size_t>(j) * TS, np, s);
    __syncthreads();
    T* out = XT + static_cast<size_t>(j) * TS * np + static_cast<size_t>(i) * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) out[static_cast<size_t>(e / TS) * np + e % TS] = s[(e / TS) * TP + e % TS];
}

// ---- conjugate gradients on the FP64 reduced matrix, dense preconditioner M^-1 = D X^T X D.
// One cooperative persistent kernel runs the whole solve: per iteration the block-CSR SpMV (a
// warp per pose block row or border row), x/r updates, the two triangular products of the
// preconditioner (a warp per row) and the direction update, separated by five grid barriers.
// Dot products go through per-block partials that every block sums in the same fixed order, so
// all blocks take the same convergence / breakdown decision and no result depends on timing.
namespace {
constexpr int kCgThreads = 256;
constexpr int kCgWarps = kCgThreads / 32;
constexpr int kCgPart = 4;  // partial slots per block
}  // namespace

namespace cgk = cooperative_groups;

// Block sum of v (all threads), written by thread 0 to *dst.
__device__ __forceinline__ void block_partial(double v, double* s_red, double* dst) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kCgWarps; ++w) t += s_red[w];
        *dst = t;
    }
    __syncthreads();
}

// Sum over blocks of partial slot `slot`, identical in every block (fixed order: lane-strided
// sums, then a fixed shuffle tree).
__device__ __forceinline__ double grid_total(const double* part, int slot, double* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        double v = 0.0;
        for (int k = lane; k < static_cast<int>(gridDim.x); k += 32) v += part[k * kCgPart + slot];
        v = warp_sum(v);
        if (lane == 0) s_red[kCgWarps] = v;
    }
    __syncthreads();
    const double t = s_red[kCgWarps];
    __syncthreads();
    return t;
}

// out_i = so_i * sum_j M_ij (si_j in_j), j <= i (LOWER) or j >= i; one warp per row, rows
// interleaved over all warps of the grid; optional partial of dot_with . out.
template <typename T, bool LOWER>
__device__ __forceinline__ double tri_rows(const T* __restrict__ M, int np, int n, const double* __restrict__ in,
                                           const double* __restrict__ si, double* __restrict__ out,
                                           const double* __restrict__ so, const double* __restrict__ dot_with) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kCgWarps + (threadIdx.x >> 5), nw = gridDim.x * kCgWarps;
    double contrib = 0.0;
    for (int i = gw; i < n; i += nw) {
        const T* row = M + static_cast<size_t>(i) * np;
        const int j0 = LOWER ? 0 : i, j1 = LOWER ? i + 1 : n;
        T acc = T(0);
        for (int j = j0 + lane; j < j1; j += 32) acc += row[j] * static_cast<T>(si ? si[j] * in[j] : in[j]);
        double v = warp_sum(static_cast<double>(acc));
        if (so) v *= so[i];
        if (lane == 0) {
            out[i] = v;
            if (dot_with) contrib += dot_with[i] * v;
        }
    }
    return contrib;
}

// q = S p over the pose block rows and the border rows; returns this thread's share of p.q.
__device__ __forceinline__ double spmv_rows(const PcgSystem<double>& sys, const double* __restrict__ p,
                                            double* __restrict__ q) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kCgWarps + (threadIdx.x >> 5), nw = gridDim.x * kCgWarps;
    const int nb = sys.nb, n6 = 6 * sys.ncb;
    double pq = 0.0;
    for (int r = gw; r < sys.ncb + nb; r += nw) {
        if (r < sys.ncb) {
            double acc[6] = {0, 0, 0, 0, 0, 0};
            for (int e = sys.row_ptr[r] + lane; e < sys.row_ptr[r + 1]; e += 32) {
                const int j = sys.col_idx[e];
                const double* A = sys.vals + static_cast<size_t>(e) * 36;
                double pj[6];
#pragma unroll
                for (int c = 0; c < 6; ++c) pj[c] = p[6 * j + c];
#pragma unroll
                for (int a = 0; a < 6; ++a)
#pragma unroll
                    for (int c = 0; c < 6; ++c) acc[a] = fma(A[a * 6 + c], pj[c], acc[a]);
            }
            const double* Bi = sys.border + static_cast<size_t>(r) * 6 * nb;
            for (int c = lane; c < nb; c += 32)
#pragma unroll
                for (int a = 0; a < 6; ++a) acc[a] = fma(Bi[a * nb + c], p[n6 + c], acc[a]);
#pragma unroll
            for (int a = 0; a < 6; ++a) acc[a] = warp_sum(acc[a]);
            if (lane < 6) {
                double v = acc[0];
#pragma unroll
                for (int a = 1; a < 6; ++a)
                    if (lane == a) v = acc[a];
                q[6 * r + lane] = v;
                pq += p[6 * r + lane] * v;
            }
        } else {
            const int c = r - sys.ncb;
            double v = 0.0;
            for (int k = lane; k < n6; k += 32) v = fma(sys.border[static_cast<size_t>(k) * nb + c], p[k], v);
            for (int d = lane; d < nb; d += 32) v = fma(sys.Cm[c * nb + d], p[n6 + d], v);
            v = warp_sum(v);
            if (lane == 0) {
                q[n6 + c] = v;
                pq += p[n6 + c] * v;
            }
        }
    }
    return pq;
}

// out: [0] iterations, [1] relative residual, [2] converged, [3] status (1: breakdown)
template <typename T>
__global__ void __launch_bounds__(kCgThreads) k_dense_cg(PcgSystem<double> sys, const T* __restrict__ X,
                                                         const T* __restrict__ XT, int np,
                                                         const double* __restrict__ dscale,
                                                         const double* __restrict__ b, double* __restrict__ x,
                                                         double* __restrict__ r, double* __restrict__ z,
                                                         double* __restrict__ p, double* __restrict__ q,
                                                         double* __restrict__ w, double* __restrict__ part,
                                                         double* __restrict__ out, double rel_tol, double abs_tol,
                                                         int max_it) {
    cgk::grid_group grid = cgk::this_grid();
    __shared__ double s_red[kCgWarps + 1];
    const int n = 6 * sys.ncb + sys.nb;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    double* mypart = part + static_cast<size_t>(blockIdx.x) * kCgPart;
    // r = b, x = 0; w = X D r
    double bb = 0.0;
    for (int i = gt; i < n; i += nt) {
        x[i] = 0.0;
        r[i] = b[i];
        bb += b[i] * b[i];
    }
    block_partial(bb, s_red, mypart + 0);
    grid.sync();
    tri_rows<T, true>(X, np, n, b, dscale, w, nullptr, nullptr);
    grid.sync();
    block_partial(tri_rows<T, false>(XT, np, n, w, nullptr, z, dscale, b), s_red, mypart + 1);
    grid.sync();
    const double bnorm = sqrt(grid_total(part, 0, s_red));
    double rz = grid_total(part, 1, s_red);
    const double tol = fmax(rel_tol * bnorm, abs_tol);
    for (int i = gt; i < n; i += nt) p[i] = z[i];
    double rn = bnorm;
    int it = 0, status = 0;
    bool converged = rn <= tol;
    grid.sync();
    while (!converged && it < max_it) {
        block_partial(spmv_rows(sys, p, q), s_red, mypart + 2);
        grid.sync();
        const double pq = grid_total(part, 2, s_red);
        if (!(pq > 0.0) || !isfinite(pq) || !isfinite(rz)) {
            status = 1;
            break;
        }
        const double alpha = rz / pq;
        double rr = 0.0;
        for (int i = gt; i < n; i += nt) {
            x[i] = fma(alpha, p[i], x[i]);
            const double rv = fma(-alpha, q[i], r[i]);
            r[i] = rv;
            rr += rv * rv;
        }
        block_partial(rr, s_red, mypart + 0);
        grid.sync();
        ++it;
        rn = sqrt(grid_total(part, 0, s_red));
        if (!isfinite(rn)) {
            status = 1;
            break;
        }
        if (rn <= tol) {
            converged = true;
            break;
        }
        tri_rows<T, true>(X, np, n, r, dscale, w, nullptr, nullptr);
        grid.sync();
        block_partial(tri_rows<T, false>(XT, np, n, w, nullptr, z, dscale, r), s_red, mypart + 1);
        grid.sync();
        const double rz_new = grid_total(part, 1, s_red);
        const double beta = rz_new / rz;
        rz = rz_new;
        for (int i = gt; i < n; i += nt) p[i] = fma(beta, p[i], z[i]);
        grid.sync();
    }
    if (gt == 0) {
        out[0] = it;
        out[1] = bnorm > 0.0 ? rn / bnorm : 0.0;
        out[2] = converged ? 1.0 : 0.0;
        out[3] = status;
    }
}

// ---------------------------------------------------------------- host orchestration
template <typename T>
static void set_smem(const void* fn, size_t bytes) {
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

template <typename T>
size_t dense_bytes(int n) {
    const int np = ((n + TS - 1) / TS) * TS;
    return 2 * static_cast<size_t>(np) * np * sizeof(T) + static_cast<size_t>(np / TS) * TS * TS * sizeof(T);
}

template <typename T>
int dense_factor(const PcgSystem<double>& sys, DenseWork<T>& W, double shift, cudaStream_t st, int* launches) {
    const int n = W.n, np = W.np, nt = W.nt;
    const size_t two_tiles = 2 * static_cast<size_t>(TS) * TP * sizeof(T);
    static bool attrs = false;
    if (!attrs) {
        set_smem<T>(reinterpret_cast<const void*>(&k_trsm_col<T>), two_tiles);
        set_smem<T>(reinterpret_cast<const void*>(&k_syrk_update<T>), two_tiles);
        set_smem<T>(reinterpret_cast<const void*>(&k_tile_inverse<T>), two_tiles);
        set_smem<T>(reinterpret_cast<const void*>(&k_trtri_row<T>), two_tiles);
        set_smem<T>(reinterpret_cast<const void*>(&k_trtri_update<T>), two_tiles);
        set_smem<T>(reinterpret_cast<const void*>(&k_transpose_lower<T>), two_tiles / 2);
        attrs = true;
    }
    int L = 0;
    cudaMemsetAsync(W.status, 0, sizeof(int), st);
    cudaMemsetAsync(W.A, 0, static_cast<size_t>(np) * np * sizeof(T), st);
    k_dense_scale<<<(n + 255) / 256, 256, 0, st>>>(sys, W.dscale, W.status);
    const long long nfill = static_cast<long long>(sys.row_ptr ? W.nnzb : 0) * 36 + 6LL * sys.ncb * sys.nb +
                            static_cast<long long>(sys.nb) * sys.nb;
    if (nfill > 0) k_dense_fill<T><<<static_cast<unsigned>((nfill + 255) / 256), 256, 0, st>>>(sys, W.dscale, W.A, np);
    k_dense_diag<T><<<(np + 255) / 256, 256, 0, st>>>(W.A, n, np, shift);
    L += 3;
    for (int k = 0; k < nt; ++k) {
        k_potrf_diag<T><<<1, 256, 0, st>>>(W.A, np, k, W.status);
        ++L;
        const int m = nt - 1 - k;
        if (m > 0) {
            k_trsm_col<T><<<m, 64, two_tiles, st>>>(W.A, np, k);
            k_syrk_update<T><<<m * (m + 1) / 2, 256, two_tiles, st>>>(W.A, np, k);
            L += 2;
        }
    }
    k_tile_inverse<T><<<nt, 64, two_tiles, st>>>(W.A, np, W.Dinv);
    const long long nn = static_cast<long long>(np) * np;
    k_identity<T><<<static_cast<unsigned>((nn + 255) / 256), 256, 0, st>>>(W.X, np);
    L += 2;
    for (int k = 0; k < nt; ++k) {
        k_trtri_row<T><<<k + 1, 256, two_tiles, st>>>(W.X, np, W.Dinv, k);
        ++L;
        if (k + 1 < nt) {
            k_trtri_update<T><<<(nt - 1 - k) * (k + 1), 256, two_tiles, st>>>(W.A, W.X, np, k);
            ++L;
        }
    }
    k_transpose_lower<T><<<nt * (nt + 1) / 2, 256, two_tiles / 2, st>>>(W.X, W.A, np);
    ++L;
    if (launches) *launches += L;
    if (cudaGetLastError() != cudaSuccess) return -1;
    int status = 0;
    cudaMemcpyAsync(&status, W.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    return status;
}

template <typename T>
int dense_pcg(const PcgSystem<double>& sys, DenseWork<T>& W, const double* b, double rel_tol, double abs_tol,
              int max_it, int* iterations, double* relres, bool* converged, double* h_scal, cudaStream_t st,
              int* launches) {
    if (W.coop_grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_cg<T>, kCgThreads, 0);
        W.coop_grid = std::max(1, std::min(per_sm, 2) * sms);
    }
    const int grid = W.coop_grid;
    PcgSystem<double> s = sys;
    const T* X = W.X;
    const T* XT = W.A;
    int np = W.np;
    const double* dscale = W.dscale;
    double rt = rel_tol, at = abs_tol;
    int mi = max_it;
    void* args[] = {&s, &X, &XT, &np, &dscale, &b, &W.x, &W.r, &W.z, &W.p, &W.q, &W.w, &W.part, &W.scal, &rt, &at, &mi};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_dense_cg<T>), dim3(grid),
                                                      dim3(kCgThreads), args, 0, st);
    if (e != cudaSuccess) return -1;
    if (launches) *launches += 1;
    cudaMemcpyAsync(h_scal, W.scal, 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *iterations = static_cast<int>(h_scal[0]);
    *relres = h_scal[1];
    *converged = h_scal[2] != 0.0;
    return h_scal[3] != 0.0 ? 1 : 0;
}

template int dense_factor<float>(const PcgSystem<double>&, DenseWork<float>&, double, cudaStream_t, int*);
template int dense_factor<double>(const PcgSystem<double>&, DenseWork<double>&, double, cudaStream_t, int*);
template int dense_pcg<float>(const PcgSystem<double>&, DenseWork<float>&, const double*, double, double, int, int*,
                              double*, bool*, double*, cudaStream_t, int*);
template int dense_pcg<double>(const PcgSystem<double>&, DenseWork<double>&, const double*, double, double, int, int*,
                               double*, bool*, double*, cudaStream_t, int*);

}  // namespace pb
