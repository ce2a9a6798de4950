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
// iterations.  The factorisation with its inverse and the whole CG solve are each one cooperative
// persistent kernel (grid barriers between phases, no host round trips).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

namespace cgk = cooperative_groups;

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

// Loads a global 64x64 tile (row stride np, 16-byte aligned rows) into shared memory, row-major
// or transposed, with 16-byte loads.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int n = 4;
    __device__ static __forceinline__ float get(const float4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }
    __device__ static __forceinline__ float dot(const float4& a, const float4& b) {
        return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    }
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int n = 2;
    __device__ static __forceinline__ double get(const double2& v, int i) { return i == 0 ? v.x : v.y; }
    __device__ static __forceinline__ double dot(const double2& a, const double2& b) { return a.x * b.x + a.y * b.y; }
};

template <typename T, bool TRANSPOSE>
__device__ __forceinline__ void tile_load(const T* __restrict__ g, int np, T* __restrict__ s) {
    using V = Vec16<T>;
    constexpr int per_row = TS / V::n;
    for (int e = threadIdx.x; e < TS * per_row; e += blockDim.x) {
        const int r = e / per_row, c0 = (e % per_row) * V::n;
        const typename V::type v = *reinterpret_cast<const typename V::type*>(g + static_cast<size_t>(r) * np + c0);
#pragma unroll
        for (int q = 0; q < V::n; ++q) {
            if (TRANSPOSE) s[(c0 + q) * TP + r] = V::get(v, q);
            else s[r * TP + c0 + q] = V::get(v, q);
        }
    }
}

// Lower-triangle elements of a 64x64 tile owned by this thread (up to 9 of 2080).
__device__ __forceinline__ int owned_elements(int* ii, int* ll) {
    int cnt = 0;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        const int e = threadIdx.x + 256 * s;
        if (e < TS * (TS + 1) / 2) {
            const int i = tri_row(e);
            ii[s] = i;
            ll[s] = e - i * (i + 1) / 2;
            ++cnt;
        } else {
            ii[s] = -1;
            ll[s] = -1;
        }
    }
    return cnt;
}

// Block 0 of step k: L_kk (written to A_kk, zeros above the diagonal) and D_k = L_kk^-1.
//
// The factorisation is the unscaled right-looking elimination (after step j, column j holds
// d_j * L_:j): every lower element (i, l) receives a_il = fma(-(a_ij a_lj), 1 / d_j, a_il) for
// j < l in increasing j (one rounding of the product, one of the update, in every phase).  It runs in four panels of 16 columns so that the block synchronises 12 times instead of once
// per column: warp 0 eliminates the panel's 16 x 16 diagonal block on its own (warp barriers) and
// records 1 / d_j, then the rows below take the panel's steps in registers (16 lanes per row, the
// row's pivot entries by shuffle), then every thread applies the panel's 16 steps, in order, to
// its elements of the trailing block.  Each element sees the same updates in the same order as a
// column-by-column elimination.  The inverse R = L^-1 (R = I, R_ic -= L_ij R_jc / L_jj for
// i > j >= c, then R_ic / L_ii) is independent per column: four lanes own a column (rows split
// mod 4, held in registers) and pass row j between them by shuffle, with no block barrier.
template <typename T>
__device__ void diag_factor_inverse(T* __restrict__ A, T* __restrict__ Dinv, int np, int k, T* sA, T* sB,
                                    int* __restrict__ status) {
    T* Akk = A + static_cast<size_t>(k) * TS * np + static_cast<size_t>(k) * TS;
    tile_load<T, false>(Akk, np, sA);
    int ii[9], ll[9];
    owned_elements(ii, ll);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ T s_inv[TS];  // 1 / d_j of the elimination, then 1 / L_jj of the inverse
    constexpr int PW = 16;   // panel width
    __syncthreads();
    for (int c0 = 0; c0 < TS; c0 += PW) {
        // (a) the panel's diagonal block, warp 0.  FP32: in registers, lane r holds columns 0-7 of
        // row c0 + r, lane r + 16 its columns 8-15, and pivot entries reach the other lanes by
        // shuffle.  FP64: in shared memory, each lane updating its own few of the block's 120
        // elements, which issues a quarter of the FP64 instructions of the register form (every
        // lane of that form steps through every column).
        if (warp == 0 && sizeof(T) == 8) {
            int ri[4], rl[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int e = lane + 32 * t;  // e < 120: row r, column e - r (r - 1) / 2 + 1
                int r = 1;
                while (r * (r + 1) / 2 <= e) ++r;
                ri[t] = e < 120 ? r : -1;
                rl[t] = e < 120 ? e - r * (r - 1) / 2 + 1 : 0x7fff;
            }
            for (int j = c0; j < c0 + PW; ++j) {
                __syncwarp();
                const T d = sA[j * TP + j];
                if (!(d > T(0))) {
                    if (lane == 0) atomicOr(status, 2);
                }
                const T inv = d > T(0) ? T(1) / d : T(0);
                if (lane == 0) s_inv[j] = inv;
                const int rj = j - c0;
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (rl[t] > rj && ri[t] >= 0) {
                        const int i = c0 + ri[t], l = c0 + rl[t];
                        sA[i * TP + l] = fma(-(sA[i * TP + j] * sA[l * TP + j]), inv, sA[i * TP + l]);
                    }
            }
            __syncwarp();
        } else if (warp == 0) {
            const int ri = lane & 15, half = lane >> 4;
            T a[PW / 2];
#pragma unroll
            for (int q = 0; q < PW / 2; ++q) a[q] = sA[(c0 + ri) * TP + c0 + 8 * half + q];
#pragma unroll
            for (int rj = 0; rj < PW; ++rj) {
                const int hj = rj >> 3;  // half holding column rj
                const T d = __shfl_sync(0xffffffffu, a[rj & 7], rj + 16 * hj);
                if (!(d > T(0))) {
                    if (lane == 0) atomicOr(status, 2);
                }
                const T inv = d > T(0) ? T(1) / d : T(0);
                if (lane == 0) s_inv[c0 + rj] = inv;
                const T aij = __shfl_sync(0xffffffffu, a[rj & 7], ri + 16 * hj);
#pragma unroll
                for (int rl = 1; rl < PW; ++rl) {
                    if (rl <= rj) continue;
                    const T alj = __shfl_sync(0xffffffffu, a[rj & 7], rl + 16 * hj);
                    if (half == (rl >> 3) && ri >= rl) a[rl & 7] = fma(-(aij * alj), inv, a[rl & 7]);
                }
            }
#pragma unroll
            for (int q = 0; q < PW / 2; ++q) sA[(c0 + ri) * TP + c0 + 8 * half + q] = a[q];
        }
        __syncthreads();
        // (b) rows below the diagonal block, panel columns: two rows per warp, a lane per column
        const int nbelow = TS - c0 - PW;
        for (int task = warp; task < nbelow / 2; task += static_cast<int>(blockDim.x >> 5)) {
            const int i = c0 + PW + 2 * task + (lane >> 4), l = c0 + (lane & 15);
            T a = sA[i * TP + l];
#pragma unroll
            for (int j = c0; j < c0 + PW; ++j) {
                const T aij = __shfl_sync(0xffffffffu, a, (lane & 16) | (j - c0));
                if (l > j) a = fma(-(aij * sA[l * TP + j]), s_inv[j], a);
            }
            sA[i * TP + l] = a;
        }
        __syncthreads();
        // (c) the trailing block: elements (i, l), c0 + 16 <= l <= i < 64, the panel's steps in order
        const int m = nbelow, ntrail = m * (m + 1) / 2;
        for (int e = threadIdx.x; e < ntrail; e += blockDim.x) {
            const int t = tri_row(e);
            const int i = c0 + PW + t, l = c0 + PW + (e - t * (t + 1) / 2);
            T a = sA[i * TP + l];
#pragma unroll
            for (int j = c0; j < c0 + PW; ++j) a = fma(-(sA[i * TP + j] * sA[l * TP + j]), s_inv[j], a);
            sA[i * TP + l] = a;
        }
        __syncthreads();
    }
    T v[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        if (ii[s] < 0) continue;
        const T d = sA[ll[s] * TP + ll[s]];
        const T sd = d > T(0) ? sqrt(d) : T(1);
        v[s] = ii[s] == ll[s] ? sd : sA[ii[s] * TP + ll[s]] / sd;
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        if (ii[s] < 0) continue;
        sA[ii[s] * TP + ll[s]] = v[s];
        if (ii[s] != ll[s]) sA[ll[s] * TP + ii[s]] = T(0);
    }
    __syncthreads();
    // 1 / L_jj once per row for the inverse
    if (threadIdx.x < TS) s_inv[threadIdx.x] = T(1) / sA[threadIdx.x * TP + threadIdx.x];
    __syncthreads();
    {
        // column c = 8 warp + lane / 4; this lane holds rows i = part + 4 q
        const int c = 8 * warp + (lane >> 2), part = lane & 3;
        T r[TS / 4];
#pragma unroll
        for (int q = 0; q < TS / 4; ++q) r[q] = part + 4 * q == c ? T(1) : T(0);
#pragma unroll
        for (int j = 0; j < TS; ++j) {
            // row j of the column, final from the steps before j, from the lane that holds it
            const T rj = __shfl_sync(0xffffffffu, r[j >> 2], (lane & ~3) | (j & 3));
            if (8 * warp <= j) {  // some column of this warp has c <= j
                const T inv = s_inv[j];
#pragma unroll
                for (int q = 0; q < TS / 4; ++q) {
                    if (4 * q + 3 <= j) continue;  // every row of this slot is <= j
                    const int i = part + 4 * q;
                    if (i > j && c <= j) r[q] = fma(-(sA[i * TP + j] * rj), inv, r[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < TS / 4; ++q) sB[(part + 4 * q) * TP + c] = r[q];
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 9; ++s)
        if (ii[s] >= 0) v[s] = sB[ii[s] * TP + ll[s]] / sA[ii[s] * TP + ii[s]];
    __syncthreads();
    T* D = Dinv + static_cast<size_t>(k) * TS * TS;
    for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) {
        const int r = e / TS, c = e % TS;
        Akk[static_cast<size_t>(r) * np + c] = sA[r * TP + c];
        D[e] = T(0);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 9; ++s)
        if (ii[s] >= 0) D[ii[s] * TS + ll[s]] = v[s];
}

// C = (accumulate ? C : 0) + alpha * sA sB over one 64x64 tile (row stride ldc).
template <typename T>
__device__ __forceinline__ void tile_product_store(T* __restrict__ C, int ldc, const T* sA, const T* sB, T alpha,
                                                   bool accumulate) {
    T acc[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][q] = T(0);
    tile_mma<T>(sA, sB, acc);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            T* c = C + static_cast<size_t>(ty + 16 * m) * ldc + tx + 16 * q;
            *c = accumulate ? *c + alpha * acc[m][q] : alpha * acc[m][q];
        }
}

template <typename T>
__global__ void __launch_bounds__(256) k_potrf_coop(T* __restrict__ A, T* __restrict__ X, T* __restrict__ Dinv, int np,
                                                   int nt, int* __restrict__ status) {
    cgk::grid_group grid = cgk::this_grid();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);
    T* sB = sA + TS * TP;
    auto tile = [np](T* M, int i, int j) { return M + static_cast<size_t>(i) * TS * np + static_cast<size_t>(j) * TS; };
    // X = I
    const int nrow = np, nthreads = gridDim.x * blockDim.x;
    for (int r = blockIdx.x; r < nrow; r += gridDim.x)
        for (int c = threadIdx.x; c < np; c += blockDim.x) X[static_cast<size_t>(r) * np + c] = r == c ? T(1) : T(0);
    (void)nthreads;
    grid.sync();
    if (blockIdx.x == 0) diag_factor_inverse<T>(A, Dinv, np, 0, sA, sB, status);
    grid.sync();
    for (int k = 0; k < nt; ++k) {
        const int m = nt - 1 - k;
        const T* Dk = Dinv + static_cast<size_t>(k) * TS * TS;
        for (int it = blockIdx.x; it < m + k + 1; it += gridDim.x) {
            if (it < m) {
                // L_ik = A_ik D_k^T
                T* Aik = tile(A, k + 1 + it, k);
                tile_load<T, false>(Aik, np, sA);
                tile_load<T, true>(Dk, TS, sB);
                __syncthreads();
                tile_product_store<T>(Aik, np, sA, sB, T(1), false);
            } else {
                // X_kj = D_k R_kj
                T* Xkj = tile(X, k, it - m);
                tile_load<T, false>(Dk, TS, sA);
                tile_load<T, false>(Xkj, np, sB);
                __syncthreads();
                tile_product_store<T>(Xkj, np, sA, sB, T(1), false);
            }
            __syncthreads();
        }
        grid.sync();
        // Trailing update and R update.  Item 0 is the next diagonal tile (k+1, k+1): block 0
        // updates it and factors it at once (lookahead), while the other blocks share the rest.
        const int ntrail = m * (m + 1) / 2;
        const int nitems = ntrail + m * (k + 1);
        const int first_it = blockIdx.x == 0 ? 0 : (gridDim.x > 1 ? blockIdx.x : 1);
        const int stride = gridDim.x > 1 ? static_cast<int>(gridDim.x) - 1 : 1;
        for (int it = first_it; it < nitems; it = (it == 0 && gridDim.x > 1) ? nitems : it + stride) {
            if (it < ntrail) {
                // A_ij -= L_ik L_jk^T
                const int t = tri_row(it);
                const int i = k + 1 + t, j = k + 1 + (it - t * (t + 1) / 2);
                tile_load<T, false>(tile(A, i, k), np, sA);
                tile_load<T, true>(tile(A, j, k), np, sB);
                __syncthreads();
                tile_product_store<T>(tile(A, i, j), np, sA, sB, T(-1), true);
            } else {
                // R_ij -= L_ik X_kj
                const int q = it - ntrail;
                const int i = k + 1 + q / (k + 1), j = q % (k + 1);
                tile_load<T, false>(tile(A, i, k), np, sA);
                tile_load<T, false>(tile(X, k, j), np, sB);
                __syncthreads();
                tile_product_store<T>(tile(X, i, j), np, sA, sB, T(-1), true);
            }
            __syncthreads();
            if (it == 0 && m > 0) {
                // tile (k+1, k+1) is final: factor it for the next step
                __threadfence_block();
                diag_factor_inverse<T>(A, Dinv, np, k + 1, sA, sB, status);
            }
        }
        grid.sync();
    }
    // X^T into the upper triangle of A (tile (j, i) = X_ij^T, j <= i).  The preconditioner is
    // applied as X^T (X u): forming X^T X explicitly in the factor's precision would square the
    // condition number of its rounding error.
    for (int it = blockIdx.x; it < nt * (nt + 1) / 2; it += gridDim.x) {
        const int i = tri_row(it), j = it - i * (i + 1) / 2;
        tile_load<T, true>(tile(X, i, j), np, sA);
        __syncthreads();
        T* dst = tile(A, j, i);
        for (int e = threadIdx.x; e < TS * TS; e += blockDim.x) {
            const int r = e / TS, c = e % TS;
            dst[static_cast<size_t>(r) * np + c] = sA[r * TP + c];
        }
        __syncthreads();
    }
}

// ---- conjugate gradients on the FP64 reduced matrix, preconditioner D X^T X D (X = L^-1).
// One cooperative persistent kernel runs the whole solve; per iteration four phases separated
// by grid barriers: (1) the direction update fused with the block-CSR SpMV, (2) the x / r
// updates, (3) w = X D r and (4) z = D X^T w (a warp per row).  Grid-wide sums: p.q after (1),
// r.r after (2), r.z after (4).  (Reading r.r together with r.z after (4), one sum fewer, measured
// slower at 500 cameras: 82.7 against 79.0 ms of CG per solve.)
// FP64 arithmetic issues at 1/64 of the FP32 rate on this part: an SM sub-partition retires one
// warp-wide FP64 instruction about every 64 cycles.  The phases are therefore shaped by their
// FP64 instructions per sub-partition rather than by bytes: the SpMV runs as short work items (32
// pose blocks, or 256 entries of a border row, per warp) whose partial sums the owners of the
// rows add in a fixed order, and the dot-product reductions do their FP64 adds on four warps.
// Dot products go through per-block partials that every block sums in the same fixed order, so
// all blocks take the same convergence / breakdown decision and no result depends on timing.
namespace {
constexpr int kCgThreads = 256;
constexpr int kCgWarps = kCgThreads / 32;
constexpr int kCgPart = 4;  // partial slots per block
}  // namespace

// Block sum of v (all threads), written by thread 0 to *dst: warps 0-3 (one per sub-partition)
// each add 64 of the values, thread 0 the four sums.  Every caller passes a grid barrier before
// s_vals / s_q are written again.
__device__ __forceinline__ void block_partial(double v, double* s_vals, double* s_q, double* dst) {
    s_vals[threadIdx.x] = v;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < 4) {
        double t = s_vals[64 * warp + lane] + s_vals[64 * warp + 32 + lane];
        t = warp_sum(t);
        if (lane == 0) s_q[warp] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) *dst = (s_q[0] + s_q[1]) + (s_q[2] + s_q[3]);
}

// Sums over blocks of partial slots `slot` and `slot + 1` (TWO) or `slot` alone, identical in
// every block: warps 0-3 each add a quarter of the blocks' partials (lane l: every 32nd), thread 0
// the four sums, broadcast through s_tot (a grid barrier separates two uses of one slot).
template <bool TWO>
__device__ __forceinline__ void grid_totals(const double* part, int slot, double* s_q, double* s_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = static_cast<int>(gridDim.x);
    if (warp < 4) {
        const int k0 = G * warp / 4, k1 = G * (warp + 1) / 4;
        double t0 = 0.0, t1 = 0.0;
#pragma unroll 4
        for (int k = k0 + lane; k < k1; k += 32) {
            t0 += part[k * kCgPart + slot];
            if (TWO) t1 += part[k * kCgPart + slot + 1];
        }
        t0 = warp_sum(t0);
        if (TWO) t1 = warp_sum(t1);
        if (lane == 0) {
            s_q[4 + warp] = t0;
            if (TWO) s_q[8 + warp] = t1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s_tot[slot] = (s_q[4] + s_q[5]) + (s_q[6] + s_q[7]);
        if (TWO) s_tot[slot + 1] = (s_q[8] + s_q[9]) + (s_q[10] + s_q[11]);
    }
    __syncthreads();
}

// Warp sums of eight per-lane values with nine FP64 adds: a transposing butterfly in which, at
// each of the first three levels, a lane keeps half of its values and adds its partner's share of
// them.  The total of value x ends in lanes 4x .. 4x + 3 (all four hold the same bits).
__device__ __forceinline__ double warp_sum8(double (&a)[8]) {
    const int lane = threadIdx.x & 31;
    {
        const bool up = lane & 16;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double send = up ? a[j] : a[4 + j];
            const double keep = up ? a[4 + j] : a[j];
            a[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
    }
    {
        const bool up = lane & 8;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const double send = up ? a[j] : a[2 + j];
            const double keep = up ? a[2 + j] : a[j];
            a[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
    }
    double t;
    {
        const bool up = lane & 4;
        const double send = up ? a[0] : a[1];
        const double keep = up ? a[1] : a[0];
        t = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    return t;
}

// out_i = so_i * sum_j M_ij in_j over j <= i (LOWER) or j >= i, with in and the product in the
// factor's type T (FP32 on the mixed path: the preconditioner needs no more); one warp per row,
// rows interleaved over all warps of the grid, 16-byte loads from an aligned start (the extra
// elements lie in the diagonal tile, where the triangular factor is zero, and the padding of
// `in` beyond n is zero).  Writes out_t (T) or out_d (double, scaled by so) and returns this
// thread's share of dot_with . out_d.
template <typename T, bool LOWER>
__device__ __forceinline__ double tri_rows(const T* __restrict__ M, int np, int n, const T* __restrict__ in,
                                           T* __restrict__ out_t, double* __restrict__ out_d,
                                           const double* __restrict__ so, const double* __restrict__ dot_with) {
    using V = Vec16<T>;
    using VV = typename V::type;
    const int lane = threadIdx.x & 31;
    // warp-major row order: consecutive rows go to different blocks (SMs)
    const int gw = (threadIdx.x >> 5) * gridDim.x + blockIdx.x, nw = gridDim.x * kCgWarps;
    const VV* in_v = reinterpret_cast<const VV*>(in);
    double contrib = 0.0;
    for (int i = gw; i < n; i += nw) {
        const VV* row = reinterpret_cast<const VV*>(M + static_cast<size_t>(i) * np);
        const int q0 = LOWER ? 0 : i / V::n, q1 = LOWER ? (i + V::n) / V::n : (n + V::n - 1) / V::n;
        T acc = T(0);
#pragma unroll 8
        for (int q = q0 + lane; q < q1; q += 32) acc += V::dot(row[q], in_v[q]);
        acc = warp_sum(acc);
        if (lane == 0) {
            if (out_t) out_t[i] = acc;
            if (out_d) {
                const double v = static_cast<double>(acc) * so[i];
                out_d[i] = v;
                if (dot_with) contrib += dot_with[i] * v;
            }
        }
    }
    return contrib;
}

// Direction update fused with the SpMV: p = z + beta p_old, written to p_new by the first work
// item of each row, and the partial products of S p, with the entries of p formed on the fly by
// the same expression (so bitwise equal to p_new).  On the first iteration (beta == 0) p = z
// exactly, whatever p_old holds.  Work items, one warp each, in the warp-major order that spreads
// consecutive items over the blocks: segment s < pose_seg of pose block row r (its blocks
// 32 s .. 32 s + 31, a lane per block; the border columns with segment 0), then segment
// s < border_seg of border row c (a contiguous 256-entry share of its pose and intrinsic
// columns).  Item sums go to qpart: pose item (r, s) at 6 (r pose_seg + s), border item (c, s)
// at 6 ncb pose_seg + c border_seg + s; q is their sum over s, formed in order where q is read.
// Returns this thread's share of p.q = sum over items of p_i (item sum)_i.
__device__ __forceinline__ double spmv_update(const PcgSystem<double>& sys, const double* __restrict__ z,
                                              double beta, const double* __restrict__ p_old,
                                              double* __restrict__ p_new, double* __restrict__ qpart, int pose_seg,
                                              int border_seg) {
    const int lane = threadIdx.x & 31;
    // warp-major item order: consecutive items go to different blocks (SMs)
    const int gw = (threadIdx.x >> 5) * gridDim.x + blockIdx.x, nw = gridDim.x * kCgWarps;
    const int nb = sys.nb, n6 = 6 * sys.ncb, nrow = n6 + nb;
    const int npose = sys.ncb * pose_seg;
    const bool first = beta == 0.0;
    auto pv = [&](int i) { return first ? z[i] : fma(beta, p_old[i], z[i]); };
    double pq = 0.0;
    for (int t = gw; t < npose + nb * border_seg; t += nw) {
        if (t < npose) {
            const int r = t / pose_seg, sg = t - r * pose_seg;
            const int e0 = sys.row_ptr[r] + 32 * sg, e1 = sys.row_ptr[r + 1];
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const int e = e0 + lane;
            if (e < e1) {
                const int j = sys.col_idx[e];
                const double* A = sys.vals + static_cast<size_t>(e) * 36;
                double pj[6];
#pragma unroll
                for (int c = 0; c < 6; ++c) pj[c] = pv(6 * j + c);
#pragma unroll
                for (int a = 0; a < 6; ++a)
#pragma unroll
                    for (int c = 0; c < 6; ++c) acc[a] = fma(A[a * 6 + c], pj[c], acc[a]);
            }
            if (sg == 0) {
                const double* Bi = sys.border + static_cast<size_t>(r) * 6 * nb;
                for (int c = lane; c < nb; c += 32) {
                    const double pc = pv(n6 + c);
#pragma unroll
                    for (int a = 0; a < 6; ++a) acc[a] = fma(Bi[a * nb + c], pc, acc[a]);
                }
            }
            const double v = warp_sum8(acc);
            const int x = lane >> 2;
            if ((lane & 3) == 0 && x < 6) {
                const int i = 6 * r + x;
                const double pi = pv(i);
                qpart[6 * t + x] = v;
                if (sg == 0) p_new[i] = pi;
                pq += pi * v;
            }
        } else {
            const int u = t - npose, c = u / border_seg, sg = u - c * border_seg;
            const int k0 = min(nrow, 256 * sg), k1 = min(nrow, 256 * (sg + 1));
            const double* Bc = sys.border_t + static_cast<size_t>(c) * n6;
            const double* Cc = sys.Cm + static_cast<size_t>(c) * nb;
            double v = 0.0;
#pragma unroll 4
            for (int k = k0 + lane; k < k1; k += 32) v = fma(k < n6 ? Bc[k] : Cc[k - n6], pv(k), v);
            v = warp_sum(v);
            if (lane == 0) {
                const int i = n6 + c;
                const double pi = pv(i);
                qpart[6 * npose + u] = v;
                if (sg == 0) p_new[i] = pi;
                pq += pi * v;
            }
        }
    }
    return pq;
}

// out: [0] iterations, [1] relative residual, [2] converged, [3] status (1: breakdown)
template <typename T>
__global__ void __launch_bounds__(kCgThreads, 2) k_dense_cg(PcgSystem<double> sys, const T* __restrict__ X,
                                                         const T* __restrict__ XT, int np,
                                                         const double* __restrict__ dscale,
                                                         const double* __restrict__ b, double* __restrict__ x,
                                                         double* __restrict__ r, double* __restrict__ z,
                                                         double* __restrict__ p, double* __restrict__ p2,
                                                         double* __restrict__ qpart, int pose_seg, int border_seg,
                                                         T* __restrict__ u, T* __restrict__ w,
                                                         double* __restrict__ part, double* __restrict__ out,
                                                         double rel_tol, double abs_tol, int max_it) {
    cgk::grid_group grid = cgk::this_grid();
    __shared__ double s_vals[kCgThreads];
    __shared__ double s_q[12];
    __shared__ double s_tot[kCgPart];
    const int n = 6 * sys.ncb + sys.nb;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    double* mypart = part + static_cast<size_t>(blockIdx.x) * kCgPart;
    // r = b, x = 0, u = D r; z = D M u
    double bb = 0.0;
    for (int i = gt; i < n; i += nt) {
        x[i] = 0.0;
        r[i] = b[i];
        u[i] = static_cast<T>(dscale[i] * b[i]);
        bb += b[i] * b[i];
    }
    block_partial(bb, s_vals, s_q, mypart + 0);
    grid.sync();
    tri_rows<T, true>(X, np, n, u, w, nullptr, nullptr, nullptr);
    grid.sync();
    block_partial(tri_rows<T, false>(XT, np, n, w, nullptr, z, dscale, b), s_vals, s_q, mypart + 1);
    grid.sync();
    grid_totals<true>(part, 0, s_q, s_tot);
    const double bnorm = sqrt(s_tot[0]);
    double rz = s_tot[1];
    const double tol = fmax(rel_tol * bnorm, abs_tol);
    double rn = bnorm, beta = 0.0;
    int it = 0, status = 0;
    bool converged = rn <= tol;
    double* p_old = p2;
    double* p_cur = p;
    while (!converged && it < max_it) {
        // p = z + beta p and the partial products of S p (the direction buffers alternate)
        {
            double* t = p_old;
            p_old = p_cur;
            p_cur = t;
        }
        block_partial(spmv_update(sys, z, beta, p_old, p_cur, qpart, pose_seg, border_seg), s_vals, s_q, mypart + 2);
        grid.sync();
        grid_totals<false>(part, 2, s_q, s_tot);
        const double pq = s_tot[2];
        if (!(pq > 0.0) || !isfinite(pq) || !isfinite(rz)) {
            status = 1;
            break;
        }
        const double alpha = rz / pq;
        double rr = 0.0;
        const int n6 = 6 * sys.ncb;
        for (int i = gt; i < n; i += nt) {
            x[i] = fma(alpha, p_cur[i], x[i]);
            // (S p)_i: the row's item sums in order
            double qi;
            if (i < n6) {
                const double* qs = qpart + 6 * (i / 6) * pose_seg + i % 6;
                qi = qs[0];
                for (int sg = 1; sg < pose_seg; ++sg) qi += qs[6 * sg];
            } else {
                const double* qs = qpart + 6 * sys.ncb * pose_seg + (i - n6) * border_seg;
                qi = qs[0];
                for (int sg = 1; sg < border_seg; ++sg) qi += qs[sg];
            }
            const double rv = fma(-alpha, qi, r[i]);
            r[i] = rv;
            u[i] = static_cast<T>(dscale[i] * rv);
            rr += rv * rv;
        }
        block_partial(rr, s_vals, s_q, mypart + 0);
        grid.sync();
        ++it;
        grid_totals<false>(part, 0, s_q, s_tot);
        rn = sqrt(s_tot[0]);
        if (!isfinite(rn)) {
            status = 1;
            break;
        }
        if (rn <= tol) {
            converged = true;
            break;
        }
        tri_rows<T, true>(X, np, n, u, w, nullptr, nullptr, nullptr);
        grid.sync();
        block_partial(tri_rows<T, false>(XT, np, n, w, nullptr, z, dscale, r), s_vals, s_q, mypart + 1);
        grid.sync();
        grid_totals<false>(part, 1, s_q, s_tot);
        const double rz_new = s_tot[1];
        beta = rz_new / rz;
        rz = rz_new;
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
    static std::once_flag attrs;
    std::call_once(attrs, [&] { set_smem<T>(reinterpret_cast<const void*>(&k_potrf_coop<T>), two_tiles); });
    int L = 0;
    cudaMemsetAsync(W.status, 0, sizeof(int), st);
    cudaMemsetAsync(W.A, 0, static_cast<size_t>(np) * np * sizeof(T), st);
    k_dense_scale<<<(n + 255) / 256, 256, 0, st>>>(sys, W.dscale, W.status);
    const long long nfill = static_cast<long long>(sys.row_ptr ? W.nnzb : 0) * 36 + 6LL * sys.ncb * sys.nb +
                            static_cast<long long>(sys.nb) * sys.nb;
    if (nfill > 0) k_dense_fill<T><<<static_cast<unsigned>((nfill + 255) / 256), 256, 0, st>>>(sys, W.dscale, W.A, np);
    k_dense_diag<T><<<(np + 255) / 256, 256, 0, st>>>(W.A, n, np, shift);
    L += 3;
    if (W.fact_grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_potrf_coop<T>, 256, two_tiles);
        W.fact_grid = std::max(1, std::min(per_sm, 2) * sms);
    }
    {
        T* A = W.A;
        T* X = W.X;
        T* Dv = W.Dinv;
        int npv = np, ntv = nt;
        int* stv = W.status;
        void* args[] = {&A, &X, &Dv, &npv, &ntv, &stv};
        // one block per lower tile at most: small systems take a small grid
        const int fgrid = std::max(1, std::min(W.fact_grid, nt * (nt + 1) / 2));
        if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_potrf_coop<T>), dim3(fgrid), dim3(256),
                                        args, two_tiles, st) != cudaSuccess)
            return -1;
        ++L;
    }
    if (launches) *launches += L;
    if (cudaGetLastError() != cudaSuccess) return -1;
    int status = 0;
    cudaMemcpyAsync(&status, W.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    // opt-in trace (PB_GPU_TRACE=1): one line per factorisation
    static const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
    if (trace)
        std::fprintf(stderr, "PB_GPU_FACTOR precision=%d n=%d shift=%.3e status=%d\n", sizeof(T) == 4 ? 1 : 0, n, shift,
                     status);
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
    // one warp per row of the triangular products: small systems (local windows) take a small
    // grid and leave the rest of the device to concurrent work
    const int grid = std::max(1, std::min(W.coop_grid, (W.n + kCgWarps - 1) / kCgWarps));
    PcgSystem<double> s = sys;
    const T* X = W.X;
    const T* XT = W.A;
    int np = W.np;
    const double* dscale = W.dscale;
    double rt = rel_tol, at = abs_tol;
    int mi = max_it;
    int ps = W.pose_seg, bs = W.border_seg;
    void* args[] = {&s, &X, &XT, &np, &dscale, &b, &W.x, &W.r, &W.z, &W.p, &W.w, &W.qpart, &ps, &bs, &W.ut, &W.wt,
                    &W.part, &W.scal, &rt, &at, &mi};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_dense_cg<T>), dim3(grid),
                                                      dim3(kCgThreads), args, 0, st);
    if (e != cudaSuccess) return -1;
    if (launches) *launches += 1;
    cudaMemcpyAsync(h_scal, W.scal, 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *iterations = static_cast<int>(h_scal[0]);
    *relres = h_scal[1];
    *converged = h_scal[2] != 0.0;
    // opt-in trace (PB_GPU_TRACE=1): one line per CG launch
    static const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
    if (trace)
        std::fprintf(stderr, "PB_GPU_CG precision=%d iterations=%d relres=%.3e converged=%d max_it=%d grid=%d\n",
                     sizeof(T) == 4 ? 1 : 0, *iterations, *relres, *converged ? 1 : 0, max_it, grid);
    return h_scal[3] != 0.0 ? 1 : 0;
}

template int dense_factor<float>(const PcgSystem<double>&, DenseWork<float>&, double, cudaStream_t, int*);
template int dense_factor<double>(const PcgSystem<double>&, DenseWork<double>&, double, cudaStream_t, int*);
template int dense_pcg<float>(const PcgSystem<double>&, DenseWork<float>&, const double*, double, double, int, int*,
                              double*, bool*, double*, cudaStream_t, int*);
template int dense_pcg<double>(const PcgSystem<double>&, DenseWork<double>&, const double*, double, double, int, int*,
                               double*, bool*, double*, cudaStream_t, int*);

}  // namespace pb
