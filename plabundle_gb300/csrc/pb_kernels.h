// pb_kernels.h -- launch interface of the GB300 kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "pb_device.cuh"
#include "pb_internal.h"

namespace pb {

constexpr int kMaxAlpha = 8;  // trial step lengths evaluated per objective pass

// Outputs of the assembly kernel (per-chunk partials) and per-track / per-observation data kept
// for the back-substitution.  Partials are the accumulator pairs of Acc<T>: (hi, lo) float pairs
// of the two-sum accumulation on the FP32 path, doubles on the FP64 path.
template <typename T>
struct AsmOutT {
    using P = typename Acc<T>::part_type;
    P* part_pair;     // pair partials * 36
    P* part_cam;      // camera partials * (12 + ng*6*ni)
    P* part_chunk;    // chunks * (nb*nb + 2*nb)
    double* part_cost;
    int* part_flags;  // bit 0: singular point system, bit 1: invalid projection
    double* trk_data; // processed tracks * kTrackRec (FP64 point factor, q, rhs)
    T* obs_rec;       // processed observations: A rows (2 x (6 + ni)) and Y (2 x 3), for the back-substitution
};

// The assembly kernel is instantiated for both precisions; AsmOut carries untyped pointers.
struct AsmOut {
    void* part_pair_v;
    void* part_cam_v;
    void* part_chunk_v;
    double* part_cost;
    int* part_flags;
    void* trk_data_v;
    void* obs_rec_v;
};

// Reduced system of one precision: pose CSR values (both triangles), border B (6*ncb x nb),
// intrinsic block C (nb x nb), rhs and direct rhs (n), result[0] cost, result[1] flags.
template <typename T>
struct RedOut {
    T* vals;
    T* border;
    T* border_t;  // B^T (nb x 6*ncb), for coalesced border rows in the solvers
    T* Cm;
    T* rhs;
    T* direct;
    double* result;
};

// Reduced system extended by the primary point blocks of scale-bar tracks (pb_survey.cu): border
// columns and Cm rows nb .. nb + 3 npr - 1 hold the promoted points.
struct ExtSys {
    double* border;    // 6 ncb x nbx
    double* border_t;  // nbx x 6 ncb
    double* Cm;        // nbx x nbx
    double* rhs;       // nx
    int nbx, nx;       // nb + 3 npr, n + 3 npr
};

template <typename T>
void launch_assemble(const Shape& S, const DevPtrs& D, const AsmOut& O, double damping, size_t smem, cudaStream_t st);
template <typename T>
void launch_reduce(const Shape& S, const DevPtrs& D, const AsmOut& O, const RedOut<double>& R, double damping,
                   cudaStream_t st);
void launch_reduce_sums64(const Shape& S, const DevPtrs& D, const AsmOut& O, const RedOut<double>& R, cudaStream_t st);
// Observations in processing order (cam, u, v, weight and its float-float copy, track) gathered
// from the original-order arrays through obs_orig and trk_obs_begin.
void launch_gather_obs(long long nop, int ntp, const DevPtrs& D, cudaStream_t st);

// terms: processed observations * 3 doubles (per-observation terms, summed per track in order)
template <typename T>
void launch_back_substitute(const Shape& S, const DevPtrs& D, const double* trk_data, const T* obs_rec, const double* step_c,
                            double* step_p, double* terms, double* part, const double* direct64, double* out,
                            cudaStream_t st);
template <typename T>
void launch_linearize_export(const Shape& S, const DevPtrs& D, double* res, double* jp, double* jpose, double* ji,
                             double* nw, double* cost, signed char* valid, cudaStream_t st);
void pb_set_assemble_smem_f32(size_t bytes);
void pb_set_assemble_smem_f64(size_t bytes);
void launch_effective(const Shape& S, const DevPtrs& D, cudaStream_t st);
// Rig problems (pb_rig.cu): capture and sensor state, the chain maps of the camera blocks and the
// reduced system over the rig's pose blocks (captures, then sensors).
constexpr int kRigSegTerms = 64;  // pose terms summed by one warp before the per-block sum
constexpr int kRigItemSeg = 32;   // camera blocks of a rig block summed by one warp (border, rhs)
struct RigDev {
    int ncap, nsen, nrb, ncb, nup, nnzb;
    double* cap_state;   // ncap * 12: rotation (9), centre (3)
    double* sen_state;   // nsen * 12
    double* cap_input;
    double* sen_input;
    double* cap_trial;   // kMaxAlpha * ncap * 12
    double* sen_trial;   // kMaxAlpha * nsen * 12
    double* cap_saved;   // snapshots of pb_gpu_save_state
    double* sen_saved;
    int* cam_capture;    // nc
    int* cam_sensor;     // nc
    int* capture_block;  // ncap: rig block or -1
    int* sensor_block;   // nsen
    int* cb_camera;      // ncb: camera of each camera block
    int* cb_cap;         // ncb: capture rig block, or -1
    int* cb_sen;         // ncb: sensor rig block, or -1
    double* maps;        // ncb * 72: Mc (6x6 row-major, camera delta = Mc capture delta), then Ms
    // rig pose CSR and the term lists of the map (see RigModel)
    int* row_ptr;
    int* col_idx;
    int* diag_pos;
    int* up_pos;
    int* up_tpos;
    int* term_begin;
    int* terms;          // 2 per term: camera-block CSR position, a << 2 | sensor row << 1 | sensor column
    const int* cb_col_idx;  // column indices of the camera-block CSR
    // segments of the pose terms (consecutive terms of one upper block, at most kRigSegTerms):
    // seg_begin[s] first term of segment s (nseg + 1); up_seg_begin[u] first segment of upper
    // block u (nup + 1); seg_part the segments' partial sums (36 each)
    int nseg;
    int* seg_begin;
    int* up_seg_begin;
    double* seg_part;
    // segments of the camera blocks of one rig block (at most kRigItemSeg): bseg_begin[g] first
    // item of segment g (nbseg + 1), blk_seg_begin[I] first segment of rig block I (nrb + 1),
    // bpart the segments' border and rhs partials (6 (nbw + 1) each)
    int nbseg;
    int* bseg_begin;
    int* blk_seg_begin;
    double* bpart;
    int* blk_begin;
    int* blk_items;
    // the rig system: pose blocks, border (6 nrb x nbw) and its transpose, right-hand side
    double* vals;
    double* border;
    double* border_t;
    double* rhs;
    double* xv;          // the solution mapped back to camera blocks (6 ncb + nbw)
    double* step_r;      // the rig solution (6 nrb + nbw), read by the trial states
    double* sq;          // squared sum of the rig solution's pose and intrinsic entries
};
void launch_rig_maps(const RigDev& R, cudaStream_t st);
// The camera-block system (vals, border of width nbw, rhs of 6 ncb + nbw) onto the rig blocks;
// the rig pose diagonal damped by finalizePrimaryDiagonal(1 + damping, 1).
void launch_rig_transform(const RigDev& R, const double* vals, const double* border, const double* rhs, int nbw,
                          double damping, cudaStream_t st);
// xr (6 nrb + nbw) -> R.xv (6 ncb + nbw), R.step_r = xr, R.sq = sum of xr^2 over 6 nrb + nglob.
void launch_rig_expand(const RigDev& R, const double* xr, int nbw, int nglob, cudaStream_t st);
// Trial captures, sensors and composed camera poses (pose entries 0-11 of the trial cameras).
void launch_rig_trial(const RigDev& R, int nc, const double* alphas, int n_alpha, double* cams_trial, cudaStream_t st);
void launch_rig_accept(const RigDev& R, int a, cudaStream_t st);

void launch_cost(const Shape& S, const DevPtrs& D, const double* step_c, const double* step_p, const double* alphas,
                 int n_alpha, int use_trial, double* part, double* out, cudaStream_t st,
                 const RigDev* rig = nullptr);
void launch_accept(const Shape& S, const DevPtrs& D, const double* step_p, double alpha, int a, cudaStream_t st);
// Scale bars (pb_survey.cu): the extended system of the current state (`flags` bit 2: a promoted
// observation did not project; `bar_cost`: the bars' robust cost), the split of its solution into
// the camera / intrinsic step and the promoted point steps (`out`: their squared sum), and the
// bars' cost of the trial states or of the current state.
void launch_extend_system(const Shape& S, const DevPtrs& D, const RedOut<double>& R, const ExtSys& X, double damping,
                          int* flags, double* bar_cost, cudaStream_t st);
void launch_ext_step(const Shape& S, const DevPtrs& D, const double* xsol, double* step_c, double* step_p, double* out,
                     cudaStream_t st);
void launch_bar_cost(const Shape& S, const DevPtrs& D, const double* step_p, const double* alphas, int n_alpha,
                     int use_trial, double* out, cudaStream_t st);
void launch_strict_rms(const Shape& S, const DevPtrs& D, const double* cams, const double* init_points,
                       const int* proc_of_track, int use_state, int nt, double* out, cudaStream_t st);
// Quality finalisation on the device (finalizeBundleAdjustResult): out[0] filter threshold,
// out[1] candidate tracks, out[2] kept tracks, out[3] / out[4] sums of the kept tracks' RMS before
// / after; valid[nt] the valid mask.  part: quality_part_size(nt) doubles.
size_t quality_part_size(int nt);
void launch_quality(int nt, const signed char* active, const double* rms_before, const double* rms_after, int enable,
                    double max_err, double sigma, signed char* valid, double* part, double* out, cudaStream_t st);

// PCG (pb_pcg.cu)
template <typename T>
struct PcgSystem {
    int ncb, nb, ng, ni;
    const int* row_ptr;
    const int* col_idx;
    const int* diag_pos;
    const T* vals;
    const T* border;
    const T* border_t;  // B^T, nb x 6*ncb
    const T* Cm;
    T* Dinv;       // ncb * 36 block-Jacobi inverses
    T* Cinv;       // ng * ni * ni
};

struct PcgResult {
    int iterations;
    int converged;
    int status;     // 0 ok, 1 breakdown (not positive definite), 2 preconditioner not SPD
    double rnorm;
    double bnorm;
};

template <typename T>
int pcg_precondition(const PcgSystem<T>& sys, int* d_status, cudaStream_t st);
// Solves sys x = b with block-Jacobi PCG in one cooperative persistent kernel.
template <typename T>
int pcg_solve(const PcgSystem<T>& sys, const T* b, T* x, T* work, double* partials, PcgResult* d_result,
              double abs_tol, double rel_tol, int max_iter, int grid, cudaStream_t st);
template <typename T>
int pcg_grid_size(int ncb);
// r64 = b64 - A x64 (FP64 accumulation over the stored matrix), returns norms in out[0..1].
template <typename T>
void residual64(const PcgSystem<T>& sys, const double* b64, const double* x64, double* r64, double* out,
                cudaStream_t st);
// Dense Cholesky preconditioner + FP64 CG (pb_dense.cu).  A holds the scaled matrix, then its
// factor L, then X^T; X holds L^-1; Dinv the inverses of the diagonal tiles of L.
template <typename T>
struct DenseWork {
    int n = 0, np = 0, nt = 0, nnzb = 0;
    T* A = nullptr;
    T* X = nullptr;
    T* Dinv = nullptr;
    double* dscale = nullptr;
    int* status = nullptr;
    double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *w = nullptr;
    // SpMV work items of the CG: pose_seg per pose block row (32 blocks each), border_seg per border
    // row (256 entries each); qpart holds their sums (6 ncb pose_seg + nb border_seg doubles)
    int pose_seg = 0, border_seg = 0;
    double* qpart = nullptr;
    T *ut = nullptr, *wt = nullptr;  // scaled residual and X D r in the factor's type
    double* part = nullptr;  // per-block partials of the cooperative CG (grid * 4)
    double* scal = nullptr;
    int coop_grid = 0;       // blocks of the cooperative CG launch
    int fact_grid = 0;       // blocks of the cooperative factorisation
};

template <typename T>
size_t dense_bytes(int n);
// Returns 0 on success, a status bitmask when the scaled matrix is not positive definite at this
// shift (bit 1: non-positive diagonal, bit 2: non-positive pivot), -1 on a CUDA error.
template <typename T>
int dense_factor(const PcgSystem<double>& sys, DenseWork<T>& W, double shift, cudaStream_t st, int* launches);
// CG on S x = b (FP64 S and vectors); the solution is left in W.x.  Returns 0, 1 on breakdown,
// -1 on a CUDA error.
template <typename T>
int dense_pcg(const PcgSystem<double>& sys, DenseWork<T>& W, const double* b, double rel_tol, double abs_tol,
              int max_it, int* iterations, double* relres, bool* converged, double* h_scal, cudaStream_t st,
              int* launches);

// Backward pass (pb_adjoint.cu).  Per-observation record of the exact Hessian in the local chart
// (pose 6 | point 3 | intrinsic columns ni): pose-pose (upper 6x6), pose-point (6x3), point-point
// (upper 3x3), pose-intrinsic (6 x ni), point-intrinsic (3 x ni), intrinsic (upper ni x ni), the
// FP64 Jacobian rows (2 x (9 + ni)), W2 = 2 rho' w I + 4 rho'' w^2 r r^T (3) and lam = 2 rho' w r (2).
struct AdjLayout {
    int ni = 0, stride = 0;
    __host__ __device__ int hcc() const { return 0; }
    __host__ __device__ int hcp() const { return 21; }
    __host__ __device__ int hpp() const { return 39; }
    __host__ __device__ int hck() const { return 45; }
    __host__ __device__ int hpk() const { return 45 + 6 * ni; }
    __host__ __device__ int hkk() const { return 45 + 9 * ni; }
    __host__ __device__ int jac() const { return 45 + 9 * ni + ni * (ni + 1) / 2; }
    __host__ __device__ int w2() const { return jac() + 2 * (9 + ni); }
    static AdjLayout make(int n_int) {
        AdjLayout L;
        L.ni = n_int;
        L.stride = L.w2() + 5;
        return L;
    }
};
constexpr int kAdjMaxStride = 68 + 11 * kMaxNI + kMaxNI * (kMaxNI + 1) / 2;

struct AdjBuffers {
    AdjLayout lay;
    double* rec;            // nop * stride
    double* vinv;           // ntp * 9 inverse point blocks
    double* gpt;            // ntp * 3 dL/d(final point), world (processing order)
    double* gcam;           // nc * 6 dL/d(final pose): rotation increment, world centre
    double* gint;           // ng * kP dL/d(group parameters)
    double* mu_p;           // ntp * 3 point part of the adjoint solution (point chart)
    double* grad_obs;       // nop * 2 dL/d(u, v) (processing order)
    double* grad_fixed_cam; // nc * 6 cross terms of fixed cameras (zeroed by the caller)
    double* grad_fixed_pt;  // ntp * 3 cross terms of fixed tracks (world)
    double* gauge;          // 4: cross terms of the anchor centre (3) and the gauge baseline (zeroed)
    AsmOut part;            // FP64 chunk partials of the point elimination
    int newton;             // 1: right-hand side -grad F (a Newton step of the objective) instead of dL/dz
    int* flags;             // bit 0: singular point block, bit 1: invalid projection, bit 2: pattern miss
};

void launch_adjoint_hessian(const Shape& S, const DevPtrs& D, const AdjBuffers& B, cudaStream_t st);
void launch_adjoint_rhs(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const RedOut<double>& R, cudaStream_t st);
size_t adjoint_assemble_smem(const Shape& S);
// Point elimination into FP64 chunk partials (part: part_pair_v / part_cam_v / part_chunk_v as
// double, part_cost / part_flags zero), their reduction into R, and the finalisation.
void launch_adjoint_schur(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const AsmOut& part,
                          const RedOut<double>& R, cudaStream_t st);
void launch_adjoint_gradient(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const double* mu, cudaStream_t st);

// Damped Schur solves of host block normal equations (pb_schur.cu).
struct SchurWork;
SchurWork* schur_work_create();
void schur_work_destroy(SchurWork* w);
int schur_solve(SchurWork* w, int device, cudaStream_t st, const pb_bne* eq, double damping, const pb_schur_options& op,
                double* primary_step, double* eliminated_step, pb_schur_report* report, std::string* err);

void to_double(const float* in, double* out, int n, cudaStream_t st);
void to_double(const double* in, double* out, int n, cudaStream_t st);
void to_float(const double* in, float* out, int n, cudaStream_t st);
void axpy64(double* x, const float* d, int n, cudaStream_t st);

}  // namespace pb
