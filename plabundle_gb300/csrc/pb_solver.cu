// pb_solver.cu -- context (workspace), device buffers, the Levenberg-Marquardt / Armijo driver of
// the online reduced-Schur path, and the C ABI declared in include/pb_gpu.h.
//
// The driver restates optimizePointsWithPlaMatrix's online branch
// (src/internal/BundleAdjustPlaMatrix.cpp:162-631): relinearise, eliminate points, solve the
// reduced system, back-substitute, Armijo line search with alpha = 1, 1/2, ... on the FP64
// objective, damping x10 on a singular point system / linear failure, /10 on acceptance, and
// termination when the line search fails.  Trial step lengths are evaluated in batches on the
// device; the first one that meets the reference rule is accepted, so the accepted step equals
// the serial search's.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <limits>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "pb_kernels.h"

using namespace pb;

namespace {

constexpr double kNaN = std::numeric_limits<double>::quiet_NaN();
constexpr double kInfD = std::numeric_limits<double>::infinity();

// Device memory of a context: slabs carved by a bump pointer (256-byte aligned).  release()
// rewinds the slabs for the next problem instead of freeing them, so a context that solves one
// problem after another (local-BA windows) stops calling cudaMalloc once its slabs are large
// enough; free_all() returns the memory.  Buffers are not cleared: whatever must start at zero
// is set explicitly by its user.
struct DeviceArena {
    struct Slab {
        char* base;
        size_t size, used;
    };
    std::vector<Slab> slabs;
    size_t bytes = 0;
    static constexpr size_t kAlign = 256, kMinSlab = size_t(8) << 20;
    template <typename T>
    T* alloc(size_t count) {
        if (count == 0) count = 1;
        const size_t need = (count * sizeof(T) + kAlign - 1) & ~(kAlign - 1);
        for (Slab& sl : slabs)
            if (sl.size - sl.used >= need) {
                T* p = reinterpret_cast<T*>(sl.base + sl.used);
                sl.used += need;
                bytes += need;
                return p;
            }
        const size_t size = std::max(need, kMinSlab);
        void* p = nullptr;
        if (cudaMalloc(&p, size) != cudaSuccess) throw std::bad_alloc();
        slabs.push_back({static_cast<char*>(p), size, need});
        bytes += need;
        return static_cast<T*>(p);
    }
    void release() {
        for (Slab& sl : slabs) sl.used = 0;
        bytes = 0;
    }
    void free_all() {
        for (Slab& sl : slabs) cudaFree(sl.base);
        slabs.clear();
        bytes = 0;
    }
};

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Assembly outputs of one arithmetic type (chunk partials, per-track factors, robust weights).
template <typename T>
struct PrecisionBuffers {
    bool ready = false;
    AsmOut out{};
};

}  // namespace

struct pb_gpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string error;
    HostModel model;
    bool uploaded = false;
    long long structure_hash = 0;
    int pattern_builds = 0, pattern_reuses = 0;
    DeviceArena arena;   // structure buffers
    DeviceArena parena[2];
    Shape S[2]{};
    DevPtrs D[2]{};
    PrecisionBuffers<double> p64;
    PrecisionBuffers<float> p32;
    // reduced system (FP64 on both paths) and its solvers
    RedOut<double> red{};
    PcgSystem<double> sys{};
    double* pcg_x = nullptr;
    double* pcg_work = nullptr;
    int pcg_grid = 1;
    DeviceArena darena;           // dense preconditioner buffers (depend on the reduced dimension only)
    DenseWork<float> dw32;
    DenseWork<double> dw64;
    double shift32 = 1e-7;  // last FP32 factor shift that factorised
    int f32_age = -1;       // LM solves served by the current kept dense factor (-1: none)
    int factor_reuse = 0;   // pb_solve_options.factor_reuse of the running solve
    bool f32_stale = false; // the last accepted step changed the cost by more than 1 %
    int f32_base_iters = 0; // CG iterations of the first solve with that factor
    bool dense_ready[2] = {false, false};
    int last_solver = 0;
    // shared FP64 buffers
    double* groups_init = nullptr;
    double* step_c = nullptr;
    double* step_p = nullptr;
    double* direct64 = nullptr;
    double* rhs64 = nullptr;
    double* x64 = nullptr;
    double* r64 = nullptr;
    double* res_out = nullptr;
    double* bs_part = nullptr;
    double* bs_terms = nullptr;  // per processed observation: its term of the point back-substitution
    double* bs_out = nullptr;
    double* cost_part = nullptr;
    double* cost_out = nullptr;
    double* alphas_d = nullptr;
    double* pcg_part = nullptr;
    PcgResult* pcg_res = nullptr;
    int* pre_status = nullptr;
    double* rms_before_d = nullptr;
    double* rms_after_d = nullptr;
    signed char* active_d = nullptr;   // nt: active-track mask
    signed char* valid_d = nullptr;    // nt: valid mask of the last solve
    double* quality_part = nullptr;
    double* quality_out = nullptr;     // threshold, candidates, kept, sum RMS before / after
    bool quality_host_stale = false;   // valid / rms_after live on the device only
    double* init_points_all = nullptr;
    int* proc_of_track = nullptr;
    // pinned host scratch
    double* h_scratch = nullptr;
    // results of the last solve
    std::vector<double> rms_before, rms_after;
    std::vector<signed char> valid;
    int last_precision = PB_PRECISION_FP64;
    bool have_system = false;
    volatile int cancel = 0;
    // timing
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double kt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int launches = 0;
    int solved = 0;
    // backward pass (exact-Hessian records and outputs) and the state snapshot
    DeviceArena aarena;
    AdjBuffers adj{};
    bool adj_ready = false;
    int adj_prec = 0;
    DeviceArena sarena;
    double* snap_cams = nullptr;
    double* snap_points = nullptr;
    double* snap_groups = nullptr;
    bool snap_valid = false;
    std::vector<long long> proc_of_obs;  // original observation -> processing index (-1: not processed)
    // damped Schur solves of host block normal equations (pb_gpu_solve_damped_schur)
    SchurWork* schur = nullptr;
    // scale bars: the reduced system extended by the promoted points (pb_survey.cu)
    bool ext_on = false;
    ExtSys ext{};
    PcgSystem<double> sysx{};
    int* ext_flags = nullptr;
    double* bar_d = nullptr;  // bar cost of the current state, then of the trial states
    // cost history of the last solve: the initial cost, then the cost after every accepted step,
    // with the LM iteration and the host time since the solve started
    std::vector<int> hist_it;
    std::vector<double> hist_cost, hist_ms;
    // rigs: capture / sensor state and the reduced system over the rig's pose blocks (pb_rig.cu)
    bool rig_on = false;
    RigDev rig{};
    PcgSystem<double> sysr{};
};

namespace {

size_t smem_budget(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    return v > 0 ? static_cast<size_t>(v) - 1024 : 48 * 1024;
}

template <typename T>
void upload(T* dst, const std::vector<T>& src, cudaStream_t st) {
    if (!src.empty()) check(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st), "H2D");
}

template <typename T>
T* upload_new(DeviceArena& a, const std::vector<T>& src, cudaStream_t st) {
    T* p = a.alloc<T>(src.size());
    upload(p, src, st);
    return p;
}

void group_record(const HostGroup& g, double* rec) {
    for (int p = 0; p < kP; ++p) {
        rec[p] = g.params[p];
        rec[kP + p] = g.prior[p];
        rec[2 * kP + p] = g.invSigma[p];
        rec[3 * kP + p] = g.lower[p];
        rec[4 * kP + p] = g.upper[p];
        rec[5 * kP + p] = g.enabled[p] ? 1.0 : 0.0;
    }
}

// Builds the structure buffers shared by both precisions.
void upload_structure(pb_gpu_ctx* c) {
    HostModel& m = c->model;
    DeviceArena& A = c->arena;
    cudaStream_t st = c->stream;
    const int nc = m.nc, nt = m.nt, ntp = static_cast<int>(m.trk_order.size());
    const long long nop = static_cast<long long>(m.p_obs_orig.size());
    DevPtrs D{};
    Shape S{};
    S.nc = nc;
    S.ntp = ntp;
    S.nop = nop;
    S.ncb = m.ncb;
    S.ng = m.ng;
    S.ni = m.ni;
    S.nb = m.ng * m.ni;
    S.n = 6 * m.ncb + S.nb;
    S.nupper = static_cast<int>(m.up_row.size());
    S.nnzb = static_cast<int>(m.col_idx.size());
    S.loss = m.loss;
    S.loss_scale = m.loss_scale;
    // a rig camera never takes the gauge tangent (cameraPosePrimaryTerms,
    // BundleAdjustPlaMatrixAssembly.cpp:204): the capture of the scale camera is fixed instead
    S.rig = m.rig.on ? 1 : 0;
    S.gauge_anchor = m.rig.on ? -1 : m.gauge_anchor;
    S.gauge_scale = m.rig.on ? -1 : m.gauge_scale;
    S.gauge_baseline = m.rig.on ? 0.0 : m.gauge_baseline;
    for (int i = 0; i < kMaxNI; ++i) S.int_cols[i] = i < m.ni ? m.int_cols[i] : 0;
    S.ref_param = m.ref_param ? 1 : 0;
    S.ncp = static_cast<int>(m.cp_proc.size() / 12);
    S.cp_huber = m.cp_huber;
    S.npr = m.npr;
    S.nbar = static_cast<int>(m.bar_tracks.size() / 2);
    S.bar_huber = m.bar_huber;
    {
        const float2 ls = ff_pack(m.loss_scale);
        S.loss_scale_hi = ls.x;
        S.loss_scale_lo = ls.y;
    }

    D.cams_input = upload_new(A, m.cams_in, st);
    D.cams_ref = upload_new(A, m.cams_ref, st);
    D.cams_state = A.alloc<double>(m.cams_in.size());
    D.cams_eff = A.alloc<double>(m.cams_in.size());
    D.cams_ff = A.alloc<float2>(static_cast<size_t>(nc) * kCamFF);
    D.cams_trial = A.alloc<double>(static_cast<size_t>(kMaxAlpha) * m.cams_in.size());
    D.cam_block = upload_new(A, m.camera_block, st);
    std::vector<int> grp(nc, -1);
    if (m.ng > 0) grp = m.calib_group;
    D.cam_group = upload_new(A, grp, st);
    std::vector<double> groups(std::max(1, m.ng) * kGroupRec, 0.0);
    for (int g = 0; g < m.ng; ++g) group_record(m.groups[g], &groups[static_cast<size_t>(g) * kGroupRec]);
    c->groups_init = upload_new(A, groups, st);
    D.groups = A.alloc<double>(groups.size());
    D.groups_trial = A.alloc<double>(static_cast<size_t>(kMaxAlpha) * groups.size());
    D.gauge_basis = A.alloc<double>(12);
    check(cudaMemsetAsync(D.gauge_basis, 0, 12 * sizeof(double), st), "memset");
    // tracks in processing order
    std::vector<int> tblock(ntp), torig(ntp);
    std::vector<double> pts(static_cast<size_t>(ntp) * 3);
    for (int p = 0; p < ntp; ++p) {
        const int t = m.trk_order[p];
        torig[p] = t;
        tblock[p] = m.track_block[t];
        for (int a = 0; a < 3; ++a) pts[static_cast<size_t>(p) * 3 + a] = m.points_in[static_cast<size_t>(t) * 3 + a];
    }
    D.trk_obs_begin = upload_new(A, m.trk_obs_begin, st);
    D.trk_block = upload_new(A, tblock, st);
    {
        // points that move (eliminated or promoted) and the scale-bar records in processing order
        std::vector<int> tfree(ntp), tprom(ntp, -1), pproc(std::max(1, m.npr), 0);
        std::vector<int> pot_h(nt, -1);
        for (int p = 0; p < ntp; ++p) {
            const int t = m.trk_order[p];
            pot_h[t] = p;
            tprom[p] = m.track_prom.empty() ? -1 : m.track_prom[t];
            tfree[p] = (m.track_block[t] >= 0 || tprom[p] >= 0) ? 1 : 0;
            if (tprom[p] >= 0) pproc[tprom[p]] = p;
        }
        D.trk_free = upload_new(A, tfree, st);
        D.trk_prom = upload_new(A, tprom, st);
        D.prom_proc = upload_new(A, pproc, st);
        const int nbar = static_cast<int>(m.bar_tracks.size() / 2);
        std::vector<int> bp(std::max(1, 2 * nbar), -1);
        std::vector<double> bpar(std::max(1, 2 * nbar), 0.0);
        for (int i = 0; i < nbar; ++i) {
            for (int e = 0; e < 2; ++e) {
                const int t = m.bar_tracks[2 * i + e];
                bp[2 * i + e] = m.active_track[t] ? pot_h[t] : -1;
            }
            // linearizeScaleBar: weight = scaleBarWeight * weight, residual scale sqrt(weight) / sigma
            const double* d = &m.bar_data[static_cast<size_t>(i) * 3];
            bpar[2 * i] = d[0];
            bpar[2 * i + 1] = std::sqrt(m.bar_weight * d[2]) / std::max(1e-9, d[1]);
        }
        D.bar_pidx = upload_new(A, bp, st);
        D.bar_par = upload_new(A, bpar, st);
    }
    D.trk_orig = upload_new(A, torig, st);
    D.points0 = upload_new(A, pts, st);
    D.points = A.alloc<double>(pts.size());
    D.pscale = A.alloc<double>(std::max<size_t>(1, pts.size() / 3));
    D.pscale_ff = A.alloc<float2>(std::max<size_t>(1, pts.size() / 3));
    {
        std::vector<int> cpb = m.trk_cp_begin;
        if (cpb.empty()) cpb.assign(static_cast<size_t>(ntp) + 1, 0);
        D.trk_cp_begin = upload_new(A, cpb, st);
        std::vector<double> cpr = m.cp_proc;
        if (cpr.empty()) cpr.assign(12, 0.0);
        D.cp_rec = upload_new(A, cpr, st);
    }
    // observations: the original-order arrays (strict RMS) are uploaded once, and the
    // processing-order arrays are gathered from them on the device
    std::vector<int> rbad(m.no, 0);
    std::vector<double> rw(m.no, 0.0);
    for (long long k = 0; k < m.no; ++k) {
        const double w = std::isfinite(m.obs_weight[k]) && m.obs_weight[k] > 0 ? m.obs_weight[k] : 0.0;
        const double s = std::isfinite(m.obs_scale[k]) && m.obs_scale[k] > 0 ? m.obs_scale[k] : 1.0;
        rw[k] = w / (s * s);
        const int cam = m.obs_cam[k];
        rbad[k] = (rw[k] > 0.0 && (cam < 0 || cam >= nc || !std::isfinite(m.obs_u[k]) || !std::isfinite(m.obs_v[k]))) ? 1 : 0;
    }
    std::vector<int> rcam(m.obs_cam);
    for (auto& v : rcam) v = (v >= 0 && v < nc) ? v : 0;
    D.raw_offsets = upload_new(A, m.offs, st);
    D.raw_cam = upload_new(A, rcam, st);
    D.raw_u = upload_new(A, m.obs_u, st);
    D.raw_v = upload_new(A, m.obs_v, st);
    D.raw_w = upload_new(A, rw, st);
    D.raw_bad = upload_new(A, rbad, st);
    D.obs_orig = upload_new(A, m.p_obs_orig, st);
    D.obs_cam = A.alloc<int>(static_cast<size_t>(std::max<long long>(1, nop)));
    D.obs_u = A.alloc<double>(static_cast<size_t>(std::max<long long>(1, nop)));
    D.obs_v = A.alloc<double>(static_cast<size_t>(std::max<long long>(1, nop)));
    D.obs_w = A.alloc<double>(static_cast<size_t>(std::max<long long>(1, nop)));
    D.obs_w_ff = A.alloc<float2>(static_cast<size_t>(std::max<long long>(1, nop)));
    D.obs_trk = A.alloc<int>(static_cast<size_t>(std::max<long long>(1, nop)));
    launch_gather_obs(nop, ntp, D, st);
    check(cudaGetLastError(), "gather launch");
    // pose CSR
    D.row_ptr = upload_new(A, m.row_ptr, st);
    D.col_idx = upload_new(A, m.col_idx, st);
    D.diag_pos = upload_new(A, m.diag_pos, st);
    D.up_csr = upload_new(A, m.up_csr, st);
    D.up_csr_t = upload_new(A, m.up_csr_t, st);
    // initial points of every track for the strict RMS before
    c->init_points_all = upload_new(A, m.points_in, st);
    std::vector<int> pot(nt, -1);
    for (int p = 0; p < ntp; ++p) pot[m.trk_order[p]] = p;
    c->proc_of_track = upload_new(A, pot, st);
    // FP64 work buffers
    const int n = S.n;
    c->step_c = A.alloc<double>(n);
    c->step_p = A.alloc<double>(static_cast<size_t>(ntp) * 3);
    c->rhs64 = A.alloc<double>(n);
    c->x64 = A.alloc<double>(n);
    c->r64 = A.alloc<double>(n);
    c->res_out = A.alloc<double>(2 + static_cast<size_t>(std::max(1, (m.ncb + 7) / 8)) * kMaxNB);
    const int bs_blocks = std::max(1, (ntp + 255) / 256);
    c->bs_part = A.alloc<double>(2 * static_cast<size_t>(bs_blocks));
    c->bs_terms = A.alloc<double>(3 * static_cast<size_t>(std::max<long long>(1, nop)));
    c->bs_out = A.alloc<double>(4);
    const long long cost_blocks = std::max<long long>(1, (nop + 255) / 256);
    c->cost_part = A.alloc<double>(static_cast<size_t>(cost_blocks) * kMaxAlpha * 2);
    c->cost_out = A.alloc<double>(kMaxAlpha);
    c->alphas_d = A.alloc<double>(kMaxAlpha);
    c->pcg_res = A.alloc<PcgResult>(1);
    c->pre_status = A.alloc<int>(1);
    c->rms_before_d = A.alloc<double>(nt);
    c->rms_after_d = A.alloc<double>(nt);
    c->active_d = upload_new(A, m.active_track, st);
    c->valid_d = A.alloc<signed char>(nt);
    c->quality_part = A.alloc<double>(quality_part_size(nt));
    c->quality_out = A.alloc<double>(5);
    c->quality_host_stale = false;
    // reduced system (FP64) and the block-Jacobi PCG buffers
    c->red.vals = A.alloc<double>(static_cast<size_t>(std::max(1, S.nnzb)) * 36);
    c->red.border = A.alloc<double>(static_cast<size_t>(std::max(1, S.ncb)) * 6 * std::max(1, S.nb));
    c->red.border_t = A.alloc<double>(static_cast<size_t>(std::max(1, S.ncb)) * 6 * std::max(1, S.nb));
    c->red.Cm = A.alloc<double>(static_cast<size_t>(std::max(1, S.nb * S.nb)));
    c->red.rhs = A.alloc<double>(std::max(1, n));
    c->red.direct = A.alloc<double>(std::max(1, n));
    c->red.result = A.alloc<double>(2);
    check(cudaMemsetAsync(c->red.vals, 0, static_cast<size_t>(std::max(1, S.nnzb)) * 36 * sizeof(double), st), "memset");
    check(cudaMemsetAsync(c->red.border, 0, static_cast<size_t>(std::max(1, S.ncb)) * 6 * std::max(1, S.nb) * sizeof(double), st),
          "memset");
    check(cudaMemsetAsync(c->red.border_t, 0, static_cast<size_t>(std::max(1, S.ncb)) * 6 * std::max(1, S.nb) * sizeof(double), st),
          "memset");
    c->direct64 = c->red.direct;
    PcgSystem<double>& sy = c->sys;
    sy.ncb = S.ncb;
    sy.nb = S.nb;
    sy.ng = S.ng;
    sy.ni = S.ni;
    sy.row_ptr = D.row_ptr;
    sy.col_idx = D.col_idx;
    sy.diag_pos = D.diag_pos;
    sy.vals = c->red.vals;
    sy.border = c->red.border;
    sy.border_t = c->red.border_t;
    sy.Cm = c->red.Cm;
    sy.Dinv = A.alloc<double>(static_cast<size_t>(std::max(1, S.ncb)) * 36);
    sy.Cinv = A.alloc<double>(static_cast<size_t>(std::max(1, S.ng)) * kMaxNI * kMaxNI);
    c->pcg_x = A.alloc<double>(std::max(1, n));
    c->pcg_work = A.alloc<double>(static_cast<size_t>(std::max(1, n)) * 4);
    c->ext_on = S.nbar > 0;
    if (c->ext_on) {
        ExtSys& X = c->ext;
        X.nbx = S.nb + 3 * S.npr;
        X.nx = n + 3 * S.npr;
        X.border = A.alloc<double>(static_cast<size_t>(std::max(1, 6 * S.ncb)) * std::max(1, X.nbx));
        X.border_t = A.alloc<double>(static_cast<size_t>(std::max(1, 6 * S.ncb)) * std::max(1, X.nbx));
        X.Cm = A.alloc<double>(static_cast<size_t>(std::max(1, X.nbx)) * std::max(1, X.nbx));
        X.rhs = A.alloc<double>(std::max(1, X.nx));
        c->sysx = sy;
        c->sysx.nb = X.nbx;
        c->sysx.border = X.border;
        c->sysx.border_t = X.border_t;
        c->sysx.Cm = X.Cm;
        c->ext_flags = A.alloc<int>(1);
        c->bar_d = A.alloc<double>(kMaxAlpha + 2);  // [0] current, [1 .. kMaxAlpha] trials, then the step sum
    }
    c->rig_on = m.rig.on;
    if (c->rig_on) {
        const RigModel& rm = m.rig;
        RigDev& R = c->rig;
        R = RigDev{};
        R.ncap = rm.ncap;
        R.nsen = rm.nsen;
        R.nrb = rm.nrb;
        R.ncb = m.ncb;
        R.nup = static_cast<int>(rm.up_pos.size());
        R.nnzb = static_cast<int>(rm.col_idx.size());
        R.cap_input = upload_new(A, rm.cap_in, st);
        R.sen_input = upload_new(A, rm.sen_in, st);
        R.cap_state = A.alloc<double>(rm.cap_in.size());
        R.sen_state = A.alloc<double>(rm.sen_in.size());
        R.cap_trial = A.alloc<double>(static_cast<size_t>(kMaxAlpha) * rm.cap_in.size());
        R.sen_trial = A.alloc<double>(static_cast<size_t>(kMaxAlpha) * rm.sen_in.size());
        R.cap_saved = A.alloc<double>(rm.cap_in.size());
        R.sen_saved = A.alloc<double>(rm.sen_in.size());
        R.cam_capture = upload_new(A, rm.cam_capture, st);
        R.cam_sensor = upload_new(A, rm.cam_sensor, st);
        std::vector<int> kb = rm.capture_block, sb = rm.sensor_block;
        if (kb.empty()) kb.assign(rm.ncap, -1);
        if (sb.empty()) sb.assign(rm.nsen, -1);
        R.capture_block = upload_new(A, kb, st);
        R.sensor_block = upload_new(A, sb, st);
        R.cb_camera = upload_new(A, rm.cb_camera, st);
        R.cb_cap = upload_new(A, rm.cb_cap_block, st);
        R.cb_sen = upload_new(A, rm.cb_sen_block, st);
        R.maps = A.alloc<double>(static_cast<size_t>(std::max(1, m.ncb)) * 72);
        R.row_ptr = upload_new(A, rm.row_ptr, st);
        R.col_idx = upload_new(A, rm.col_idx, st);
        R.diag_pos = upload_new(A, rm.diag_pos, st);
        R.up_pos = upload_new(A, rm.up_pos, st);
        R.up_tpos = upload_new(A, rm.up_tpos, st);
        R.term_begin = upload_new(A, rm.term_begin, st);
        R.terms = upload_new(A, rm.terms, st);
        R.cb_col_idx = D.col_idx;
        R.blk_begin = upload_new(A, rm.blk_begin, st);
        R.blk_items = upload_new(A, rm.blk_items, st);
        {
            // segments of at most kRigSegTerms consecutive pose terms of one upper block
            std::vector<int> sb, ub(1, 0);
            for (int u = 0; u < R.nup; ++u) {
                for (int t = rm.term_begin[u]; t < rm.term_begin[u + 1]; t += kRigSegTerms) sb.push_back(t);
                ub.push_back(static_cast<int>(sb.size()));
            }
            sb.push_back(rm.term_begin.empty() ? 0 : rm.term_begin.back());
            R.nseg = static_cast<int>(sb.size()) - 1;
            R.seg_begin = upload_new(A, sb, st);
            R.up_seg_begin = upload_new(A, ub, st);
            R.seg_part = A.alloc<double>(static_cast<size_t>(std::max(1, R.nseg)) * 36);
            // segments of at most kRigItemSeg camera blocks of one rig block (border, rhs)
            std::vector<int> ib, bb(1, 0);
            for (int I = 0; I < rm.nrb; ++I) {
                for (int t = rm.blk_begin[I]; t < rm.blk_begin[I + 1]; t += kRigItemSeg) ib.push_back(t);
                bb.push_back(static_cast<int>(ib.size()));
            }
            ib.push_back(rm.blk_begin.empty() ? 0 : rm.blk_begin.back());
            R.nbseg = static_cast<int>(ib.size()) - 1;
            R.bseg_begin = upload_new(A, ib, st);
            R.blk_seg_begin = upload_new(A, bb, st);
            R.bpart = A.alloc<double>(static_cast<size_t>(std::max(1, R.nbseg)) * 6 *
                                      ((c->ext_on ? c->ext.nbx : S.nb) + 1));
        }
        const int nbw = c->ext_on ? c->ext.nbx : S.nb;
        const size_t nr6 = static_cast<size_t>(6) * rm.nrb;
        R.vals = A.alloc<double>(static_cast<size_t>(std::max(1, R.nnzb)) * 36);
        R.border = A.alloc<double>(std::max<size_t>(1, nr6 * nbw));
        R.border_t = A.alloc<double>(std::max<size_t>(1, nr6 * nbw));
        R.rhs = A.alloc<double>(nr6 + nbw + 1);
        R.xv = A.alloc<double>(static_cast<size_t>(6) * m.ncb + nbw + 1);
        R.step_r = A.alloc<double>(nr6 + nbw + 1);
        R.sq = A.alloc<double>(1);
        check(cudaMemsetAsync(R.step_r, 0, (nr6 + nbw + 1) * sizeof(double), st), "memset");
        PcgSystem<double>& sr = c->sysr;
        sr = c->ext_on ? c->sysx : sy;
        sr.ncb = rm.nrb;
        sr.nb = nbw;
        sr.row_ptr = R.row_ptr;
        sr.col_idx = R.col_idx;
        sr.diag_pos = R.diag_pos;
        sr.vals = R.vals;
        sr.border = R.border;
        sr.border_t = R.border_t;
        sr.Dinv = A.alloc<double>(static_cast<size_t>(std::max(1, rm.nrb)) * 36);
    }
    c->pcg_grid = pcg_grid_size<double>(S.ncb);
    c->S[0] = c->S[1] = S;
    c->D[0] = c->D[1] = D;
    // strict RMS before (input cameras, initial points)
    launch_strict_rms(S, D, D.cams_input, c->init_points_all, c->proc_of_track, 0, nt, c->rms_before_d, st);
    c->rms_before.assign(nt, 0.0);
    check(cudaMemcpyAsync(c->rms_before.data(), c->rms_before_d, nt * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "upload");
}

template <typename T>
PrecisionBuffers<T>& pbuf(pb_gpu_ctx* c);
template <>
PrecisionBuffers<double>& pbuf<double>(pb_gpu_ctx* c) { return c->p64; }
template <>
PrecisionBuffers<float>& pbuf<float>(pb_gpu_ctx* c) { return c->p32; }

template <typename T>
void prepare_precision(pb_gpu_ctx* c, int precision) {
    PrecisionBuffers<T>& B = pbuf<T>(c);
    if (B.ready) return;
    HostModel& m = c->model;
    std::string err;
    if (!m.chunks_ready[precision]) {
        const int rc = build_chunks(&m, precision, smem_budget(c->device), &err);
        if (rc) throw std::runtime_error(err);
    }
    const ChunkSet& cs = m.chunks[precision];
    DeviceArena& A = c->parena[precision];
    cudaStream_t st = c->stream;
    Shape& S = c->S[precision];
    DevPtrs& D = c->D[precision];
    S.nchunks = cs.n();
    S.max_obs = cs.max_obs;
    S.max_cams = cs.max_cams;
    S.max_pairs = cs.max_pairs;
    S.max_tracks = cs.max_tracks;
    D.ch_obs_begin = upload_new(A, cs.obs_begin, st);
    D.ch_cam_begin = upload_new(A, cs.cam_begin, st);
    D.ch_cams = upload_new(A, cs.cams, st);
    D.ch_pair_begin = upload_new(A, cs.pair_begin, st);
    D.ch_pairs = upload_new(A, cs.pairs, st);
    D.up_contrib_begin = upload_new(A, cs.up_contrib_begin, st);
    D.up_contrib = upload_new(A, cs.up_contrib, st);
    D.cam_contrib_begin = upload_new(A, cs.cam_contrib_begin, st);
    D.cam_contrib = upload_new(A, cs.cam_contrib, st);
    D.obs_lcam = upload_new(A, cs.obs_lcam, st);
    D.slot_item_begin = upload_new(A, cs.slot_item_begin, st);
    D.slot_items = upload_new(A, cs.slot_items, st);
    D.lcam_obs_begin = upload_new(A, cs.lcam_obs_begin, st);
    D.lcam_obs = upload_new(A, cs.lcam_obs, st);
    D.warp_task_begin = upload_new(A, cs.warp_task_begin, st);
    D.task_list = upload_new(A, cs.task_list, st);
    const int camrec = 12 + S.ng * 6 * S.ni, chrec = S.nb * S.nb + 2 * S.nb;
    // chunk partials: accumulator pairs of the assembly (float2 on the FP32 path, double on FP64)
    using PT = typename Acc<T>::part_type;
    B.out.part_pair_v = A.alloc<PT>(cs.n_pair_partials() * 36);
    B.out.part_cam_v = A.alloc<PT>(cs.n_cam_partials() * camrec);
    B.out.part_chunk_v = A.alloc<PT>(static_cast<size_t>(std::max(1, S.nchunks)) * std::max(1, chrec));
    B.out.part_cost = A.alloc<double>(std::max(1, S.nchunks));
    B.out.part_flags = A.alloc<int>(std::max(1, S.nchunks));
    B.out.trk_data_v = A.alloc<double>(static_cast<size_t>(S.ntp) * kTrackRec);
    B.out.obs_rec_v = A.alloc<T>(static_cast<size_t>(S.nop) * (2 * (6 + S.ni) + 6));
    c->pcg_part = nullptr;
    B.ready = true;
    check(cudaStreamSynchronize(st), "prepare");
}

void ensure_pcg_partials(pb_gpu_ctx* c) {
    if (c->pcg_part) return;
    c->pcg_part = c->arena.alloc<double>(static_cast<size_t>(2 * std::max(c->pcg_grid, 160)) * (2 + kMaxNB));
}

void set_assemble_smem(int precision, size_t bytes);
double extend_system(pb_gpu_ctx* c, double damping);

void record_history(pb_gpu_ctx* c, int iteration, double cost, std::chrono::steady_clock::time_point t0) {
    c->hist_it.push_back(iteration);
    c->hist_cost.push_back(cost);
    c->hist_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
}

// Accepts trial `slot` (step length alpha): cameras, groups, points and, for rigs, captures and
// sensors.
void accept_trial(pb_gpu_ctx* c, double alpha, int slot) {
    launch_accept(c->S[0], c->D[0], c->step_p, alpha, slot, c->stream);
    c->launches += 1;
    if (c->rig_on) {
        launch_rig_accept(c->rig, slot, c->stream);
        c->launches += 1;
    }
}

// Rigs: the chain maps at the current state and the rig system of the last assembly.
void rig_transform(pb_gpu_ctx* c, double damping) {
    const Shape& S = c->S[0];
    const int nbw = c->ext_on ? c->ext.nbx : S.nb;
    launch_rig_maps(c->rig, c->stream);
    launch_rig_transform(c->rig, c->red.vals, c->ext_on ? c->ext.border : c->red.border,
                         c->ext_on ? c->ext.rhs : c->red.rhs, nbw, damping, c->stream);
    c->launches += 5;
    check(cudaGetLastError(), "rig map launch");
}

// The solution of the solved system in camera-block numbering: the rig solution mapped back
// (and its squared sum kept for the step RMS), or the solution itself.
const double* camera_block_solution(pb_gpu_ctx* c, const double* x) {
    if (!c->rig_on) return x;
    const Shape& S = c->S[0];
    const int nbw = c->ext_on ? c->ext.nbx : S.nb;
    launch_rig_expand(c->rig, x, nbw, S.nb, c->stream);
    c->launches += 2;
    check(cudaGetLastError(), "rig expand launch");
    return c->rig.xv;
}

struct Timer {
    pb_gpu_ctx* c;
    int slot;
    Timer(pb_gpu_ctx* ctx, int s) : c(ctx), slot(s) {
        if (c->timing) cudaEventRecord(c->ev0, c->stream);
    }
    ~Timer() {
        if (!c->timing) return;
        cudaEventRecord(c->ev1, c->stream);
        cudaEventSynchronize(c->ev1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        c->kt[2 * slot] += ms;
        c->kt[2 * slot + 1] += 1;
    }
};

template <typename T>
void assemble(pb_gpu_ctx* c, double damping, int precision, double* cost, int* flags) {
    prepare_precision<T>(c, precision);
    PrecisionBuffers<T>& B = pbuf<T>(c);
    const Shape& S = c->S[precision];
    const DevPtrs& D = c->D[precision];
    const size_t smem = chunk_smem_bytes(precision, S.max_obs, S.max_tracks, S.ni, S.nb);
    set_assemble_smem(precision, smem);
    {
        Timer t(c, 0);
        launch_assemble<T>(S, D, B.out, damping, smem, c->stream);
        c->launches += S.nchunks > 0 ? 1 : 0;
    }
    {
        Timer t(c, 3);
        launch_reduce<T>(S, D, B.out, c->red, damping, c->stream);
        c->launches += 2;  // k_reduce_sums, k_finalize
    }
    check(cudaGetLastError(), "assemble launch");
    check(cudaMemcpyAsync(c->h_scratch, c->red.result, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "assemble");
    *cost = c->h_scratch[0];
    *flags = static_cast<int>(c->h_scratch[1]);
    c->last_precision = precision;
    c->have_system = true;
    // scale bars: every assembly extends the reduced system by the promoted points and adds the
    // bars' cost, so that every solve of this context sees the extended system
    if (c->ext_on && !(*flags & 6)) *cost += extend_system(c, damping);
    // rigs: the camera-block system onto the rig's pose blocks, damped there
    if (c->rig_on && !(*flags & 6)) rig_transform(c, damping);
}

// Reduced solve.  Returns 0 ok, 1 breakdown / not positive definite (retried by the LM driver
// with more damping, as the reference does for "breakdown" / "positive definite" failures,
// BundleAdjustPlaMatrix.cpp:34-40, :359-369).
template <typename T>
DenseWork<T>& dwork(pb_gpu_ctx* c);
template <>
DenseWork<float>& dwork<float>(pb_gpu_ctx* c) { return c->dw32; }
template <>
DenseWork<double>& dwork<double>(pb_gpu_ctx* c) { return c->dw64; }

template <typename T>
void ensure_dense(pb_gpu_ctx* c) {
    const int idx = std::is_same<T, float>::value ? 1 : 0;
    if (c->dense_ready[idx]) return;
    DenseWork<T>& W = dwork<T>(c);
    const Shape& S = c->S[0];
    DeviceArena& A = c->darena;
    // the system solved: the reduced one, its extension by promoted points (scale bars), or
    // either mapped onto the rig's pose blocks
    const int nbsol = c->ext_on ? c->ext.nbx : S.nb;
    const int npose = c->rig_on ? c->model.rig.nrb : S.ncb;
    const std::vector<int>& prow = c->rig_on ? c->model.rig.row_ptr : c->model.row_ptr;
    const int nsol = 6 * npose + nbsol;
    W.n = nsol;
    W.nt = std::max(1, (nsol + 63) / 64);
    W.np = W.nt * 64;
    W.nnzb = c->rig_on ? c->rig.nnzb : S.nnzb;
    W.A = A.alloc<T>(static_cast<size_t>(W.np) * W.np);
    W.X = A.alloc<T>(static_cast<size_t>(W.np) * W.np);
    W.Dinv = A.alloc<T>(static_cast<size_t>(W.nt) * 64 * 64);
    W.dscale = A.alloc<double>(W.n);
    W.status = A.alloc<int>(1);
    W.x = A.alloc<double>(W.n);
    W.r = A.alloc<double>(W.n);
    W.z = A.alloc<double>(W.n);
    W.p = A.alloc<double>(W.n);
    W.q = A.alloc<double>(W.n);
    {
        // SpMV work items of the CG: 32 pose blocks per item (the longest block row sets the
        // items per row), 256 entries of a border row per item
        int longest = 0;
        for (int r = 0; r < npose; ++r) longest = std::max(longest, prow[r + 1] - prow[r]);
        W.pose_seg = npose > 0 ? std::max(1, (longest + 31) / 32) : 0;
        W.border_seg = nbsol > 0 ? (nsol + 255) / 256 : 0;
        W.qpart = A.alloc<double>(std::max<size_t>(1, 6 * static_cast<size_t>(npose) * W.pose_seg +
                                                          static_cast<size_t>(nbsol) * W.border_seg));
    }
    W.w = A.alloc<double>(W.n);
    W.ut = A.alloc<T>(W.np);
    W.wt = A.alloc<T>(W.np);
    // the CG's triangular products read these vectors up to the padded size: padding stays zero
    check(cudaMemsetAsync(W.ut, 0, static_cast<size_t>(W.np) * sizeof(T), c->stream), "memset");
    check(cudaMemsetAsync(W.wt, 0, static_cast<size_t>(W.np) * sizeof(T), c->stream), "memset");
    // partials of the cooperative CG: 4 per block, at most 32 blocks per SM
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    W.part = A.alloc<double>(static_cast<size_t>(std::max(1, sms)) * 32 * 4);
    W.scal = A.alloc<double>(8);
    c->dense_ready[idx] = true;
}

constexpr int kMaxFactorAge = 10;     // LM solves one FP32 factor may precondition (at n <= 3000)
constexpr int kReuseIterations = 60;  // CG iterations allowed on a kept factor before refactoring

// A factorisation costs ~n^3 and a CG iteration ~n^2: at n = 3016 one factorisation costs about
// 95 CG iterations, at n = 18016 several hundred.  The age limit of a kept factor therefore grows
// with n (a size rule, not a timing rule, so that repeated solves stay identical); the cap on the
// CG iterations of a reuse still refactors as soon as the kept factor preconditions badly.
int max_factor_age(int n) { return std::max(kMaxFactorAge, n / 300); }

template <typename T>
int solve_dense(pb_gpu_ctx* c, double rel, double abs_tol, int max_it, bool* converged, int* iterations,
                double* relres) {
    ensure_dense<T>(c);
    DenseWork<T>& W = dwork<T>(c);
    const bool f32 = std::is_same<T, float>::value;
    const PcgSystem<double>& sys = c->rig_on ? c->sysr : (c->ext_on ? c->sysx : c->sys);
    const double* rhs = c->rig_on ? c->rig.rhs : (c->ext_on ? c->ext.rhs : c->red.rhs);
    // factor reuse across LM iterations: the mixed path's default; the FP64 path on request
    // (pb_solve_options.factor_reuse), which gives an FP64 arm with the mixed path's policy
    const bool reuse = f32 ? c->factor_reuse != 2 : c->factor_reuse == 1;
    int spent = 0;
    // the age limit follows the dimension of the system factored (the rig system for a rig problem)
    if (reuse && c->f32_age >= 0 && c->f32_age < max_factor_age(W.n) && !c->f32_stale) {
        // The reduced matrix changes little between LM iterations: the FP32 factor of an earlier
        // one still preconditions the CG on the current FP64 matrix.  A factorisation costs
        // about as much as a hundred CG iterations, so the kept factor is used until the CG
        // needs more than kReuseIterations on it.
        const int cap = std::min(max_it, std::max(kReuseIterations, 4 * c->f32_base_iters));
        const int rc = dense_pcg<T>(sys, W, rhs, rel, abs_tol, cap, iterations, relres, converged, c->h_scratch + 40,
                                    c->stream, &c->launches);
        if (rc < 0) throw CudaError(std::string("dense CG failed: ") + cudaGetErrorString(cudaGetLastError()));
        if (rc == 0 && *converged) {
            ++c->f32_age;
            check(cudaMemcpyAsync(c->step_c, camera_block_solution(c, W.x), c->S[0].n * sizeof(double),
                                  cudaMemcpyDeviceToDevice, c->stream),
                  "D2D");
            return 0;
        }
        spent = *iterations;
    }
    // FP32 factor of the Jacobi-scaled matrix with a small shift (FP32 rounding of a matrix of
    // condition ~1e9 is not positive definite unshifted); the CG that follows runs on the
    // FP64 matrix, so the shift only costs iterations.  It starts at the last shift that
    // factorised and grows tenfold on failure.  The FP64 factor starts unshifted.
    double shift = f32 ? c->shift32 : 0.0;
    int st = 0;
    static const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
    const auto tf0 = std::chrono::steady_clock::now();
    int attempts = 0;
    for (int attempt = 0; attempt < 6; ++attempt) {
        ++attempts;
        st = dense_factor<T>(sys, W, shift, c->stream, &c->launches);
        if (st < 0) throw CudaError(std::string("dense factorisation failed: ") + cudaGetErrorString(cudaGetLastError()));
        if (st == 0 || (st & 1)) break;
        shift = shift == 0.0 ? 1e-9 : shift * 10.0;
    }
    const auto tf1 = std::chrono::steady_clock::now();
    if (st) return 1;
    if (f32) c->shift32 = shift;
    const int rc = dense_pcg<T>(sys, W, rhs, rel, abs_tol, max_it, iterations, relres, converged, c->h_scratch + 40,
                                c->stream, &c->launches);
    if (trace)
        std::fprintf(stderr, "PB_GPU_TRACE dense n=%d factor_attempts=%d shift=%.1e factor_ms=%.3f cg_ms=%.3f cg_it=%d\n",
                     W.n, attempts, shift, std::chrono::duration<double, std::milli>(tf1 - tf0).count(),
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tf1).count(),
                     *iterations);
    if (rc < 0) throw CudaError(std::string("dense CG failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (reuse) {
        c->f32_age = rc == 0 ? 1 : -1;
        c->f32_base_iters = *iterations;
    }
    *iterations += spent;
    if (rc) return 1;
    check(cudaMemcpyAsync(c->step_c, camera_block_solution(c, W.x), c->S[0].n * sizeof(double),
                          cudaMemcpyDeviceToDevice, c->stream),
          "D2D");
    return 0;
}

int solve_block_jacobi(pb_gpu_ctx* c, double rel, double abs_tol, int max_it, bool* converged, int* iterations,
                       double* relres) {
    ensure_pcg_partials(c);
    cudaStream_t st = c->stream;
    check(cudaMemsetAsync(c->pre_status, 0, sizeof(int), st), "memset");
    pcg_precondition<double>(c->sys, c->pre_status, st);
    if (pcg_solve<double>(c->sys, c->red.rhs, c->pcg_x, c->pcg_work, c->pcg_part, c->pcg_res, abs_tol, rel, max_it,
                          c->pcg_grid, st))
        throw CudaError(std::string("PCG launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    c->launches += 2;
    PcgResult res{};
    int pre = 0;
    check(cudaMemcpyAsync(c->h_scratch, c->pre_status, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaMemcpyAsync(c->h_scratch + 1, c->pcg_res, sizeof(PcgResult), cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "pcg");
    std::memcpy(&pre, c->h_scratch, sizeof(int));
    std::memcpy(&res, c->h_scratch + 1, sizeof(PcgResult));
    if (pre || res.status) return 1;
    check(cudaMemcpyAsync(c->step_c, c->pcg_x, c->S[0].n * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
    *converged = res.converged != 0;
    *iterations = res.iterations;
    *relres = res.bnorm > 0 ? res.rnorm / res.bnorm : 0.0;
    return 0;
}

// Automatic choice of the reduced solver: the dense-factor preconditioned CG while the factor
// fits comfortably (FP32 factor and inverse: 2 n^2 x 4 B, 8.6 GB at n = 32768; the FP64 path's
// factor costs 2n^3/3 FP64 flops every iteration, so it stops at n = 16384), block-Jacobi PCG
// beyond.  Both solve to the same relative residual; the preconditioner only sets the iteration
// count (block-Jacobi needs thousands per LM iteration on a 3 000-camera block).
bool dense_solver_fits(int n, int precision) { return n <= (precision == PB_PRECISION_MIXED ? 32768 : 16384); }

int solve_reduced(pb_gpu_ctx* c, const pb_solve_options& op, bool* converged, int* iterations, double* relres,
                  int* sweeps) {
    // the reference's tolerances: 2e-10 on the online path, 1e-12 on the general path
    // (BundleAdjustPlaMatrix.cpp:321-330)
    const double rel = op.linear_relative_tolerance > 0 ? op.linear_relative_tolerance
                                                         : (op.general_path ? 1.0e-12 : 2.0e-10);
    const double abs_tol = op.linear_absolute_tolerance > 0 ? op.linear_absolute_tolerance : 1.0e-12;
    const int P = c->rig_on ? c->model.rig.P : c->model.P;
    const int max_it = op.max_linear_iterations > 0 ? op.max_linear_iterations : std::max(200, 30 * P);
    int solver = (op.linear_solver == 1 || op.linear_solver == 2)
                     ? op.linear_solver
                     : (dense_solver_fits(c->S[0].n, c->last_precision) ? 1 : 2);
    if (c->ext_on && !c->rig_on) {
        // the promoted points live in the dense border: the dense-factor CG solves the extension
        if (!dense_solver_fits(c->ext.nx, c->last_precision))
            throw std::runtime_error("scale bars need the dense reduced solver, and the reduced dimension exceeds its limit "
                                     "(32 768 mixed, 16 384 FP64)");
        solver = 1;
    }
    if (c->rig_on) {
        // the rig system (a few thousand unknowns: captures, sensors, groups, promoted points) is
        // solved by the dense-factor CG
        const int nr = 6 * c->model.rig.nrb + (c->ext_on ? c->ext.nbx : c->S[0].nb);
        if (!dense_solver_fits(nr, c->last_precision))
            throw std::runtime_error("rig problems need the dense reduced solver, and the rig system exceeds its limit "
                                     "(32 768 mixed, 16 384 FP64)");
        solver = 1;
    }
    c->last_solver = solver;
    *converged = false;
    *iterations = 0;
    *sweeps = 0;
    *relres = 0.0;
    Timer t(c, 1);
    int rc;
    if (solver == 2) {
        rc = solve_block_jacobi(c, rel, abs_tol, max_it, converged, iterations, relres);
    } else if (c->last_precision == PB_PRECISION_MIXED) {
        rc = solve_dense<float>(c, rel, abs_tol, max_it, converged, iterations, relres);
        *sweeps = *iterations;  // FP64-residual corrections of the FP32 factor
    } else {
        rc = solve_dense<double>(c, rel, abs_tol, max_it, converged, iterations, relres);
    }
    return rc;
}

void back_substitute(pb_gpu_ctx* c, double* dd, double* point_sq, double* cam_sq) {
    const int precision = c->last_precision;
    const Shape& S = c->S[precision];
    const DevPtrs& D = c->D[precision];
    if (precision == PB_PRECISION_FP64)
        launch_back_substitute<double>(S, D, static_cast<const double*>(c->p64.out.trk_data_v),
                                       static_cast<const double*>(c->p64.out.obs_rec_v), c->step_c, c->step_p,
                                       c->bs_terms, c->bs_part, c->direct64, c->bs_out, c->stream);
    else
        launch_back_substitute<float>(S, D, static_cast<const double*>(c->p32.out.trk_data_v),
                                      static_cast<const float*>(c->p32.out.obs_rec_v), c->step_c, c->step_p, c->bs_terms,
                                      c->bs_part, c->direct64, c->bs_out, c->stream);
    c->launches += 3;
    check(cudaGetLastError(), "back-substitution launch");
    check(cudaMemcpyAsync(c->h_scratch, c->bs_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (c->rig_on)
        check(cudaMemcpyAsync(c->h_scratch + 3, c->rig.sq, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "back-substitution");
    *dd = c->h_scratch[0];
    *point_sq = c->h_scratch[1];
    // the step RMS of a rig problem is taken over the rig's parameters, not the cameras'
    *cam_sq = c->rig_on ? c->h_scratch[3] : c->h_scratch[2];
}

void eval_costs(pb_gpu_ctx* c, const double* alphas, int n, int use_trial, double* out) {
    const Shape& S = c->S[0];
    const DevPtrs& D = c->D[0];
    if (use_trial) {
        std::memcpy(c->h_scratch + 16, alphas, n * sizeof(double));
        check(cudaMemcpyAsync(c->alphas_d, c->h_scratch + 16, n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "H2D");
    }
    {
        Timer t(c, 2);
        launch_cost(S, D, c->step_c, c->step_p, c->alphas_d, n, use_trial, c->cost_part, c->cost_out, c->stream,
                    c->rig_on ? &c->rig : nullptr);
        c->launches += use_trial ? (c->rig_on ? 4 : 3) : 2;
        if (c->ext_on) {
            launch_bar_cost(S, D, c->step_p, c->alphas_d, n, use_trial, c->bar_d + 1, c->stream);
            c->launches += 1;
        }
    }
    check(cudaGetLastError(), "cost launch");
    check(cudaMemcpyAsync(c->h_scratch, c->cost_out, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (c->ext_on)
        check(cudaMemcpyAsync(c->h_scratch + 8, c->bar_d + 1, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
              "D2H");
    check(cudaStreamSynchronize(c->stream), "cost");
    std::memcpy(out, c->h_scratch, n * sizeof(double));
    // the scale bars' robust cost (assembleScaleBars, BundleAdjustPlaMatrixAssemblySurvey.cpp:131-186)
    if (c->ext_on)
        for (int i = 0; i < n; ++i) out[i] += c->h_scratch[8 + i];
}

// Scale bars: the reduced system of the last assembly extended by the promoted points; returns
// the bars' cost at the current state.
double extend_system(pb_gpu_ctx* c, double damping) {
    const Shape& S = c->S[0];
    check(cudaMemsetAsync(c->ext_flags, 0, sizeof(int), c->stream), "memset");
    launch_extend_system(S, c->D[0], c->red, c->ext, damping, c->ext_flags, c->bar_d, c->stream);
    c->launches += S.npr > 0 ? 4 : 3;
    check(cudaGetLastError(), "extension launch");
    check(cudaMemcpyAsync(c->h_scratch, c->bar_d, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(c->h_scratch + 1, c->ext_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "extension");
    int flags = 0;
    std::memcpy(&flags, c->h_scratch + 1, sizeof(int));
    if (flags & 2) throw std::runtime_error("linearisation produced an invalid projection");
    return c->h_scratch[0];
}

// Scale bars: the promoted points' steps of the last extended solve into the point steps;
// returns their squared sum.
double promoted_steps(pb_gpu_ctx* c) {
    const double* xsol = c->rig_on ? c->rig.xv : (c->last_precision == PB_PRECISION_MIXED ? c->dw32.x : c->dw64.x);
    launch_ext_step(c->S[0], c->D[0], xsol, c->step_c, c->step_p, c->bar_d + kMaxAlpha + 1, c->stream);
    c->launches += 1;
    check(cudaGetLastError(), "promoted step launch");
    check(cudaMemcpyAsync(c->h_scratch, c->bar_d + kMaxAlpha + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "promoted steps");
    return c->h_scratch[0];
}

void reset_state(pb_gpu_ctx* c) {
    const HostModel& m = c->model;
    const DevPtrs& D = c->D[0];
    cudaStream_t st = c->stream;
    check(cudaMemcpyAsync(D.cams_state, D.cams_input, m.cams_in.size() * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
    check(cudaMemcpyAsync(D.groups, c->groups_init, static_cast<size_t>(std::max(1, m.ng)) * kGroupRec * sizeof(double),
                          cudaMemcpyDeviceToDevice, st),
          "D2D");
    check(cudaMemcpyAsync(D.points, D.points0, m.trk_order.size() * 3 * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
    if (c->rig_on) {
        check(cudaMemcpyAsync(c->rig.cap_state, c->rig.cap_input, m.rig.cap_in.size() * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "D2D");
        check(cudaMemcpyAsync(c->rig.sen_state, c->rig.sen_input, m.rig.sen_in.size() * sizeof(double),
                              cudaMemcpyDeviceToDevice, st),
              "D2D");
    }
    launch_effective(c->S[0], D, st);
    c->launches += 1;
    c->have_system = false;
}

void finalize_quality(pb_gpu_ctx* c, const pb_solve_options& op, pb_solve_report* rep) {
    const HostModel& m = c->model;
    const int nt = m.nt;
    cudaStream_t st = c->stream;
    // finalizeBundleAdjustResult (BundleAdjustQuality.cpp:403-502): strict RMS, filter threshold,
    // valid mask and means on the device; five numbers come back
    launch_strict_rms(c->S[0], c->D[0], c->D[0].cams_eff, c->init_points_all, c->proc_of_track, 1, nt, c->rms_after_d, st);
    launch_quality(nt, c->active_d, c->rms_before_d, c->rms_after_d, op.enable_point_filter, op.filter_max_reproj_error,
                   op.filter_sigma_factor, c->valid_d, c->quality_part, c->quality_out, st);
    c->launches += 4;
    check(cudaMemcpyAsync(c->h_scratch, c->quality_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "quality");
    c->quality_host_stale = true;
    const double thr = c->h_scratch[0], kept_d = c->h_scratch[2], sb = c->h_scratch[3], sa = c->h_scratch[4];
    const int kept = static_cast<int>(kept_d);
    rep->filter_threshold = thr;
    rep->optimized_tracks = kept;
    rep->mean_rms_before = kept ? sb / kept : kInfD;
    rep->mean_rms_after = kept ? sa / kept : kInfD;
    rep->valid_track_ratio = nt ? static_cast<double>(kept) / nt : 0.0;
    if (kept == 0 && (rep->status == PB_SOLVE_SUCCESS || rep->status == PB_SOLVE_NO_CONVERGENCE)) {
        rep->status = PB_SOLVE_NUMERICAL_FAILURE;
        rep->solution_usable = 0;
    }
}

// The valid mask and strict RMS after the last solve, fetched from the device on first use.
void fetch_quality(pb_gpu_ctx* c) {
    if (!c->quality_host_stale) return;
    const int nt = c->model.nt;
    c->valid.assign(nt, 0);
    c->rms_after.assign(nt, 0.0);
    check(cudaMemcpy(c->valid.data(), c->valid_d, nt * sizeof(signed char), cudaMemcpyDeviceToHost), "D2H");
    check(cudaMemcpy(c->rms_after.data(), c->rms_after_d, nt * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
    c->quality_host_stale = false;
}

int do_assemble(pb_gpu_ctx* c, double damping, int precision, double* cost, int* flags) {
    if (precision == PB_PRECISION_FP64) assemble<double>(c, damping, precision, cost, flags);
    else assemble<float>(c, damping, precision, cost, flags);
    return 0;
}

// The LM / Armijo driver (online branch of optimizePointsWithPlaMatrix).
void lm_solve(pb_gpu_ctx* c, const pb_solve_options& op, pb_solve_report* rep) {
    c->f32_age = -1;  // every solve starts from a fresh factor: repeated solves run identically
    c->f32_stale = false;
    c->factor_reuse = (op.factor_reuse >= 0 && op.factor_reuse <= 2) ? op.factor_reuse : 0;
    const auto t0 = std::chrono::steady_clock::now();
    const HostModel& m = c->model;
    std::memset(rep, 0, sizeof(*rep));
    for (double& v : c->kt) v = 0.0;
    c->launches = 0;
    c->hist_it.clear();
    c->hist_cost.clear();
    c->hist_ms.clear();
    rep->active_tracks = m.active_tracks;
    rep->observation_count = m.obs_count;
    rep->rejected_initial_tracks = m.rejected;
    rep->camera_blocks = m.rig.on ? m.rig.nrb : m.ncb;
    rep->rig_capture_blocks = m.rig.ncapb;
    rep->rig_sensor_blocks = m.rig.nsenb;
    rep->intrinsic_blocks = m.ng;
    rep->pattern_builds = c->pattern_builds;
    rep->pattern_reuses = c->pattern_reuses;
    if (!(op.robust_loss >= 0 && op.robust_loss <= 2 && std::isfinite(op.robust_loss_scale) && op.robust_loss_scale > 0)) {
        rep->status = PB_SOLVE_INVALID_INPUT;
        c->error = "invalid image robust loss";
        return;
    }
    const float2 ls = ff_pack(op.robust_loss_scale);
    for (int p = 0; p < 2; ++p) {
        c->S[p].loss = op.robust_loss;
        c->S[p].loss_scale = op.robust_loss_scale;
        c->S[p].loss_scale_hi = ls.x;
        c->S[p].loss_scale_lo = ls.y;
    }
    reset_state(c);
    if (m.obs_count == 0) {
        rep->status = PB_SOLVE_INVALID_INPUT;
        return;
    }
    const int precision = op.precision == PB_PRECISION_MIXED ? PB_PRECISION_MIXED : PB_PRECISION_FP64;
    // Opt-in per-iteration trace on stderr (PB_GPU_TRACE=1), one line per linear solve.
    const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
    double current = kNaN, damping = 0.0;
    int iterations = 0;
    bool converged = m.P == 0 && m.ntb == 0;
    bool failed = false, cancelled = false;
    const double n_global = static_cast<double>(6 * (m.rig.on ? m.rig.nrb : m.ncb) + m.ng * m.ni);
    const double n_point = 3.0 * m.ntb;
    auto t_asm = 0.0, t_lin = 0.0, t_bs = 0.0, t_obj = 0.0;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    // The mixed-path assembly computes no cost (its linearisation is float-float): the FP64 cost
    // of the state comes from the cost kernel, here for the initial state and afterwards from the
    // line search that accepted the state.
    const bool cost_from_assembly = precision != PB_PRECISION_MIXED;
    try {
        if (converged || !cost_from_assembly) {
            double cst;
            eval_costs(c, nullptr, 1, 0, &cst);
            current = cst;
            rep->initial_cost = current;
            record_history(c, 0, current, t0);
            if (converged) ++rep->objective_evaluations;
        }
        const int budget = std::max(1, op.max_iterations);
        bool terminate = false;
        while (iterations < budget && !converged && !terminate) {
            if (c->cancel) { cancelled = true; break; }
            bool relinearize = false;
            while (iterations < budget && !converged && !relinearize) {
                if (c->cancel) { cancelled = true; break; }
                double cost;
                int flags;
                auto ta = now();
                do_assemble(c, damping, precision, &cost, &flags);
                t_asm += ms(ta, now());
                if (flags & 4) throw std::runtime_error("assembly chunk table inconsistent (bounds check)");
                if (flags & 2) throw std::runtime_error("online Schur linearisation produced an invalid projection");
                ++rep->linearizations;
                ++rep->objective_evaluations;
                if (cost_from_assembly) {
                    current = cost;
                    if (rep->linearizations == 1) {
                        rep->initial_cost = current;
                        record_history(c, 0, current, t0);
                    }
                }
                if (flags & 1) {
                    ++iterations;
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                bool lconv = false;
                int lit = 0, sweeps = 0;
                double relres = 0.0;
                auto tl = now();
                const int lrc = solve_reduced(c, op, &lconv, &lit, &relres, &sweeps);
                t_lin += ms(tl, now());
                if (lrc) {
                    ++iterations;
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                rep->linear_iterations += lit;
                rep->refinement_sweeps += sweeps;
                ++iterations;
                if (!lconv) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                double dd, psq, csq;
                auto tb = now();
                back_substitute(c, &dd, &psq, &csq);
                t_bs += ms(tb, now());
                if (!std::isfinite(dd)) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                const double rg = n_global > 0 ? std::sqrt(csq / n_global) : 0.0;
                const double rp = n_point > 0 ? std::sqrt(psq / n_point) : 0.0;
                // Armijo: alpha_k = 2^-k, first k with cost <= f - c alpha dd and cost < f
                double cand = kInfD, alpha = 1.0;
                int accepted_slot = -1;
                double accepted_alpha = 1.0;
                int k0 = 0;
                auto tc = now();
                while (k0 < op.line_search_steps && accepted_slot < 0) {
                    const int nbatch = std::min(k0 == 0 ? 1 : kMaxAlpha, op.line_search_steps - k0);
                    double al[kMaxAlpha], costs[kMaxAlpha];
                    for (int i = 0; i < nbatch; ++i) al[i] = std::ldexp(1.0, -(k0 + i));
                    eval_costs(c, al, nbatch, 1, costs);
                    for (int i = 0; i < nbatch; ++i) {
                        ++rep->objective_evaluations;
                        cand = costs[i];
                        alpha = al[i];
                        const double limit = current - op.armijo_coefficient * alpha * dd;
                        if (std::isfinite(cand) && cand <= limit && cand < current) {
                            accepted_slot = i;
                            accepted_alpha = alpha;
                            break;
                        }
                    }
                    k0 += nbatch;
                }
                t_obj += ms(tc, now());
                if (trace)
                    std::fprintf(stderr,
                                 "PB_GPU_TRACE it=%d precision=%d cost=%.15e lambda=%.3e lin_it=%d sweeps=%d "
                                 "relres=%.3e dd=%.6e rms_global=%.3e rms_point=%.3e alpha=%.6g cand=%.15e "
                                 "accepted=%d\n",
                                 iterations, precision, current, damping, lit, sweeps, relres, dd, rg, rp,
                                 accepted_slot >= 0 ? accepted_alpha : alpha, cand, accepted_slot >= 0 ? 1 : 0);
                if (accepted_slot >= 0) {
                    accept_trial(c, accepted_alpha, accepted_slot);
                    // a large cost decrease means a large change of the reduced matrix: the next
                    // solve refactors instead of trying the kept FP32 factor first
                    c->f32_stale = current - cand > 1e-2 * current;
                    current = cand;
                    record_history(c, iterations, current, t0);
                    ++rep->accepted_steps;
                    damping /= 10.0;
                    converged = accepted_alpha * rg <= 1e-6 && accepted_alpha * rp <= 1e-6;
                    relinearize = !converged;
                } else {
                    ++rep->rejected_steps;
                    terminate = true;
                    relinearize = true;
                }
            }
        }
        check(cudaStreamSynchronize(c->stream), "solve");
    } catch (const CudaError&) {
        throw;
    } catch (const std::exception& e) {
        failed = true;
        c->error = e.what();
    }
    rep->iterations = iterations;
    rep->final_cost = current;
    rep->assembly_ms = t_asm;
    rep->linear_ms = t_lin;
    rep->back_substitution_ms = t_bs;
    rep->objective_ms = t_obj;
    if (cancelled) {
        reset_state(c);
        check(cudaStreamSynchronize(c->stream), "reset");
        rep->status = PB_SOLVE_CANCELLED;
        rep->solution_usable = 0;
    } else if (failed) {
        rep->status = PB_SOLVE_NUMERICAL_FAILURE;
        rep->solution_usable = 0;
    } else {
        rep->status = converged ? PB_SOLVE_SUCCESS : PB_SOLVE_NO_CONVERGENCE;
        rep->solution_usable = std::isfinite(current) ? 1 : 0;
        finalize_quality(c, op, rep);
    }
    rep->gpu_kernel_launches = c->launches;
    rep->total_ms = ms(t0, now());
    c->solved = 1;
}

// The general (non-online) branch of optimizePointsWithPlaMatrix (BundleAdjustPlaMatrix.cpp:
// 236-542 with use_reference_online_schur false).  The reference builds the undamped block normal
// equations once per linearisation and hands them, with the current damping, to
// solveDampedSchurComplement; a rejected step retries the same equations with ten times the
// damping.  Here the damped Schur complement of the equations at the current state is formed by
// the fused assembly kernel, which linearises and eliminates in one pass: for image and
// control-point terms the damped Schur complement of H (primary and point diagonals scaled by
// 1 + damping) is exactly what the online assembly computes with that damping, so a retry re-runs
// the kernel at the unchanged state.  The driver differs from the online branch in:
//   - relative linear tolerance 1e-12;
//   - a step whose RMS (global and point) is at most 1e-6 ends the solve before any line search;
//   - the directional decrease is the finite difference (f(x) - f(x + 1e-4 d)) / 1e-4 of the
//     objective along the step (0 when that trial is not lower);
//   - Armijo accepts at cost <= f - c alpha dd (cost < f alone when dd is 0); when no step length
//     passes, the last (smallest) trial is still accepted if it lowers the cost;
//   - a rejected step (or a linear solve short of its tolerance) multiplies the damping by ten and
//     solves again at the same state; a solver breakdown is a numerical failure of the solve.
void lm_solve_general(pb_gpu_ctx* c, const pb_solve_options& op, pb_solve_report* rep) {
    c->f32_age = -1;
    c->f32_stale = false;
    c->factor_reuse = (op.factor_reuse >= 0 && op.factor_reuse <= 2) ? op.factor_reuse : 0;
    const auto t0 = std::chrono::steady_clock::now();
    const HostModel& m = c->model;
    std::memset(rep, 0, sizeof(*rep));
    for (double& v : c->kt) v = 0.0;
    c->launches = 0;
    c->hist_it.clear();
    c->hist_cost.clear();
    c->hist_ms.clear();
    rep->active_tracks = m.active_tracks;
    rep->observation_count = m.obs_count;
    rep->rejected_initial_tracks = m.rejected;
    rep->camera_blocks = m.rig.on ? m.rig.nrb : m.ncb;
    rep->rig_capture_blocks = m.rig.ncapb;
    rep->rig_sensor_blocks = m.rig.nsenb;
    rep->promoted_point_blocks = m.npr;
    rep->general_path_used = 1;
    rep->intrinsic_blocks = m.ng;
    rep->pattern_builds = c->pattern_builds;
    rep->pattern_reuses = c->pattern_reuses;
    if (!(op.robust_loss >= 0 && op.robust_loss <= 2 && std::isfinite(op.robust_loss_scale) && op.robust_loss_scale > 0)) {
        rep->status = PB_SOLVE_INVALID_INPUT;
        c->error = "invalid image robust loss";
        return;
    }
    const float2 ls = ff_pack(op.robust_loss_scale);
    for (int p = 0; p < 2; ++p) {
        c->S[p].loss = op.robust_loss;
        c->S[p].loss_scale = op.robust_loss_scale;
        c->S[p].loss_scale_hi = ls.x;
        c->S[p].loss_scale_lo = ls.y;
    }
    reset_state(c);
    if (m.obs_count == 0) {
        rep->status = PB_SOLVE_INVALID_INPUT;
        return;
    }
    const int precision = op.precision == PB_PRECISION_MIXED ? PB_PRECISION_MIXED : PB_PRECISION_FP64;
    const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
    double current = kNaN, damping = 0.0;
    int iterations = 0;
    bool converged = m.P == 0 && m.ntb == 0 && m.npr == 0;
    bool failed = false, cancelled = false;
    const double n_global = static_cast<double>(6 * (m.rig.on ? m.rig.nrb : m.ncb) + m.ng * m.ni);
    const double n_point = 3.0 * (m.ntb + m.npr);
    auto t_asm = 0.0, t_lin = 0.0, t_bs = 0.0, t_obj = 0.0;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const bool cost_from_assembly = precision != PB_PRECISION_MIXED;
    try {
        if (converged || !cost_from_assembly) {
            double cst;
            eval_costs(c, nullptr, 1, 0, &cst);
            current = cst;
            rep->initial_cost = current;
            record_history(c, 0, current, t0);
            if (converged) ++rep->objective_evaluations;
        }
        const int budget = std::max(1, op.max_iterations);
        while (iterations < budget && !converged) {
            if (c->cancel) { cancelled = true; break; }
            // buildNormalEquations: one linearisation and objective evaluation per state
            ++rep->linearizations;
            ++rep->objective_evaluations;
            bool linearized = false;
            bool relinearize = false;
            while (iterations < budget && !converged && !relinearize) {
                if (c->cancel) { cancelled = true; break; }
                double cost;
                int flags;
                auto ta = now();
                do_assemble(c, damping, precision, &cost, &flags);
                t_asm += ms(ta, now());
                if (flags & 4) throw std::runtime_error("assembly chunk table inconsistent (bounds check)");
                if (flags & 2) throw std::runtime_error("linearisation produced an invalid projection");
                if (cost_from_assembly && !linearized) {
                    current = cost;
                    if (rep->linearizations == 1) {
                        rep->initial_cost = current;
                        record_history(c, 0, current, t0);
                    }
                }
                linearized = true;
                if (flags & 1) throw std::runtime_error("eliminated point block is not numerically SPD (positive definite)");
                bool lconv = false;
                int lit = 0, sweeps = 0;
                double relres = 0.0;
                auto tl = now();
                const int lrc = solve_reduced(c, op, &lconv, &lit, &relres, &sweeps);
                t_lin += ms(tl, now());
                if (lrc) throw std::runtime_error("reduced system is not numerically SPD (positive definite)");
                rep->linear_iterations += lit;
                rep->refinement_sweeps += sweeps;
                ++iterations;
                if (!lconv) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                double dd_bs, psq, csq;
                auto tb = now();
                back_substitute(c, &dd_bs, &psq, &csq);
                if (c->ext_on) psq += promoted_steps(c);
                t_bs += ms(tb, now());
                const double rg = n_global > 0 ? std::sqrt(csq / n_global) : 0.0;
                const double rp = n_point > 0 ? std::sqrt(psq / n_point) : 0.0;
                if (rg <= 1e-6 && rp <= 1e-6) {
                    converged = true;
                    continue;
                }
                auto tc = now();
                // directional decrease by a forward difference of the objective along the step;
                // the difference point and the first trial (alpha = 1) share one objective pass
                // (slot 0: the trial, slot 1: the difference point; each slot's sum is formed
                // on its own, so the costs are those of two separate passes)
                double dd = 0.0;
                double first_trial = kNaN;
                {
                    const double h = 1.0e-4;
                    double fd;
                    if (op.line_search_steps > 0) {
                        const double al2[2] = {1.0, h};
                        double c2[2];
                        eval_costs(c, al2, 2, 1, c2);
                        first_trial = c2[0];
                        fd = c2[1];
                    } else {
                        eval_costs(c, &h, 1, 1, &fd);
                    }
                    ++rep->objective_evaluations;
                    if (std::isfinite(fd) && fd < current) dd = (current - fd) / h;
                }
                double cand = kInfD, alpha = 1.0;
                int accepted_slot = -1;
                double accepted_alpha = 1.0;
                int last_slot = -1;
                int k0 = 0;
                while (k0 < op.line_search_steps && accepted_slot < 0) {
                    const int nbatch = std::min(k0 == 0 ? 1 : kMaxAlpha, op.line_search_steps - k0);
                    double al[kMaxAlpha], costs[kMaxAlpha];
                    for (int i = 0; i < nbatch; ++i) al[i] = std::ldexp(1.0, -(k0 + i));
                    if (k0 == 0) costs[0] = first_trial;  // evaluated with the difference point
                    else eval_costs(c, al, nbatch, 1, costs);
                    for (int i = 0; i < nbatch; ++i) {
                        ++rep->objective_evaluations;
                        cand = costs[i];
                        alpha = al[i];
                        last_slot = i;
                        const double limit = dd > 0.0 ? current - op.armijo_coefficient * alpha * dd : current;
                        if (std::isfinite(cand) && cand <= limit && cand < current) {
                            accepted_slot = i;
                            accepted_alpha = alpha;
                            break;
                        }
                    }
                    k0 += nbatch;
                }
                t_obj += ms(tc, now());
                // the last trial evaluated (the smallest step length) is accepted when it lowers
                // the cost even without the Armijo condition
                const bool accept = std::isfinite(cand) && cand < current;
                if (accept && accepted_slot < 0) {
                    accepted_slot = last_slot;
                    accepted_alpha = alpha;
                }
                if (trace)
                    std::fprintf(stderr,
                                 "PB_GPU_TRACE general it=%d precision=%d cost=%.15e lambda=%.3e lin_it=%d relres=%.3e "
                                 "dd=%.6e rms_global=%.3e rms_point=%.3e alpha=%.6g cand=%.15e accepted=%d\n",
                                 iterations, precision, current, damping, lit, relres, dd, rg, rp, accepted_alpha, cand,
                                 accept ? 1 : 0);
                if (accept) {
                    accept_trial(c, accepted_alpha, accepted_slot);
                    c->f32_stale = current - cand > 1e-2 * current;
                    current = cand;
                    record_history(c, iterations, current, t0);
                    ++rep->accepted_steps;
                    damping /= 10.0;
                    converged = accepted_alpha * rg <= 1e-6 && accepted_alpha * rp <= 1e-6;
                    relinearize = !converged;
                } else {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                }
            }
        }
        check(cudaStreamSynchronize(c->stream), "solve");
    } catch (const CudaError&) {
        throw;
    } catch (const std::exception& e) {
        failed = true;
        c->error = e.what();
    }
    rep->iterations = iterations;
    rep->final_cost = current;
    rep->assembly_ms = t_asm;
    rep->linear_ms = t_lin;
    rep->back_substitution_ms = t_bs;
    rep->objective_ms = t_obj;
    if (cancelled) {
        reset_state(c);
        check(cudaStreamSynchronize(c->stream), "reset");
        rep->status = PB_SOLVE_CANCELLED;
        rep->solution_usable = 0;
    } else if (failed) {
        rep->status = PB_SOLVE_NUMERICAL_FAILURE;
        rep->solution_usable = 0;
    } else {
        rep->status = converged ? PB_SOLVE_SUCCESS : PB_SOLVE_NO_CONVERGENCE;
        rep->solution_usable = std::isfinite(current) ? 1 : 0;
        finalize_quality(c, op, rep);
    }
    rep->gpu_kernel_launches = c->launches;
    rep->total_ms = ms(t0, now());
    c->solved = 1;
}

pb_status fail(pb_gpu_ctx* c, pb_status s, const std::string& msg) {
    if (c) c->error = msg;
    return s;
}

}  // namespace

// Shared-memory opt-in for the assembly kernel (dynamic shared memory above 48 KB).
namespace {
void set_assemble_smem(int precision, size_t bytes) {
    static size_t done[2] = {0, 0};
    if (done[precision] >= bytes) return;
    if (precision == PB_PRECISION_FP64) pb_set_assemble_smem_f64(bytes);
    else pb_set_assemble_smem_f32(bytes);
    done[precision] = bytes;
}
}  // namespace

extern "C" {

const char* pb_status_name(int32_t s) {
    switch (s) {
        case PB_OK: return "ok";
        case PB_ERR_INVALID_ARGUMENT: return "invalid_argument";
        case PB_ERR_CUDA: return "cuda_error";
        case PB_ERR_NO_CONVERGENCE: return "no_convergence";
        case PB_ERR_SINGULAR_BLOCK: return "singular_block";
        case PB_ERR_CANCELLED: return "cancelled";
        case PB_ERR_BOUNDS: return "bounds_check";
        case PB_ERR_TIMEOUT: return "timeout";
        case PB_ERR_UNSUPPORTED: return "unsupported";
        case PB_ERR_INVALID_PROJECTION: return "invalid_projection";
        case PB_ERR_STATE: return "bad_state";
        default: return "unknown";
    }
}

pb_status pb_gpu_create(int32_t device, pb_gpu_ctx** out) {
    if (!out) return PB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return PB_ERR_CUDA;
    auto* c = new (std::nothrow) pb_gpu_ctx();
    if (!c) return PB_ERR_CUDA;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&c->h_scratch, 64 * sizeof(double)) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return PB_ERR_CUDA;
    }
    *out = c;
    return PB_OK;
}

pb_status pb_gpu_destroy(pb_gpu_ctx* c) {
    if (!c) return PB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->arena.free_all();
    c->parena[0].free_all();
    c->parena[1].free_all();
    c->darena.free_all();
    c->aarena.free_all();
    c->sarena.free_all();
    schur_work_destroy(c->schur);
    if (c->h_scratch) cudaFreeHost(c->h_scratch);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PB_OK;
}

const char* pb_gpu_last_error(const pb_gpu_ctx* c) { return c ? c->error.c_str() : "null context"; }

pb_status pb_gpu_upload(pb_gpu_ctx* c, const pb_problem_desc* pr, const pb_solve_options* op) {
    if (!c || !pr || !op) return fail(c, PB_ERR_INVALID_ARGUMENT, "null argument");
    try {
        cudaSetDevice(c->device);
        HostModel m;
        std::string err;
        c->shift32 = 1e-7;
        c->f32_age = -1;
        // opt-in trace (PB_GPU_TRACE=1): host model and device upload times
        static const bool trace = std::getenv("PB_GPU_TRACE") != nullptr;
        const auto t_start = std::chrono::steady_clock::now();
        const int rc = build_host_model(pr, op, &m, &err);
        const auto t_model = std::chrono::steady_clock::now();
        if (rc) {
            c->uploaded = false;
            return fail(c, rc == PB_SOLVE_UNSUPPORTED ? PB_ERR_UNSUPPORTED : PB_ERR_INVALID_ARGUMENT, err);
        }
        const bool reuse = c->uploaded && m.structure_hash == c->structure_hash && c->model.no == m.no;
        if (reuse) {
            // same structure: keep pattern, chunks and launch shapes; refresh the numeric inputs
            m.chunks[0] = std::move(c->model.chunks[0]);
            m.chunks[1] = std::move(c->model.chunks[1]);
            m.chunks_ready[0] = c->model.chunks_ready[0];
            m.chunks_ready[1] = c->model.chunks_ready[1];
            const bool r64 = c->p64.ready, r32 = c->p32.ready;
            DevPtrs d0 = c->D[0], d1 = c->D[1];
            Shape s0 = c->S[0], s1 = c->S[1];
            c->model = std::move(m);
            c->arena.release();
            c->pcg_part = nullptr;
            upload_structure(c);
            // restore the chunk fields of the per-precision descriptors
            auto keep_chunks = [](DevPtrs& dst, const DevPtrs& src, Shape& sd, const Shape& ss) {
                dst.ch_obs_begin = src.ch_obs_begin; dst.ch_cam_begin = src.ch_cam_begin; dst.ch_cams = src.ch_cams;
                dst.ch_pair_begin = src.ch_pair_begin; dst.ch_pairs = src.ch_pairs;
                dst.up_contrib_begin = src.up_contrib_begin; dst.up_contrib = src.up_contrib;
                dst.cam_contrib_begin = src.cam_contrib_begin; dst.cam_contrib = src.cam_contrib; dst.obs_lcam = src.obs_lcam;
                dst.slot_item_begin = src.slot_item_begin; dst.slot_items = src.slot_items;
                dst.lcam_obs_begin = src.lcam_obs_begin; dst.lcam_obs = src.lcam_obs;
                dst.warp_task_begin = src.warp_task_begin; dst.task_list = src.task_list;
                sd.nchunks = ss.nchunks; sd.max_obs = ss.max_obs; sd.max_cams = ss.max_cams; sd.max_pairs = ss.max_pairs; sd.max_tracks = ss.max_tracks;
            };
            keep_chunks(c->D[0], d0, c->S[0], s0);
            keep_chunks(c->D[1], d1, c->S[1], s1);
            (void)r64;
            (void)r32;
            ++c->pattern_reuses;
        } else {
            c->arena.release();
            c->parena[0].release();
            c->parena[1].release();
            c->p64 = PrecisionBuffers<double>{};
            c->p32 = PrecisionBuffers<float>{};
            c->darena.release();
            c->dense_ready[0] = c->dense_ready[1] = false;
            c->pcg_part = nullptr;
            c->model = std::move(m);
            upload_structure(c);
            ++c->pattern_builds;
        }
        c->structure_hash = c->model.structure_hash;
        c->uploaded = true;
        c->have_system = false;
        c->aarena.release();
        c->adj_ready = false;
        c->sarena.release();
        c->snap_valid = false;
        c->proc_of_obs.clear();
        reset_state(c);
        check(cudaStreamSynchronize(c->stream), "upload");
        if (trace) {
            const auto t_end = std::chrono::steady_clock::now();
            std::fprintf(stderr, "PB_GPU_UPLOAD host_model_ms=%.2f device_upload_ms=%.2f reuse=%d\n",
                         std::chrono::duration<double, std::milli>(t_model - t_start).count(),
                         std::chrono::duration<double, std::milli>(t_end - t_model).count(),
                         c->pattern_reuses > 0 ? 1 : 0);
        }
        return PB_OK;
    } catch (const std::bad_alloc&) {
        c->uploaded = false;
        return fail(c, PB_ERR_CUDA, "device allocation failed");
    } catch (const std::exception& e) {
        c->uploaded = false;
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_reset_state(pb_gpu_ctx* c) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        reset_state(c);
        check(cudaStreamSynchronize(c->stream), "reset");
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_get_sizes(pb_gpu_ctx* c, int64_t* s, double* baseline) {
    if (!c || !s || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    const HostModel& m = c->model;
    // rig problems report the reference's numbering: rig pose blocks, rig pairs, rig dimension
    const bool rig = m.rig.on;
    s[0] = m.nc; s[1] = m.nt; s[2] = m.no; s[3] = rig ? m.rig.P : m.P; s[4] = rig ? m.rig.nrb : m.ncb; s[5] = m.ng;
    s[6] = m.ntb; s[7] = m.active_tracks; s[8] = m.obs_count; s[9] = m.rejected;
    s[10] = static_cast<int64_t>(rig ? m.rig.pairs.size() : m.pairs.size());
    s[11] = 6 * (rig ? m.rig.nrb : m.ncb) + m.ng * m.ni; s[12] = m.ni; s[13] = m.gauge_anchor; s[14] = m.gauge_scale;
    s[15] = m.chunks_ready[1] ? m.chunks[1].n() : (m.chunks_ready[0] ? m.chunks[0].n() : 0);
    if (baseline) *baseline = m.gauge_baseline;
    return PB_OK;
}

pb_status pb_gpu_get_active(pb_gpu_ctx* c, int8_t* at, int32_t* cb, int32_t* ib, int32_t* tb) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    const HostModel& m = c->model;
    for (int t = 0; t < m.nt; ++t) {
        if (at) at[t] = m.active_track[t];
        if (tb) tb[t] = m.track_block[t];
    }
    // rig problems: no camera has a block of its own (ActiveProblem::cameraBlock stays -1) and the
    // groups follow the rig blocks
    for (int i = 0; i < m.nc; ++i) {
        if (cb) cb[i] = m.rig.on ? -1 : m.camera_block[i];
        if (ib) ib[i] = (m.rig.on && m.intrinsic_block[i] >= 0) ? m.rig.nrb + m.calib_group[i] : m.intrinsic_block[i];
    }
    return PB_OK;
}

pb_status pb_gpu_get_pairs(pb_gpu_ctx* c, int32_t* pairs) {
    if (!c || !pairs || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    const auto& pl = c->model.rig.on ? c->model.rig.pairs : c->model.pairs;
    for (size_t i = 0; i < pl.size(); ++i) {
        pairs[2 * i] = pl[i].first;
        pairs[2 * i + 1] = pl[i].second;
    }
    return PB_OK;
}

pb_status pb_gpu_get_history(pb_gpu_ctx* c, int32_t capacity, int32_t* iterations, double* costs, double* ms,
                             int32_t* count) {
    if (!c || !count || capacity < 0) return fail(c, PB_ERR_INVALID_ARGUMENT, "invalid history request");
    const int n = static_cast<int>(c->hist_cost.size());
    *count = n;
    for (int i = 0; i < std::min(n, capacity); ++i) {
        if (iterations) iterations[i] = c->hist_it[i];
        if (costs) costs[i] = c->hist_cost[i];
        if (ms) ms[i] = c->hist_ms[i];
    }
    return PB_OK;
}

pb_status pb_gpu_get_rig(pb_gpu_ctx* c, double* captures, double* sensors, int32_t* capture_block,
                         int32_t* sensor_block) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    const RigModel& rm = c->model.rig;
    if (!rm.on || !c->rig_on) return fail(c, PB_ERR_STATE, "the uploaded problem has no rig");
    try {
        if (captures)
            check(cudaMemcpy(captures, c->rig.cap_state, rm.cap_in.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        if (sensors)
            check(cudaMemcpy(sensors, c->rig.sen_state, rm.sen_in.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        for (int k = 0; k < rm.ncap; ++k)
            if (capture_block) capture_block[k] = rm.capture_block.empty() ? -1 : rm.capture_block[k];
        for (int s = 0; s < rm.nsen; ++s)
            if (sensor_block) sensor_block[s] = rm.sensor_block.empty() ? -1 : rm.sensor_block[s];
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_linearize_observations(pb_gpu_ctx* c, int32_t precision, double* res, double* jp, double* jpose,
                                        double* ji, double* nw, double* cost, int8_t* valid) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        const HostModel& m = c->model;
        const size_t no = static_cast<size_t>(m.no);
        DeviceArena tmp;
        double* dres = tmp.alloc<double>(no * 2);
        double* djp = tmp.alloc<double>(no * 6);
        double* djpose = tmp.alloc<double>(no * 2 * kP);
        double* dji = tmp.alloc<double>(no * 2 * kP);
        double* dnw = tmp.alloc<double>(no);
        double* dcost = tmp.alloc<double>(no);
        signed char* dvalid = tmp.alloc<signed char>(no);
        cudaStream_t st = c->stream;
        check(cudaMemsetAsync(dres, 0, no * 2 * sizeof(double), st), "memset");
        check(cudaMemsetAsync(djp, 0, no * 6 * sizeof(double), st), "memset");
        check(cudaMemsetAsync(djpose, 0, no * 2 * kP * sizeof(double), st), "memset");
        check(cudaMemsetAsync(dji, 0, no * 2 * kP * sizeof(double), st), "memset");
        check(cudaMemsetAsync(dnw, 0, no * sizeof(double), st), "memset");
        check(cudaMemsetAsync(dcost, 0, no * sizeof(double), st), "memset");
        check(cudaMemsetAsync(dvalid, 0, no, st), "memset");
        if (precision == PB_PRECISION_MIXED)
            launch_linearize_export<float>(c->S[0], c->D[0], dres, djp, djpose, dji, dnw, dcost, dvalid, st);
        else
            launch_linearize_export<double>(c->S[0], c->D[0], dres, djp, djpose, dji, dnw, dcost, dvalid, st);
        check(cudaGetLastError(), "linearize launch");
        auto d2h = [&](void* h, const void* d, size_t bytes) {
            if (h) check(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st), "D2H");
        };
        d2h(res, dres, no * 2 * sizeof(double));
        d2h(jp, djp, no * 6 * sizeof(double));
        d2h(jpose, djpose, no * 2 * kP * sizeof(double));
        d2h(ji, dji, no * 2 * kP * sizeof(double));
        d2h(nw, dnw, no * sizeof(double));
        d2h(cost, dcost, no * sizeof(double));
        d2h(valid, dvalid, no);
        check(cudaStreamSynchronize(st), "linearize");
        tmp.free_all();
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_linearize_schur(pb_gpu_ctx* c, double lambda, int32_t precision, double* cost, int32_t* singular) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    if (!std::isfinite(lambda) || lambda < 0.0) return fail(c, PB_ERR_INVALID_ARGUMENT, "invalid damping");
    try {
        double cst;
        int flags;
        do_assemble(c, lambda, precision == PB_PRECISION_MIXED ? PB_PRECISION_MIXED : PB_PRECISION_FP64, &cst, &flags);
        if (precision == PB_PRECISION_MIXED) eval_costs(c, nullptr, 1, 0, &cst);  // no cost in the mixed assembly
        if (cost) *cost = cst;
        if (singular) *singular = flags & 1;
        if (flags & 2) return fail(c, PB_ERR_INVALID_PROJECTION, "invalid projection during linearisation");
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_get_reduced(pb_gpu_ctx* c, double* dense, double* rhs, double* direct) {
    if (!c || !c->uploaded || !c->have_system) return fail(c, PB_ERR_STATE, "no reduced system assembled");
    try {
        const HostModel& m = c->model;
        const Shape& S = c->S[0];
        // rig problems: the system over the rig's pose blocks (the one that is solved); its
        // direct right-hand side is not formed and `direct` is left unwritten
        const bool rig = c->rig_on;
        if (rig && c->ext_on) return fail(c, PB_ERR_UNSUPPORTED, "the dense copy of a rig system with scale bars is not provided");
        const int npose = rig ? m.rig.nrb : S.ncb;
        const int nnzb = rig ? c->rig.nnzb : S.nnzb;
        const std::vector<int>& row_ptr = rig ? m.rig.row_ptr : m.row_ptr;
        const std::vector<int>& col_idx = rig ? m.rig.col_idx : m.col_idx;
        const int nb = S.nb, n6 = 6 * npose, n = n6 + nb;
        const size_t ts = 8;
        std::vector<char> vals(static_cast<size_t>(std::max(1, nnzb)) * 36 * ts), border(static_cast<size_t>(std::max(1, npose)) * 6 * std::max(1, nb) * ts),
            Cm(static_cast<size_t>(std::max(1, nb * nb)) * ts), r(n * ts), d(n * ts);
        const void* src_vals = rig ? c->rig.vals : c->red.vals;
        const void* src_border = rig ? c->rig.border : c->red.border;
        const void* src_C = c->red.Cm;
        const void* src_r = rig ? c->rig.rhs : c->red.rhs;
        const void* src_d = c->red.direct;
        check(cudaMemcpy(vals.data(), src_vals, static_cast<size_t>(nnzb) * 36 * ts, cudaMemcpyDeviceToHost), "D2H");
        if (nb) {
            check(cudaMemcpy(border.data(), src_border, static_cast<size_t>(npose) * 6 * nb * ts, cudaMemcpyDeviceToHost), "D2H");
            check(cudaMemcpy(Cm.data(), src_C, static_cast<size_t>(nb) * nb * ts, cudaMemcpyDeviceToHost), "D2H");
        }
        check(cudaMemcpy(r.data(), src_r, n * ts, cudaMemcpyDeviceToHost), "D2H");
        if (!rig) check(cudaMemcpy(d.data(), src_d, n * ts, cudaMemcpyDeviceToHost), "D2H");
        auto get = [&](const std::vector<char>& v, size_t i) {
            return ts == 8 ? reinterpret_cast<const double*>(v.data())[i]
                           : static_cast<double>(reinterpret_cast<const float*>(v.data())[i]);
        };
        if (dense) {
            std::fill(dense, dense + static_cast<size_t>(n) * n, 0.0);
            for (int i = 0; i < npose; ++i)
                for (int p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
                    const int j = col_idx[p];
                    for (int a = 0; a < 6; ++a)
                        for (int b = 0; b < 6; ++b)
                            dense[static_cast<size_t>(6 * i + a) * n + 6 * j + b] = get(vals, static_cast<size_t>(p) * 36 + a * 6 + b);
                }
            for (int row = 0; row < n6; ++row)
                for (int col = 0; col < nb; ++col) {
                    const double v = get(border, static_cast<size_t>(row) * nb + col);
                    dense[static_cast<size_t>(row) * n + n6 + col] = v;
                    dense[static_cast<size_t>(n6 + col) * n + row] = v;
                }
            for (int a = 0; a < nb; ++a)
                for (int b = 0; b < nb; ++b) dense[static_cast<size_t>(n6 + a) * n + n6 + b] = get(Cm, static_cast<size_t>(a) * nb + b);
        }
        for (int i = 0; i < n; ++i) {
            if (rhs) rhs[i] = get(r, i);
            if (direct && !rig) direct[i] = get(d, i);
        }
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_solve_reduced(pb_gpu_ctx* c, double* step, int32_t* converged, int32_t* iterations, double* relres) {
    if (!c || !c->uploaded || !c->have_system) return fail(c, PB_ERR_STATE, "no reduced system assembled");
    try {
        pb_solve_options op{};
        op.refinement_sweeps = 3;
        bool cv = false;
        int it = 0, sw = 0;
        double rr = 0.0;
        const int rc = solve_reduced(c, op, &cv, &it, &rr, &sw);
        if (converged) *converged = cv ? 1 : 0;
        if (iterations) *iterations = it;
        if (relres) *relres = rr;
        // the solution of the system pb_gpu_get_reduced copies: for a rig problem the rig step
        // (6 per rig block, then the intrinsic columns), else the camera-block step
        if (step) {
            if (c->rig_on)
                check(cudaMemcpy(step, c->rig.step_r, (6 * c->model.rig.nrb + c->S[0].nb) * sizeof(double),
                                 cudaMemcpyDeviceToHost),
                      "D2H");
            else
                check(cudaMemcpy(step, c->step_c, c->S[0].n * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        }
        if (rc) return fail(c, PB_ERR_SINGULAR_BLOCK, "reduced system is not numerically SPD (positive definite)");
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_back_substitute(pb_gpu_ctx* c, double* elim, double* dd, int32_t* success) {
    if (!c || !c->uploaded || !c->have_system) return fail(c, PB_ERR_STATE, "no reduced system assembled");
    try {
        double d, ps, cs;
        back_substitute(c, &d, &ps, &cs);
        if (dd) *dd = d;
        if (success) *success = std::isfinite(d) ? 1 : 0;
        if (elim) {
            const HostModel& m = c->model;
            std::vector<double> sp(m.trk_order.size() * 3);
            check(cudaMemcpy(sp.data(), c->step_p, sp.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
            for (size_t p = 0; p < m.trk_order.size(); ++p) {
                const int tb = m.track_block[m.trk_order[p]];
                if (tb < 0) continue;
                for (int a = 0; a < 3; ++a) elim[static_cast<size_t>(tb) * 3 + a] = sp[p * 3 + a];
            }
        }
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_eval_cost(pb_gpu_ctx* c, double* cost) {
    if (!c || !c->uploaded || !cost) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        eval_costs(c, nullptr, 1, 0, cost);
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_eval_cost_batch(pb_gpu_ctx* c, const double* alphas, int32_t n, double* costs) {
    if (!c || !c->uploaded || !c->have_system) return fail(c, PB_ERR_STATE, "no step available");
    if (!alphas || !costs || n <= 0) return fail(c, PB_ERR_INVALID_ARGUMENT, "bad alpha batch");
    try {
        for (int k = 0; k < n; k += kMaxAlpha) eval_costs(c, alphas + k, std::min(kMaxAlpha, n - k), 1, costs + k);
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_apply_step(pb_gpu_ctx* c, double alpha) {
    if (!c || !c->uploaded || !c->have_system) return fail(c, PB_ERR_STATE, "no step available");
    try {
        double cst;
        eval_costs(c, &alpha, 1, 1, &cst);
        accept_trial(c, alpha, 0);
        check(cudaStreamSynchronize(c->stream), "apply");
        c->have_system = false;
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_solve(pb_gpu_ctx* c, const pb_solve_options* op, pb_solve_report* rep) {
    if (!c || !op || !rep) return fail(c, PB_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        cudaSetDevice(c->device);
        c->error.clear();
        // a problem with scale bars has no online path (canUseReferenceOnlineSchur,
        // BundleAdjustPlaMatrixReferenceSchur.cpp:667-673)
        if (op->general_path || c->model.force_general) lm_solve_general(c, *op, rep);
        else lm_solve(c, *op, rep);
        return PB_OK;
    } catch (const std::exception& e) {
        rep->status = PB_SOLVE_NUMERICAL_FAILURE;
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_download_state(pb_gpu_ctx* c, double* cams, double* pts, int8_t* valid, double* rb, double* ra,
                                double* intr) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        const HostModel& m = c->model;
        if (cams)
            check(cudaMemcpy(cams, c->D[0].cams_eff, m.cams_in.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
        if (pts) {
            std::vector<double> sp(m.trk_order.size() * 3);
            check(cudaMemcpy(sp.data(), c->D[0].points, sp.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
            std::copy(m.points_in.begin(), m.points_in.end(), pts);
            for (size_t p = 0; p < m.trk_order.size(); ++p)
                for (int a = 0; a < 3; ++a) pts[static_cast<size_t>(m.trk_order[p]) * 3 + a] = sp[p * 3 + a];
        }
        if (valid || ra) fetch_quality(c);
        for (int t = 0; t < m.nt; ++t) {
            if (valid) valid[t] = c->solved && static_cast<size_t>(t) < c->valid.size() ? c->valid[t] : 0;
            if (rb) rb[t] = static_cast<size_t>(t) < c->rms_before.size() ? c->rms_before[t] : kNaN;
            if (ra) ra[t] = static_cast<size_t>(t) < c->rms_after.size() ? c->rms_after[t] : kNaN;
        }
        if (intr && m.ng > 0) {
            std::vector<double> g(static_cast<size_t>(m.ng) * kGroupRec);
            check(cudaMemcpy(g.data(), c->D[0].groups, g.size() * sizeof(double), cudaMemcpyDeviceToHost), "D2H");
            for (int gi = 0; gi < m.ng; ++gi)
                for (int p = 0; p < kP; ++p) intr[gi * kP + p] = g[static_cast<size_t>(gi) * kGroupRec + p];
        }
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_solve_problem(pb_gpu_ctx* c, const pb_problem_desc* pr, const pb_solve_options* op,
                               pb_solve_report* rep, double* cams, double* pts, int8_t* valid, double* rb, double* ra) {
    pb_status s = pb_gpu_upload(c, pr, op);
    if (s != PB_OK) {
        if (rep) {
            std::memset(rep, 0, sizeof(*rep));
            rep->status = s == PB_ERR_UNSUPPORTED ? PB_SOLVE_UNSUPPORTED : PB_SOLVE_INVALID_INPUT;
        }
        return s;
    }
    s = pb_gpu_solve(c, op, rep);
    if (s != PB_OK) return s;
    return pb_gpu_download_state(c, cams, pts, valid, rb, ra, nullptr);
}

pb_status pb_gpu_request_cancel(pb_gpu_ctx* c, int32_t cancel) {
    if (!c) return PB_ERR_INVALID_ARGUMENT;
    c->cancel = cancel;
    return PB_OK;
}

pb_status pb_gpu_kernel_times(pb_gpu_ctx* c, double* out8) {
    if (!c || !out8) return PB_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 8; ++i) out8[i] = c->kt[i];
    return PB_OK;
}

pb_status pb_gpu_get_stream(pb_gpu_ctx* c, void** stream) {
    if (!c || !stream) return PB_ERR_INVALID_ARGUMENT;
    *stream = static_cast<void*>(c->stream);
    return PB_OK;
}

pb_status pb_gpu_set_timing(pb_gpu_ctx* c, int32_t enable) {
    if (!c) return PB_ERR_INVALID_ARGUMENT;
    c->timing = enable != 0;
    return PB_OK;
}


// ------------------------------------------------------------------ state snapshot, observations
pb_status pb_gpu_save_state(pb_gpu_ctx* c) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        const HostModel& m = c->model;
        const DevPtrs& D = c->D[0];
        const size_t nc = m.cams_in.size(), np = m.trk_order.size() * 3,
                     ng = static_cast<size_t>(std::max(1, m.ng)) * kGroupRec;
        if (!c->snap_cams) {
            c->snap_cams = c->sarena.alloc<double>(nc);
            c->snap_points = c->sarena.alloc<double>(np);
            c->snap_groups = c->sarena.alloc<double>(ng);
        }
        cudaStream_t st = c->stream;
        check(cudaMemcpyAsync(c->snap_cams, D.cams_state, nc * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        check(cudaMemcpyAsync(c->snap_points, D.points, np * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        check(cudaMemcpyAsync(c->snap_groups, D.groups, ng * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        if (c->rig_on) {
            check(cudaMemcpyAsync(c->rig.cap_saved, c->rig.cap_state, m.rig.cap_in.size() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, st),
                  "D2D");
            check(cudaMemcpyAsync(c->rig.sen_saved, c->rig.sen_state, m.rig.sen_in.size() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, st),
                  "D2D");
        }
        check(cudaStreamSynchronize(st), "save_state");
        c->snap_valid = true;
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_restore_state(pb_gpu_ctx* c) {
    if (!c || !c->uploaded || !c->snap_valid) return fail(c, PB_ERR_STATE, "no saved state for this problem");
    try {
        const HostModel& m = c->model;
        const DevPtrs& D = c->D[0];
        const size_t nc = m.cams_in.size(), np = m.trk_order.size() * 3,
                     ng = static_cast<size_t>(std::max(1, m.ng)) * kGroupRec;
        cudaStream_t st = c->stream;
        check(cudaMemcpyAsync(D.cams_state, c->snap_cams, nc * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        check(cudaMemcpyAsync(D.points, c->snap_points, np * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        check(cudaMemcpyAsync(D.groups, c->snap_groups, ng * sizeof(double), cudaMemcpyDeviceToDevice, st), "D2D");
        if (c->rig_on) {
            check(cudaMemcpyAsync(c->rig.cap_state, c->rig.cap_saved, m.rig.cap_in.size() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, st),
                  "D2D");
            check(cudaMemcpyAsync(c->rig.sen_state, c->rig.sen_saved, m.rig.sen_in.size() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, st),
                  "D2D");
        }
        launch_effective(c->S[0], D, st);
        ++c->launches;
        c->have_system = false;
        check(cudaStreamSynchronize(st), "restore_state");
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_set_observations(pb_gpu_ctx* c, int64_t n, const int64_t* index, const double* u, const double* v) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    if (n < 0 || (n > 0 && (!index || !u || !v))) return fail(c, PB_ERR_INVALID_ARGUMENT, "invalid observation update");
    try {
        HostModel& m = c->model;
        if (c->proc_of_obs.empty()) {
            c->proc_of_obs.assign(static_cast<size_t>(m.no), -1);
            for (size_t p = 0; p < m.p_obs_orig.size(); ++p) c->proc_of_obs[m.p_obs_orig[p]] = static_cast<long long>(p);
        }
        const DevPtrs& D = c->D[0];
        cudaStream_t st = c->stream;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t k = index[i];
            if (k < 0 || k >= m.no || !std::isfinite(u[i]) || !std::isfinite(v[i]))
                return fail(c, PB_ERR_INVALID_ARGUMENT, "observation index out of range or non-finite measurement");
        }
        for (int64_t i = 0; i < n; ++i) {
            const int64_t k = index[i];
            m.obs_u[k] = u[i];
            m.obs_v[k] = v[i];
            check(cudaMemcpyAsync(D.raw_u + k, &m.obs_u[k], sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
            check(cudaMemcpyAsync(D.raw_v + k, &m.obs_v[k], sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
            const long long p = c->proc_of_obs[k];
            if (p >= 0) {
                check(cudaMemcpyAsync(D.obs_u + p, &m.obs_u[k], sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
                check(cudaMemcpyAsync(D.obs_v + p, &m.obs_v[k], sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
            }
        }
        check(cudaStreamSynchronize(st), "set_observations");
        c->have_system = false;
        return PB_OK;
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

// ------------------------------------------------------------------ backward pass
}  // extern "C"

namespace {

// Exact-Hessian solve of the backward pass (newton == 0: H mu = dL/dz with dL/dz already in the
// adjoint input buffers) or of a Newton step of the objective (newton == 1: H mu = -grad F).
// Leaves mu in c->step_c (primary) and c->adj.mu_p (points), dL/d(u, v) and the cross terms in
// the adjoint buffers.  ms[0..2]: Hessian, solve and gradient phases.
pb_status adjoint_core(pb_gpu_ctx* c, int newton, pb_adjoint_report* rep, float* ms) {
    const HostModel& m = c->model;
    const int prec = c->adj_prec;
    const Shape& S = c->S[prec];
    const DevPtrs& D = c->D[prec];
    cudaStream_t st = c->stream;
    const int nc = m.nc, ntp = S.ntp;
    AdjBuffers& B = c->adj;
    B.newton = newton;
    cudaEvent_t ev[4];
    for (auto& e : ev) check(cudaEventCreate(&e), "event");
    struct EvGuard {
        cudaEvent_t* e;
        ~EvGuard() { for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]); }
    } guard{ev};
    check(cudaEventRecord(ev[0], st), "event");
    // exact Hessian at the current state, reduced over the points
    const int n = S.n;
    RedOut<double>& R = c->red;
    check(cudaMemsetAsync(B.grad_fixed_cam, 0, static_cast<size_t>(nc) * 6 * sizeof(double), st), "memset");
    check(cudaMemsetAsync(B.grad_fixed_pt, 0, static_cast<size_t>(std::max(1, ntp)) * 3 * sizeof(double), st), "memset");
    check(cudaMemsetAsync(B.gauge, 0, 4 * sizeof(double), st), "memset");
    check(cudaMemsetAsync(B.flags, 0, sizeof(int), st), "memset");
    check(cudaMemsetAsync(B.mu_p, 0, static_cast<size_t>(std::max(1, ntp)) * 3 * sizeof(double), st), "memset");
    launch_effective(S, D, st);
    launch_adjoint_hessian(S, D, B, st);
    launch_adjoint_schur(S, D, B, B.part, R, st);
    launch_adjoint_rhs(S, D, B, R, st);
    c->launches += 6;
    check(cudaGetLastError(), "adjoint launch");
    check(cudaEventRecord(ev[1], st), "event");
    int flags = 0;
    check(cudaMemcpyAsync(&flags, B.flags, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "adjoint hessian");
    c->have_system = false;  // the reduced buffers now hold the exact Hessian, not an LM system
    if (rep) rep->point_blocks_singular = flags & 1;
    if (flags & 2) return fail(c, PB_ERR_INVALID_PROJECTION, "an observation does not project at this state");
    if (flags & 4) return fail(c, PB_ERR_STATE, "reduced pattern does not cover an observation pair");
    if (flags & 1) return fail(c, PB_ERR_SINGULAR_BLOCK, "a point block of the exact Hessian is singular");
    // solve H mu = dL/dz on the reduced system with the forward path's solvers
    bool conv = false;
    int it = 0;
    double rr = 0.0;
    const double rel = 1e-13, abs_tol = 1e-300;
    const int max_it = std::max(400, 30 * m.P);
    int rc;
    c->f32_age = -1;
    if (!dense_solver_fits(n, c->last_precision)) {
        rc = solve_block_jacobi(c, rel, abs_tol, max_it, &conv, &it, &rr);
    } else if (c->last_precision == PB_PRECISION_MIXED) {
        rc = solve_dense<float>(c, rel, abs_tol, max_it, &conv, &it, &rr);
    } else {
        rc = solve_dense<double>(c, rel, abs_tol, max_it, &conv, &it, &rr);
    }
    c->f32_age = -1;  // the FP32 factor held now is the exact Hessian's, not an LM matrix's
    if (rep) {
        rep->linear_iterations = it;
        rep->relative_residual = rr;
    }
    if (rc) return fail(c, PB_ERR_SINGULAR_BLOCK, "the exact Hessian is not positive definite (not a minimum?)");
    check(cudaEventRecord(ev[2], st), "event");
    launch_adjoint_gradient(S, D, B, c->step_c, st);
    ++c->launches;
    check(cudaGetLastError(), "adjoint gradient launch");
    check(cudaEventRecord(ev[3], st), "event");
    cudaEventSynchronize(ev[3]);
    cudaEventElapsedTime(&ms[0], ev[0], ev[1]);
    cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
    cudaEventElapsedTime(&ms[2], ev[2], ev[3]);
    return PB_OK;
}

// Allocates the adjoint buffers for the chunk plan of the arithmetic path last used.
pb_status adjoint_prepare(pb_gpu_ctx* c) {
    const HostModel& m = c->model;
    // the exact Hessian is written for the Euler target rotation chart and the scaled point chart
    // of image-only problems; control points switch the solve to the plain parameterisation
    if (!m.ref_param)
        return fail(c, PB_ERR_UNSUPPORTED,
                    "the backward pass covers image-only problems (no control points, scale bars or rigs)");
    // the point elimination runs over the chunk plan of the arithmetic path last used
    const int prec = c->last_precision == PB_PRECISION_MIXED ? 1 : 0;
    if (prec == 1) prepare_precision<float>(c, prec);
    else prepare_precision<double>(c, prec);
    const Shape& S = c->S[prec];
    const DevPtrs& D = c->D[prec];
    cudaStream_t st = c->stream;
    const int nc = m.nc, ntp = S.ntp;
    const long long nop = S.nop;
    AdjBuffers& B = c->adj;
    if (c->adj_ready && c->adj_prec != prec) {
    c->aarena.release();
    c->adj_ready = false;
    }
    if (!c->adj_ready) {
    DeviceArena& A = c->aarena;
    B.lay = AdjLayout::make(S.ni);
    B.rec = A.alloc<double>(static_cast<size_t>(std::max<long long>(1, nop)) * B.lay.stride);
    B.vinv = A.alloc<double>(static_cast<size_t>(std::max(1, ntp)) * 9);
    B.gpt = A.alloc<double>(static_cast<size_t>(std::max(1, ntp)) * 3);
    B.gcam = A.alloc<double>(static_cast<size_t>(nc) * 6);
    B.gint = A.alloc<double>(static_cast<size_t>(std::max(1, m.ng)) * kP);
    B.mu_p = A.alloc<double>(static_cast<size_t>(std::max(1, ntp)) * 3);
    B.grad_obs = A.alloc<double>(static_cast<size_t>(std::max<long long>(1, nop)) * 2);
    B.grad_fixed_cam = A.alloc<double>(static_cast<size_t>(nc) * 6);
    B.grad_fixed_pt = A.alloc<double>(static_cast<size_t>(std::max(1, ntp)) * 3);
    B.gauge = A.alloc<double>(4);
    B.flags = A.alloc<int>(1);
    const ChunkSet& cs = m.chunks[prec];
    const int nch = std::max(1, S.nchunks);
    B.part.part_pair_v = A.alloc<double>(std::max<size_t>(1, cs.n_pair_partials()) * 36);
    B.part.part_cam_v = A.alloc<double>(std::max<size_t>(1, cs.n_cam_partials()) * (12 + S.ng * 6 * S.ni));
    B.part.part_chunk_v = A.alloc<double>(static_cast<size_t>(nch) * std::max(1, S.nb * S.nb + 2 * S.nb));
    B.part.part_cost = A.alloc<double>(nch);
    B.part.part_flags = A.alloc<int>(nch);
    check(cudaMemsetAsync(B.part.part_cost, 0, nch * sizeof(double), st), "memset");
    check(cudaMemsetAsync(B.part.part_flags, 0, nch * sizeof(int), st), "memset");
    if (adjoint_assemble_smem(S) > smem_budget(c->device))
        return fail(c, PB_ERR_UNSUPPORTED, "adjoint chunk does not fit in shared memory");
    c->adj_prec = prec;
    c->adj_ready = true;
    }
    return PB_OK;
}

}  // namespace

extern "C" {

pb_status pb_gpu_backward(pb_gpu_ctx* c, const double* grad_cameras, const double* grad_points,
                          const double* grad_intrinsics, double* grad_observations, double* grad_initial_cameras,
                          double* grad_initial_points, pb_adjoint_report* rep) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    if (rep) std::memset(rep, 0, sizeof(*rep));
    try {
        pb_status ps = adjoint_prepare(c);
        if (ps != PB_OK) return ps;
        const HostModel& m = c->model;
        const int prec = c->adj_prec;
        const Shape& S = c->S[prec];
        const DevPtrs& D = c->D[prec];
        cudaStream_t st = c->stream;
        const int nc = m.nc, ntp = S.ntp;
        const long long nop = S.nop;
        AdjBuffers& B = c->adj;
        // inputs: dL/d(final state) (processing order for points)
        std::vector<double> gcam(static_cast<size_t>(nc) * 6, 0.0), gpt(static_cast<size_t>(std::max(1, ntp)) * 3, 0.0),
            gint(static_cast<size_t>(std::max(1, m.ng)) * kP, 0.0);
        if (grad_cameras) std::copy(grad_cameras, grad_cameras + gcam.size(), gcam.begin());
        if (grad_points)
            for (int p = 0; p < ntp; ++p)
                for (int a = 0; a < 3; ++a) gpt[static_cast<size_t>(p) * 3 + a] = grad_points[static_cast<size_t>(m.trk_order[p]) * 3 + a];
        if (grad_intrinsics && m.ng > 0) std::copy(grad_intrinsics, grad_intrinsics + static_cast<size_t>(m.ng) * kP, gint.begin());
        for (double v : gcam)
            if (!std::isfinite(v)) return fail(c, PB_ERR_INVALID_ARGUMENT, "non-finite camera gradient");
        for (double v : gpt)
            if (!std::isfinite(v)) return fail(c, PB_ERR_INVALID_ARGUMENT, "non-finite point gradient");
        for (double v : gint)
            if (!std::isfinite(v)) return fail(c, PB_ERR_INVALID_ARGUMENT, "non-finite intrinsic gradient");
        check(cudaMemcpyAsync(B.gcam, gcam.data(), gcam.size() * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
        check(cudaMemcpyAsync(B.gpt, gpt.data(), gpt.size() * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
        check(cudaMemcpyAsync(B.gint, gint.data(), gint.size() * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
        const int launches0 = c->launches;
        float ms[3] = {0.f, 0.f, 0.f};
        ps = adjoint_core(c, 0, rep, ms);
        if (ps != PB_OK) return ps;
        int flags = 0;
        std::vector<double> gobs(static_cast<size_t>(std::max<long long>(1, nop)) * 2), gfc(static_cast<size_t>(nc) * 6),
            gfp(static_cast<size_t>(std::max(1, ntp)) * 3), gauge(4), cams(m.cams_in.size());
        check(cudaMemcpyAsync(gobs.data(), B.grad_obs, gobs.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(gfc.data(), B.grad_fixed_cam, gfc.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(gfp.data(), B.grad_fixed_pt, gfp.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(gauge.data(), B.gauge, 4 * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(cams.data(), D.cams_state, cams.size() * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(&flags, B.flags, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaStreamSynchronize(st), "adjoint gradient");
        if (flags & 2) return fail(c, PB_ERR_INVALID_PROJECTION, "an observation does not project at this state");
        if (grad_observations) {
            std::fill(grad_observations, grad_observations + static_cast<size_t>(m.no) * 2, 0.0);
            for (long long p = 0; p < nop; ++p) {
                const long long k = m.p_obs_orig[p];
                grad_observations[2 * k] = gobs[2 * p];
                grad_observations[2 * k + 1] = gobs[2 * p + 1];
            }
        }
        if (grad_initial_cameras) {
            // fixed cameras: final pose = initial pose (direct term) plus the cross terms
            std::fill(grad_initial_cameras, grad_initial_cameras + static_cast<size_t>(nc) * 6, 0.0);
            for (int cam = 0; cam < nc; ++cam)
                if (m.camera_block[cam] < 0)
                    for (int a = 0; a < 6; ++a)
                        grad_initial_cameras[cam * 6 + a] = gcam[static_cast<size_t>(cam) * 6 + a] + gfc[static_cast<size_t>(cam) * 6 + a];
            // gauge: the scale camera's centre is anchor + b n(t), b = |C_scale^0 - C_anchor^0|
            const int sc = m.gauge_scale, an = m.gauge_anchor;
            if (sc >= 0 && an >= 0 && m.gauge_baseline > 0.0 && m.camera_block[sc] >= 0) {
                double nv[3], e0[3], l = 0.0, l0 = 0.0;
                for (int i = 0; i < 3; ++i) {
                    nv[i] = cams[static_cast<size_t>(sc) * kCamStride + 9 + i] - cams[static_cast<size_t>(an) * kCamStride + 9 + i];
                    e0[i] = m.cams_in[static_cast<size_t>(sc) * kCamStride + 9 + i] - m.cams_in[static_cast<size_t>(an) * kCamStride + 9 + i];
                    l += nv[i] * nv[i];
                    l0 += e0[i] * e0[i];
                }
                l = std::sqrt(l);
                l0 = std::sqrt(l0);
                const double* gs = &gcam[static_cast<size_t>(sc) * 6 + 3];
                double db = gauge[3];
                for (int i = 0; i < 3; ++i) db += gs[i] * nv[i] / l;
                for (int i = 0; i < 3; ++i) {
                    const double u0 = e0[i] / l0;
                    grad_initial_cameras[an * 6 + 3 + i] += gauge[i] + gs[i] - db * u0;
                    grad_initial_cameras[sc * 6 + 3 + i] += db * u0;
                }
            }
        }
        if (grad_initial_points) {
            std::fill(grad_initial_points, grad_initial_points + static_cast<size_t>(m.nt) * 3, 0.0);
            for (int p = 0; p < ntp; ++p) {
                const int t = m.trk_order[p];
                if (m.track_block[t] >= 0) continue;
                for (int a = 0; a < 3; ++a)
                    grad_initial_points[static_cast<size_t>(t) * 3 + a] =
                        gfp[static_cast<size_t>(p) * 3 + a] + (grad_points ? grad_points[static_cast<size_t>(t) * 3 + a] : 0.0);
            }
        }
        if (rep) {
            rep->hessian_ms = ms[0];
            rep->solve_ms = ms[1];
            rep->gradient_ms = ms[2];
            rep->total_ms = static_cast<double>(ms[0]) + ms[1] + ms[2];
            rep->gpu_kernel_launches = c->launches - launches0;
            rep->status = PB_OK;
        }
        return PB_OK;
    } catch (const std::bad_alloc&) {
        return fail(c, PB_ERR_CUDA, "device allocation failed");
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_solve_damped_schur(pb_gpu_ctx* c, const pb_bne* eq, double damping, const pb_schur_options* options,
                                    double* primary_step, double* eliminated_step, pb_schur_report* report) {
    if (!c || !eq || !options || !report) return fail(c, PB_ERR_INVALID_ARGUMENT, "null argument");
    if (!(damping >= 0.0) || !std::isfinite(damping)) return fail(c, PB_ERR_INVALID_ARGUMENT, "invalid damping");
    if (options->preconditioner_cluster_size < 0 || options->preconditioner_cluster_size > 16)
        return fail(c, PB_ERR_INVALID_ARGUMENT, "preconditioner cluster size outside 1..16");
    try {
        cudaSetDevice(c->device);
        if (!c->schur) c->schur = schur_work_create();
        std::string err;
        const int st = schur_solve(c->schur, c->device, c->stream, eq, damping, *options, primary_step, eliminated_step,
                                   report, &err);
        if (st != PB_OK) return fail(c, static_cast<pb_status>(st), err);
        return PB_OK;
    } catch (const std::bad_alloc&) {
        return fail(c, PB_ERR_CUDA, "device allocation failed");
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

pb_status pb_gpu_newton_step(pb_gpu_ctx* c, double* step_max, double* gradient_norm) {
    if (!c || !c->uploaded) return fail(c, PB_ERR_STATE, "no problem uploaded");
    try {
        pb_status ps = adjoint_prepare(c);
        if (ps != PB_OK) return ps;
        const int prec = c->adj_prec;
        const Shape& S = c->S[prec];
        const DevPtrs& D = c->D[prec];
        cudaStream_t st = c->stream;
        AdjBuffers& B = c->adj;
        check(cudaMemsetAsync(B.gcam, 0, static_cast<size_t>(S.nc) * 6 * sizeof(double), st), "memset");
        check(cudaMemsetAsync(B.gint, 0, static_cast<size_t>(std::max(1, S.ng)) * kP * sizeof(double), st), "memset");
        float ms[3];
        ps = adjoint_core(c, 1, nullptr, ms);
        if (ps != PB_OK) return ps;
        // |reduced -grad F| before the step, then state (+) step (no line search: a polish of a
        // converged state)
        std::vector<double> g(static_cast<size_t>(std::max(1, S.n))), step(g.size());
        check(cudaMemcpyAsync(g.data(), c->red.rhs, S.n * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(step.data(), c->step_c, S.n * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaMemcpyAsync(c->step_p, B.mu_p, static_cast<size_t>(std::max(1, S.ntp)) * 3 * sizeof(double),
                              cudaMemcpyDeviceToDevice, st), "D2D");
        const double alpha = 1.0;
        double cst = 0.0;
        eval_costs(c, &alpha, 1, 1, &cst);
        launch_accept(S, D, c->step_p, alpha, 0, st);
        c->launches += 1;
        check(cudaStreamSynchronize(st), "newton step");
        c->have_system = false;
        double gn = 0.0, sm = 0.0;
        for (int i = 0; i < S.n; ++i) {
            gn += g[i] * g[i];
            sm = std::max(sm, std::fabs(step[i]));
        }
        if (gradient_norm) *gradient_norm = std::sqrt(gn);
        if (step_max) *step_max = sm;
        return PB_OK;
    } catch (const std::bad_alloc&) {
        return fail(c, PB_ERR_CUDA, "device allocation failed");
    } catch (const std::exception& e) {
        return fail(c, PB_ERR_CUDA, e.what());
    }
}

}  // extern "C"
