// pb_host.cpp -- host preparation of a bundle-adjustment problem for the GB300 kernels:
// validation, gauge, active-track gate and block numbering, intrinsic groups, the reduced
// pattern, the processing order and the per-CTA chunks of the assembly kernel.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>

#include "pb_internal.h"

namespace pb {

namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();

bool finite3(const double* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// Host threads for a loop of n independent items: one per hardware thread, at most 32, and at
// least 4096 items each.
// Cap on the planning threads of the calling thread (0: none), set by pb_gpu_solve_batch so that
// its concurrent workers share the host cores instead of each spawning a full set.
thread_local int g_host_thread_cap = 0;

int host_threads(long long n) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const long long by_size = std::max(1LL, n / 4096);
    long long t = std::min<long long>(std::min<unsigned>(hw, 32u), by_size);
    if (g_host_thread_cap > 0) t = std::min<long long>(t, g_host_thread_cap);
    return static_cast<int>(t);
}

// f(i, begin, end) over `nthreads` contiguous ranges of [0, n); thread i gets range i.
template <typename F>
void parallel_ranges(int n, int nthreads, F f) {
    if (nthreads <= 1) {
        f(0, 0, n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nthreads - 1);
    for (int i = 1; i < nthreads; ++i)
        pool.emplace_back([&, i] {
            f(i, static_cast<int>(static_cast<long long>(n) * i / nthreads),
              static_cast<int>(static_cast<long long>(n) * (i + 1) / nthreads));
        });
    f(0, 0, static_cast<int>(static_cast<long long>(n) / nthreads));
    for (auto& th : pool) th.join();
}

double sanitized_weight(double w) { return std::isfinite(w) && w > 0.0 ? w : 0.0; }
double sanitized_scale(double s) { return std::isfinite(s) && s > 0.0 ? s : 1.0; }

// Projection of a world point (BundleAdjustProjection.h:58-91): false when the point is not in
// front of the camera or the pixel is not finite.
bool project(const double* cam, const double* X, double* px) {
    const double d0 = X[0] - cam[9], d1 = X[1] - cam[10], d2 = X[2] - cam[11];
    const double xc = cam[0] * d0 + cam[3] * d1 + cam[6] * d2;
    const double yc = cam[1] * d0 + cam[4] * d1 + cam[7] * d2;
    const double zc = cam[2] * d0 + cam[5] * d1 + cam[8] * d2;
    const double fwd = cam[23] != 0.0 ? -zc : zc;
    if (!(fwd > 1e-9)) return false;
    const double x = xc / zc, y = yc / zc, r2 = x * x + y * y;
    const double radial = 1.0 + cam[16] * r2 + cam[17] * r2 * r2 + cam[18] * r2 * r2 * r2;
    const double xd = x * radial + cam[19] * 2.0 * x * y + cam[20] * (r2 + 2.0 * x * x);
    const double yd = y * radial + cam[19] * (r2 + 2.0 * y * y) + cam[20] * 2.0 * x * y;
    px[0] = (cam[21] < 0 ? -1.0 : 1.0) * cam[12] * xd + cam[14];
    px[1] = (cam[22] < 0 ? -1.0 : 1.0) * cam[13] * yd + cam[15];
    return std::isfinite(px[0]) && std::isfinite(px[1]);
}

}  // namespace

void set_host_thread_cap(int cap) { g_host_thread_cap = cap > 0 ? cap : 0; }

double finite_median(std::vector<double> v, double fallback) {
    v.erase(std::remove_if(v.begin(), v.end(), [](double a) { return !std::isfinite(a); }), v.end());
    if (v.empty()) return fallback;
    const size_t n = v.size(), h = n / 2;
    std::nth_element(v.begin(), v.begin() + h, v.end());
    const double upper = v[h];
    if (n % 2) return upper;
    const double lower = *std::max_element(v.begin(), v.begin() + h);
    return 0.5 * (lower + upper);
}

void camera_parameter_block(const double* cam, double* p) {
    // CameraState::parameterBlock (CameraState.cpp:164-185) for this camera model.
    std::fill(p, p + kP, 0.0);
    p[0] = cam[12];
    p[1] = (cam[12] > 0 && cam[13] > 0) ? std::log(cam[13] / cam[12]) : std::numeric_limits<double>::quiet_NaN();
    for (int i = 2; i < 9; ++i) p[i] = cam[12 + i];
}

// Lower Cholesky factor of a symmetric positive definite 3x3 matrix with the checks of the
// control-point uncertainty factorisation (control_point.cpp:34-85): finite, symmetric to
// 1e-10 max(1, max|a|), every pivot above 1e-12 max(1, max|a|).
bool cp_cholesky(const double* a, double* L) {
    double maximum = 0.0;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const double v = a[r * 3 + c], t = a[c * 3 + r];
            if (!std::isfinite(v) || !std::isfinite(t)) return false;
            maximum = std::max(maximum, std::max(std::fabs(v), std::fabs(t)));
            if (std::fabs(v - t) > 1.0e-10 * std::max(1.0, maximum)) return false;
        }
    const double threshold = std::max(1.0, maximum) * 1.0e-12;
    for (int i = 0; i < 9; ++i) L[i] = 0.0;
    for (int j = 0; j < 3; ++j) {
        double d = a[j * 3 + j];
        for (int k = 0; k < j; ++k) d -= L[j * 3 + k] * L[j * 3 + k];
        if (!(d > 0.0) || !std::isfinite(d)) return false;
        const double ljj = std::sqrt(d);
        L[j * 3 + j] = ljj;
        for (int i = j + 1; i < 3; ++i) {
            double v = a[i * 3 + j];
            for (int k = 0; k < j; ++k) v -= L[i * 3 + k] * L[j * 3 + k];
            L[i * 3 + j] = v / ljj;
        }
    }
    for (int j = 0; j < 3; ++j)
        if (!(L[j * 3 + j] * L[j * 3 + j] > threshold)) return false;
    return true;
}

// makeControlPointWhitening (control_point.cpp:91-158): isotropic sigma -> I / sigma;
// covariance C = L L^T -> L^-1; square-root information W (W^T W positive definite) -> W.
// data: point (3), sigma, weight, kind, matrix (9).
bool cp_whitening(const double* data, double* W) {
    const int kind = static_cast<int>(data[5]);
    const double* mat = data + 6;
    for (int i = 0; i < 9; ++i) W[i] = 0.0;
    if (kind == 0) {
        const double sigma = data[3];
        if (!std::isfinite(sigma) || sigma <= 0.0) return false;
        for (int a = 0; a < 3; ++a) W[a * 3 + a] = 1.0 / sigma;
        return true;
    }
    if (kind == 1) {
        double L[9];
        if (!cp_cholesky(mat, L)) return false;
        // inverse of the lower triangle
        for (int i = 0; i < 3; ++i) {
            W[i * 3 + i] = 1.0 / L[i * 3 + i];
            for (int j = 0; j < i; ++j) {
                double v = 0.0;
                for (int k = j; k < i; ++k) v -= L[i * 3 + k] * W[k * 3 + j];
                W[i * 3 + j] = v / L[i * 3 + i];
            }
        }
        return true;
    }
    if (kind == 2) {
        for (int i = 0; i < 9; ++i)
            if (!std::isfinite(mat[i])) return false;
        double info[9], L[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += mat[k * 3 + r] * mat[k * 3 + c];
                info[r * 3 + c] = v;
            }
        if (!cp_cholesky(info, L)) return false;
        for (int i = 0; i < 9; ++i) W[i] = mat[i];
        return true;
    }
    return false;
}

// validateControlPointConstraint (control_point.cpp:205-220)
bool cp_valid(const double* data, double* W) {
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(data[a])) return false;
    if (!std::isfinite(data[4]) || data[4] <= 0.0) return false;
    return cp_whitening(data, W);
}

namespace {

// A rotation stored row-major is usable when it is finite and orthonormal with determinant +1
// (to 1e-9 on every entry of R R^T - I and on det - 1).
bool rotation_ok(const double* R) {
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(R[i])) return false;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const double v = R[r * 3] * R[c * 3] + R[r * 3 + 1] * R[c * 3 + 1] + R[r * 3 + 2] * R[c * 3 + 2];
            if (std::fabs(v - (r == c ? 1.0 : 0.0)) > 1e-9) return false;
        }
    const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                       R[2] * (R[3] * R[7] - R[4] * R[6]);
    return std::fabs(det - 1.0) <= 1e-9;
}

// The rig topology of the problem: its records, the binding of every camera, and the composed
// camera poses R = R_rig R_sensor, C = C_rig + R_rig c_sensor written into the input cameras
// (composeRigCameras, called by runConcreteBackend, src/solver.cpp:282; the README's "Rig BA"
// states the composition).  The composition function lives in the camera library, which is not
// part of the reference tree; its checks are restated: every camera bound to an existing capture
// and sensor of the same rig, proper rotations, finite centres, and at least one fixed sensor in
// every rig that has a capture (it defines the rig body frame).
int load_rig(const pb_problem_desc* pr, HostModel* m, std::string* err) {
    RigModel& R = m->rig;
    R = RigModel{};
    if (pr->n_rig_captures < 0 || pr->n_rig_sensors < 0) { *err = "rig record counts must be non-negative"; return PB_SOLVE_INVALID_INPUT; }
    if (pr->n_rig_captures == 0) return 0;
    if (pr->n_rig_sensors <= 0 || !pr->rig_captures || !pr->rig_capture_info || !pr->rig_sensors ||
        !pr->rig_sensor_info || !pr->rig_camera_capture || !pr->rig_camera_sensor) {
        *err = "rig topology arrays missing";
        return PB_SOLVE_INVALID_INPUT;
    }
    R.on = true;
    R.ncap = pr->n_rig_captures;
    R.nsen = pr->n_rig_sensors;
    R.cap_in.assign(pr->rig_captures, pr->rig_captures + static_cast<size_t>(R.ncap) * 12);
    R.sen_in.assign(pr->rig_sensors, pr->rig_sensors + static_cast<size_t>(R.nsen) * 12);
    R.cap_info.assign(pr->rig_capture_info, pr->rig_capture_info + static_cast<size_t>(R.ncap) * 2);
    R.sen_info.assign(pr->rig_sensor_info, pr->rig_sensor_info + static_cast<size_t>(R.nsen) * 2);
    for (int k = 0; k < R.ncap; ++k)
        if (!rotation_ok(&R.cap_in[k * 12]) || !finite3(&R.cap_in[k * 12 + 9])) {
            *err = "rig capture " + std::to_string(k) + " has an invalid pose";
            return PB_SOLVE_INVALID_INPUT;
        }
    for (int s = 0; s < R.nsen; ++s)
        if (!rotation_ok(&R.sen_in[s * 12]) || !finite3(&R.sen_in[s * 12 + 9])) {
            *err = "rig sensor " + std::to_string(s) + " has an invalid extrinsic";
            return PB_SOLVE_INVALID_INPUT;
        }
    R.cam_capture.assign(pr->rig_camera_capture, pr->rig_camera_capture + m->nc);
    R.cam_sensor.assign(pr->rig_camera_sensor, pr->rig_camera_sensor + m->nc);
    for (int c = 0; c < m->nc; ++c) {
        const int k = R.cam_capture[c], s = R.cam_sensor[c];
        if (k < 0 || k >= R.ncap || s < 0 || s >= R.nsen) {
            *err = "camera " + std::to_string(c) + " has no rig binding";
            return PB_SOLVE_INVALID_INPUT;
        }
        if (pr->rig_capture_info[2 * k] != pr->rig_sensor_info[2 * s]) {
            *err = "camera " + std::to_string(c) + " binds a capture and a sensor of different rigs";
            return PB_SOLVE_INVALID_INPUT;
        }
    }
    for (int k = 0; k < R.ncap; ++k) {
        const int rig = pr->rig_capture_info[2 * k];
        bool fixed_sensor = false;
        for (int s = 0; s < R.nsen && !fixed_sensor; ++s)
            fixed_sensor = pr->rig_sensor_info[2 * s] == rig && pr->rig_sensor_info[2 * s + 1] != 0;
        if (!fixed_sensor) {
            *err = "rig " + std::to_string(rig) + " has no fixed sensor to define its body frame";
            return PB_SOLVE_INVALID_INPUT;
        }
    }
    for (int c = 0; c < m->nc; ++c) {
        const double* cp = &R.cap_in[static_cast<size_t>(R.cam_capture[c]) * 12];
        const double* sp = &R.sen_in[static_cast<size_t>(R.cam_sensor[c]) * 12];
        double* cam = &m->cams_in[static_cast<size_t>(c) * kCamStride];
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q)
                cam[r * 3 + q] = cp[r * 3] * sp[q] + cp[r * 3 + 1] * sp[3 + q] + cp[r * 3 + 2] * sp[6 + q];
        for (int r = 0; r < 3; ++r)
            cam[9 + r] = cp[9 + r] + cp[r * 3] * sp[9] + cp[r * 3 + 1] * sp[10] + cp[r * 3 + 2] * sp[11];
    }
    return 0;
}

// Rig problems: the reference's block pairs over the rig numbering (prepareOffDiagonalTopology,
// BundleAdjustPlaMatrixReferenceSchur.cpp:568-659: the capture, sensor and intrinsic blocks of an
// observation pairwise, and all blocks of the observations of an eliminated track), the CSR of the
// rig pose blocks, and the term lists that map the camera-block system onto it.  A camera block a
// (camera c) enters the rig system through its capture block with Mc and its sensor block with
// Ms, so rig block (I, J) = sum over camera-block CSR entries (a, b), I in chain(a), J in chain(b),
// of M_aI^T S_ab M_bJ.
void build_rig_pattern(HostModel* m, const std::vector<unsigned char>& use) {
    RigModel& R = m->rig;
    const int P = R.P, nrb = R.nrb, nc = m->nc;
    std::vector<int> intr(nc, -1), cb(nc, -1), sb(nc, -1);
    for (int c = 0; c < nc; ++c) {
        if (m->intrinsic_block[c] >= 0) intr[c] = nrb + m->calib_group[c];
        if (!R.capture_block.empty()) {
            cb[c] = R.capture_block[R.cam_capture[c]];
            sb[c] = R.sensor_block[R.cam_sensor[c]];
        }
    }
    // tracks split over host threads, each setting the pairs of its tracks in its own P x P
    // bitset; the bitsets are OR-ed and read out row-major (the sorted pair list)
    const size_t words = (static_cast<size_t>(P) * P + 63) / 64;
    const int nthreads = host_threads(m->no);
    std::vector<std::vector<unsigned long long>> bits(nthreads, std::vector<unsigned long long>(words, 0ull));
    parallel_ranges(m->nt, nthreads, [&](int i, int t0, int t1) {
        unsigned long long* mask = bits[i].data();
        auto connect = [&](int a, int b) {
            if (a < 0 || b < 0 || a == b) return;
            const size_t bit = static_cast<size_t>(std::min(a, b)) * P + std::max(a, b);
            mask[bit >> 6] |= 1ull << (bit & 63);
        };
        std::vector<int> tb;
        for (int t = t0; t < t1; ++t) {
            if (!m->active_track[t]) continue;
            tb.clear();
            for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k) {
                if (!use[k]) continue;
                const int c = m->obs_cam[k];
                const int ob[3] = {cb[c], sb[c], intr[c]};
                connect(ob[0], ob[1]);
                connect(ob[0], ob[2]);
                connect(ob[1], ob[2]);
                if (m->track_block[t] >= 0)
                    for (int v : ob)
                        if (v >= 0) tb.push_back(v);
            }
            if (m->track_block[t] < 0) continue;
            std::sort(tb.begin(), tb.end());
            tb.erase(std::unique(tb.begin(), tb.end()), tb.end());
            for (size_t l = 0; l < tb.size(); ++l)
                for (size_t r = l + 1; r < tb.size(); ++r) connect(tb[l], tb[r]);
        }
    });
    std::vector<unsigned long long>& all = bits[0];
    for (int i = 1; i < nthreads; ++i)
        for (size_t w = 0; w < words; ++w) all[w] |= bits[i][w];
    R.pairs.clear();
    for (int r = 0; r < P; ++r)
        for (int q = r + 1; q < P; ++q) {
            const size_t bit = static_cast<size_t>(r) * P + q;
            if ((all[bit >> 6] >> (bit & 63)) & 1ull) R.pairs.emplace_back(r, q);
        }
    // rig pose CSR: the pose-pose pairs plus the diagonal
    std::vector<std::vector<int>> rows(nrb);
    for (int i = 0; i < nrb; ++i) rows[i].push_back(i);
    for (const auto& pq : R.pairs)
        if (pq.second < nrb) {
            rows[pq.first].push_back(pq.second);
            rows[pq.second].push_back(pq.first);
        }
    R.row_ptr.assign(nrb + 1, 0);
    R.col_idx.clear();
    R.diag_pos.assign(nrb, -1);
    for (int i = 0; i < nrb; ++i) {
        std::sort(rows[i].begin(), rows[i].end());
        for (int c : rows[i]) {
            if (c == i) R.diag_pos[i] = static_cast<int>(R.col_idx.size());
            R.col_idx.push_back(c);
        }
        R.row_ptr[i + 1] = static_cast<int>(R.col_idx.size());
    }
    auto csr_pos = [&](int i, int j) {
        const int* b = R.col_idx.data() + R.row_ptr[i];
        const int* e = R.col_idx.data() + R.row_ptr[i + 1];
        const int* f = std::lower_bound(b, e, j);
        return (f != e && *f == j) ? static_cast<int>(f - R.col_idx.data()) : -1;
    };
    // upper rig blocks and their terms, in CSR order
    R.up_pos.clear();
    R.up_tpos.clear();
    std::vector<int> up_of(R.col_idx.size(), -1);
    for (int i = 0; i < nrb; ++i)
        for (int p = R.row_ptr[i]; p < R.row_ptr[i + 1]; ++p) {
            const int j = R.col_idx[p];
            if (j < i) continue;
            up_of[p] = static_cast<int>(R.up_pos.size());
            R.up_pos.push_back(p);
            R.up_tpos.push_back(j == i ? -1 : csr_pos(j, i));
        }
    const int nup = static_cast<int>(R.up_pos.size());
    std::vector<std::vector<int>> lists(nup);
    const int ncb = m->ncb;
    for (int a = 0; a < ncb; ++a) {
        const int ca[2] = {R.cb_cap_block[a], R.cb_sen_block[a]};
        for (int p = m->row_ptr[a]; p < m->row_ptr[a + 1]; ++p) {
            const int b = m->col_idx[p];
            const int cbk[2] = {R.cb_cap_block[b], R.cb_sen_block[b]};
            for (int sa = 0; sa < 2; ++sa)
                for (int sbk = 0; sbk < 2; ++sbk) {
                    const int I = ca[sa], J = cbk[sbk];
                    if (I < 0 || J < 0 || I > J) continue;
                    const int q = csr_pos(I, J);
                    // every pair of chained blocks is in the reference topology: a miss would be a
                    // planner bug, and the term is then dropped rather than written out of bounds
                    if (q < 0) continue;
                    lists[up_of[q]].push_back(p);
                    lists[up_of[q]].push_back(a << 2 | sa << 1 | sbk);
                }
        }
    }
    R.term_begin.assign(nup + 1, 0);
    R.terms.clear();
    for (int u = 0; u < nup; ++u) {
        R.terms.insert(R.terms.end(), lists[u].begin(), lists[u].end());
        R.term_begin[u + 1] = static_cast<int>(R.terms.size() / 2);
    }
    // camera blocks per rig block
    std::vector<std::vector<int>> per(nrb);
    for (int a = 0; a < ncb; ++a) {
        if (R.cb_cap_block[a] >= 0) per[R.cb_cap_block[a]].push_back(a << 1);
        if (R.cb_sen_block[a] >= 0) per[R.cb_sen_block[a]].push_back(a << 1 | 1);
    }
    R.blk_begin.assign(nrb + 1, 0);
    R.blk_items.clear();
    for (int i = 0; i < nrb; ++i) {
        R.blk_items.insert(R.blk_items.end(), per[i].begin(), per[i].end());
        R.blk_begin[i + 1] = static_cast<int>(R.blk_items.size());
    }
}

}  // namespace

int build_host_model(const pb_problem_desc* pr, const pb_solve_options* op, HostModel* m, std::string* err) {
    if (!pr || !op) { *err = "null problem or options"; return PB_SOLVE_INVALID_INPUT; }
    if (pr->n_cameras <= 0 || pr->n_tracks <= 0 || !pr->cameras || !pr->track_offsets || !pr->points) {
        *err = "cameras or tracks are empty";
        return PB_SOLVE_INVALID_INPUT;
    }
    m->nc = pr->n_cameras;
    m->nt = pr->n_tracks;
    m->no = pr->n_obs;
    m->cams_in.assign(pr->cameras, pr->cameras + static_cast<size_t>(m->nc) * kCamStride);
    m->cams_ref = pr->intrinsic_reference_cameras
                      ? std::vector<double>(pr->intrinsic_reference_cameras,
                                            pr->intrinsic_reference_cameras + static_cast<size_t>(m->nc) * kCamStride)
                      : m->cams_in;
    m->points_in.assign(pr->points, pr->points + static_cast<size_t>(m->nt) * 3);
    m->offs.assign(pr->track_offsets, pr->track_offsets + m->nt + 1);
    if (m->offs[0] != 0 || m->offs[m->nt] != m->no) { *err = "track offsets do not cover the observations"; return PB_SOLVE_INVALID_INPUT; }
    for (int t = 0; t < m->nt; ++t)
        if (m->offs[t + 1] < m->offs[t]) { *err = "track offsets must be non-decreasing"; return PB_SOLVE_INVALID_INPUT; }
    if (m->no > 0 && (!pr->obs_camera || !pr->obs_u || !pr->obs_v || !pr->obs_weight || !pr->obs_scale)) {
        *err = "observation arrays missing";
        return PB_SOLVE_INVALID_INPUT;
    }
    // the observation arrays, copied by host threads over ranges
    {
        const size_t no = static_cast<size_t>(m->no);
        m->obs_cam.resize(no);
        m->obs_u.resize(no);
        m->obs_v.resize(no);
        m->obs_weight.resize(no);
        m->obs_scale.resize(no);
        const int n = static_cast<int>(std::min<long long>(m->no, std::numeric_limits<int>::max()));
        if (static_cast<long long>(n) == m->no) {
            parallel_ranges(n, host_threads(m->no), [&](int, int k0, int k1) {
                const size_t b = static_cast<size_t>(k0), c = static_cast<size_t>(k1 - k0);
                std::copy_n(pr->obs_camera + b, c, m->obs_cam.data() + b);
                std::copy_n(pr->obs_u + b, c, m->obs_u.data() + b);
                std::copy_n(pr->obs_v + b, c, m->obs_v.data() + b);
                std::copy_n(pr->obs_weight + b, c, m->obs_weight.data() + b);
                std::copy_n(pr->obs_scale + b, c, m->obs_scale.data() + b);
            });
        } else {
            std::copy_n(pr->obs_camera, no, m->obs_cam.data());
            std::copy_n(pr->obs_u, no, m->obs_u.data());
            std::copy_n(pr->obs_v, no, m->obs_v.data());
            std::copy_n(pr->obs_weight, no, m->obs_weight.data());
            std::copy_n(pr->obs_scale, no, m->obs_scale.data());
        }
    }
    m->fixed_cams.assign(pr->fixed_cameras, pr->fixed_cameras + pr->n_fixed_cameras);
    m->fixed_tracks.assign(pr->fixed_tracks, pr->fixed_tracks + pr->n_fixed_tracks);
    m->group_ids = pr->calibration_group_ids
                       ? std::vector<int>(pr->calibration_group_ids, pr->calibration_group_ids + m->nc)
                       : std::vector<int>();
    // --- rig topology: composed camera poses; without explicit calibration groups the cameras of
    // one sensor share one intrinsic block (makeSolverOptions, Conversion.cpp:83-98); a camera
    // whose capture pose and sensor extrinsic are both fixed is a fixed camera (:120-142)
    {
        const int rc = load_rig(pr, m, err);
        if (rc) return rc;
        const RigModel& R = m->rig;
        if (R.on) {
            if (m->group_ids.empty()) m->group_ids = R.cam_sensor;
            for (int c = 0; c < m->nc; ++c)
                if (R.cap_info[2 * R.cam_capture[c] + 1] && R.sen_info[2 * R.cam_sensor[c] + 1] &&
                    std::find(m->fixed_cams.begin(), m->fixed_cams.end(), c) == m->fixed_cams.end())
                    m->fixed_cams.push_back(c);
        }
    }
    for (int c = 0; c < m->nc; ++c) {
        const double* cam = &m->cams_in[static_cast<size_t>(c) * kCamStride];
        for (int i = 0; i < 21; ++i)
            if (!std::isfinite(cam[i])) { *err = "camera state must be finite"; return PB_SOLVE_INVALID_INPUT; }
        if (cam[12] <= 0.0 || cam[13] <= 0.0) { *err = "camera focal lengths must be positive"; return PB_SOLVE_INVALID_INPUT; }
        if (cam[24] < 0.0 || cam[25] < 0.0) { *err = "camera image size must be non-negative"; return PB_SOLVE_INVALID_INPUT; }
    }
    if (op->robust_loss < 0 || op->robust_loss > 2 || !std::isfinite(op->robust_loss_scale) ||
        op->robust_loss_scale <= 0.0) {
        *err = "image robust loss must be LeastSquares, Huber or Cauchy with a finite positive scale";
        return PB_SOLVE_INVALID_INPUT;
    }
    m->loss = op->robust_loss;
    m->loss_scale = op->robust_loss_scale;
    // BackendOptions::plaMatrixPreconditionerClusterSize (validateOptions: 1..16) selects how the
    // reference's block-Jacobi PCG groups blocks.  It changes the iteration count, not the solution
    // (the CG runs to the same relative residual): the dense-factor preconditioner here subsumes
    // any grouping, and the block-Jacobi PCG used beyond its size limit keeps single blocks.
    if (op->preconditioner_cluster_size < 1 || op->preconditioner_cluster_size > 16) {
        *err = "preconditioner cluster size must lie in [1, 16]";
        return PB_SOLVE_INVALID_INPUT;
    }

    // --- control points (Track::controlPointConstraints): any constraint switches the problem to
    // the plain parameterisation (enableControlPointConstraints, Conversion.cpp:106;
    // useReferencePointParameterization, BundleAdjustPlaMatrixAssembly.cpp:24-30); a constraint
    // whose weight is not positive does not linearise and is skipped (linearizeControlPoint,
    // BundleAdjustPlaMatrixConstraints.cpp:90-116)
    m->cp_track.clear();
    m->cp_rec.clear();
    // a rig selects the plain parameterisation (useReferencePointParameterization,
    // BundleAdjustPlaMatrixAssembly.cpp:24-30)
    m->ref_param = pr->n_control_points <= 0 && !m->rig.on;
    m->cp_huber = op->control_point_huber_delta;
    std::vector<double> cp_points;  // valid targets of tracks with usable observations
    std::vector<char> cp_usable_track;
    if (pr->n_control_points > 0) {
        if (!pr->control_point_track || !pr->control_point_data) { *err = "control-point arrays missing"; return PB_SOLVE_INVALID_INPUT; }
        if (!std::isfinite(op->control_point_weight) || op->control_point_weight < 0.0 ||
            !std::isfinite(op->control_point_huber_delta) || op->control_point_huber_delta <= 0.0) {
            *err = "control-point weight must be finite and non-negative and its Huber delta finite and positive";
            return PB_SOLVE_INVALID_INPUT;
        }
        // hasUsableTrackObservations (BundleAdjustValidation.cpp:94-106): two distinct cameras
        cp_usable_track.assign(m->nt, 0);
        for (int t = 0; t < m->nt; ++t) {
            int first = -1;
            for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k) {
                const int c = m->obs_cam[k];
                if (c < 0 || !std::isfinite(m->obs_u[k]) || !std::isfinite(m->obs_v[k]) || !std::isfinite(m->obs_weight[k]) ||
                    !(m->obs_weight[k] > 0.0))
                    continue;
                if (first < 0) first = c;
                else if (c != first) { cp_usable_track[t] = 1; break; }
            }
        }
        for (int i = 0; i < pr->n_control_points; ++i) {
            const int t = pr->control_point_track[i];
            if (t < 0 || t >= m->nt) { *err = "control-point track index out of range"; return PB_SOLVE_INVALID_INPUT; }
            const double* d = pr->control_point_data + static_cast<size_t>(i) * 15;
            // validateProblem rejects the whole problem (problem.cpp:253-260)
            double W[9];
            if (!cp_valid(d, W)) { *err = "track contains an invalid control-point constraint"; return PB_SOLVE_INVALID_INPUT; }
            if (cp_usable_track[t]) cp_points.insert(cp_points.end(), d, d + 3);
            const double wgt = op->control_point_weight * d[4];
            if (!(wgt > 0.0)) continue;
            const double sw = std::sqrt(wgt);
            m->cp_track.push_back(t);
            for (int k = 0; k < 9; ++k) m->cp_rec.push_back(sw * W[k]);
            m->cp_rec.insert(m->cp_rec.end(), d, d + 3);
        }
    }
    // --- scale bars (Problem::scaleBarConstraints): validateProblem rejects an invalid bar
    // (problem.cpp:342-355); any bar gives the problem an absolute scale (hasUsableScaleBar,
    // BundleAdjustValidation.cpp:242-259), switches to the plain parameterisation and to the
    // general path (useReferencePointParameterization, BundleAdjustPlaMatrixAssembly.cpp:24-30;
    // canUseReferenceOnlineSchur, BundleAdjustPlaMatrixReferenceSchur.cpp:667-673)
    m->bar_tracks.clear();
    m->bar_data.clear();
    m->bar_weight = op->scale_bar_weight;
    m->bar_huber = op->scale_bar_huber_delta;
    m->force_general = false;
    if (pr->n_scale_bars < 0) { *err = "scale-bar count must be non-negative"; return PB_SOLVE_INVALID_INPUT; }
    if (pr->n_scale_bars > 0) {
        if (!pr->scale_bar_tracks || !pr->scale_bar_data) { *err = "scale-bar arrays missing"; return PB_SOLVE_INVALID_INPUT; }
        if (!std::isfinite(op->scale_bar_weight) || !(op->scale_bar_weight > 0.0) ||
            !std::isfinite(op->scale_bar_huber_delta) || op->scale_bar_huber_delta < 0.0) {
            *err = "scale-bar weight must be finite and positive and its Huber delta finite and non-negative";
            return PB_SOLVE_INVALID_INPUT;
        }
        for (int i = 0; i < pr->n_scale_bars; ++i) {
            const int a = pr->scale_bar_tracks[2 * i], b = pr->scale_bar_tracks[2 * i + 1];
            const double* d = pr->scale_bar_data + static_cast<size_t>(i) * 3;
            if (a < 0 || b < 0 || a == b || a >= m->nt || b >= m->nt || !std::isfinite(d[0]) || !(d[0] > 0.0) ||
                !std::isfinite(d[1]) || !(d[1] > 0.0) || !std::isfinite(d[2]) || !(d[2] > 0.0)) {
                *err = "problem contains an invalid scale-bar constraint";
                return PB_SOLVE_INVALID_INPUT;
            }
            m->bar_tracks.push_back(a);
            m->bar_tracks.push_back(b);
            m->bar_data.insert(m->bar_data.end(), d, d + 3);
        }
        m->ref_param = false;
        m->force_general = true;
    }
    const bool bar_scale = !m->bar_tracks.empty();

    // hasCompleteControlPointGauge (BundleAdjustValidation.cpp:181-236): three non-collinear targets
    bool cp_complete = false;
    {
        const size_t np = cp_points.size() / 3;
        for (size_t a = 0; a < np && !cp_complete; ++a)
            for (size_t b = a + 1; b < np && !cp_complete; ++b) {
                const double ab[3] = {cp_points[b * 3] - cp_points[a * 3], cp_points[b * 3 + 1] - cp_points[a * 3 + 1],
                                      cp_points[b * 3 + 2] - cp_points[a * 3 + 2]};
                const double ab2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
                if (ab2 <= 1.0e-16) continue;
                for (size_t c = b + 1; c < np; ++c) {
                    const double ac[3] = {cp_points[c * 3] - cp_points[a * 3], cp_points[c * 3 + 1] - cp_points[a * 3 + 1],
                                          cp_points[c * 3 + 2] - cp_points[a * 3 + 2]};
                    const double ac2 = ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2];
                    const double x[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
                    const double x2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
                    if (ac2 > 1.0e-16 && x2 > 1.0e-12 * ab2 * ac2) { cp_complete = true; break; }
                }
            }
    }
    // hasControlPointBaselineToFixedCamera (BundleAdjustValidation.cpp:147-179)
    auto cp_baseline_to = [&](const std::vector<int>& fixed) {
        for (size_t i = 0; i < cp_points.size() / 3; ++i)
            for (int f : fixed) {
                const double* c = &m->cams_in[static_cast<size_t>(f) * kCamStride + 9];
                if (!std::isfinite(c[0]) || !std::isfinite(c[1]) || !std::isfinite(c[2])) continue;
                const double dx = cp_points[i * 3] - c[0], dy = cp_points[i * 3 + 1] - c[1], dz = cp_points[i * 3 + 2] - c[2];
                if (dx * dx + dy * dy + dz * dz > 1.0e-16) return true;
            }
        return false;
    };

    // --- gauge (validateAndNormalizeBundleAdjustOptions, BundleAdjustValidation.cpp:772-893)
    {
        std::vector<int> fc = m->fixed_cams;
        std::sort(fc.begin(), fc.end());
        for (size_t i = 0; i < fc.size(); ++i) {
            if (fc[i] < 0 || fc[i] >= m->nc) { *err = "fixed camera index out of range"; return PB_SOLVE_INVALID_INPUT; }
            if (i && fc[i] == fc[i - 1]) { *err = "duplicate fixed camera index"; return PB_SOLVE_INVALID_INPUT; }
        }
        const bool requested = op->gauge_anchor_camera >= 0 || op->gauge_scale_camera >= 0 || op->gauge_baseline > 0.0;
        if (requested && (op->gauge_anchor_camera < 0 || op->gauge_scale_camera < 0 || op->gauge_anchor_camera >= m->nc ||
                          op->gauge_scale_camera >= m->nc || op->gauge_anchor_camera == op->gauge_scale_camera ||
                          !std::isfinite(op->gauge_baseline) || op->gauge_baseline <= 0.0)) {
            *err = "invalid fixed-baseline gauge";
            return PB_SOLVE_INVALID_INPUT;
        }
        m->gauge_anchor = op->gauge_anchor_camera;
        m->gauge_scale = op->gauge_scale_camera;
        m->gauge_baseline = op->gauge_baseline;
        std::sort(m->fixed_tracks.begin(), m->fixed_tracks.end());
        for (size_t i = 0; i < m->fixed_tracks.size(); ++i) {
            if (m->fixed_tracks[i] < 0 || m->fixed_tracks[i] >= m->nt) { *err = "fixed track index out of range"; return PB_SOLVE_INVALID_INPUT; }
            if (i && m->fixed_tracks[i] == m->fixed_tracks[i - 1]) { *err = "duplicate fixed track index"; return PB_SOLVE_INVALID_INPUT; }
        }
        if (op->refine_camera_pose && op->gauge_policy != 2) {
            // absolute pose and scale from three non-collinear control points; scale alone from
            // a control point away from a fixed camera (:826-835)
            bool abs_scale = cp_complete || bar_scale || cp_baseline_to(fc);
            if (op->gauge_policy == 1) {
                const bool complete = (cp_complete && abs_scale) || fc.size() >= 2 || (fc.size() == 1 && abs_scale);
                if (!complete) { *err = "incomplete gauge: two fixed cameras, or a fixed camera and an absolute scale, are required"; return PB_SOLVE_UNSUPPORTED; }
            } else if (!cp_complete) {
                if (fc.empty()) {
                    m->fixed_cams.push_back(0);
                    fc.push_back(0);
                    abs_scale = abs_scale || cp_baseline_to(fc);
                }
                if (!abs_scale && fc.size() < 2) {
                    const int anchor = fc[0];
                    const double* a = &m->cams_in[static_cast<size_t>(anchor) * kCamStride + 9];
                    int best = -1;
                    double bestD = 1.0e-20;
                    for (int i = 0; i < m->nc; ++i) {
                        if (i == anchor) continue;
                        const double* c = &m->cams_in[static_cast<size_t>(i) * kCamStride + 9];
                        const double d2 = (c[0] - a[0]) * (c[0] - a[0]) + (c[1] - a[1]) * (c[1] - a[1]) +
                                          (c[2] - a[2]) * (c[2] - a[2]);
                        if (std::isfinite(d2) && d2 > bestD) { bestD = d2; best = i; }
                    }
                    if (best < 0) { *err = "automatic gauge found no second camera with a non-zero baseline"; return PB_SOLVE_UNSUPPORTED; }
                    m->gauge_anchor = anchor;
                    m->gauge_scale = best;
                    m->gauge_baseline = std::sqrt(bestD);
                }
            }
        }
    }

    // --- active tracks and block numbering (prepareActiveProblem, BundleAdjustPlaMatrixProblem.cpp:29-278)
    const int nc = m->nc, nt = m->nt;
    m->active_track.assign(nt, 0);
    m->camera_block.assign(nc, -1);
    m->intrinsic_block.assign(nc, -1);
    m->calib_group.assign(nc, -1);
    m->track_block.assign(nt, -1);
    std::vector<char> cam_has_residual(nc, 0), fixed_cam(nc, 0), fixed_trk(nt, 0);
    for (int c : m->fixed_cams) fixed_cam[c] = 1;
    for (int t : m->fixed_tracks) fixed_trk[t] = 1;
    // usable observations (valid camera, finite pixel, positive weight), flagged once
    std::vector<unsigned char> use(static_cast<size_t>(m->no), 0);
    parallel_ranges(static_cast<int>(std::min<long long>(m->no, std::numeric_limits<int>::max())),
                    host_threads(m->no), [&](int, int k0, int k1) {
                        for (int k = k0; k < k1; ++k) {
                            const int c = m->obs_cam[k];
                            use[k] = c >= 0 && c < nc && std::isfinite(m->obs_u[k]) && std::isfinite(m->obs_v[k]) &&
                                     sanitized_weight(m->obs_weight[k]) > 0.0;
                        }
                    });
    auto usable = [&](long long k) { return use[k] != 0; };
    m->active_tracks = m->obs_count = m->rejected = 0;
    // The gate projects every observation: tracks are split over host threads, each thread
    // keeps its own counts, and the counts are combined in thread order.
    struct GateCounts {
        int active = 0, obs = 0, rejected = 0;
    };
    auto gate = [&](int t0, int t1, GateCounts* gc) {
        for (int t = t0; t < t1; ++t) {
            const double* X = &m->points_in[static_cast<size_t>(t) * 3];
            if (!finite3(X)) continue;
            int first = -1, count = 0;
            bool second = false, positive = true;
            double sq = 0.0;
            for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k) {
                if (!usable(k)) continue;
                const int c = m->obs_cam[k];
                first = first < 0 ? c : first;
                second = second || c != first;
                double px[2];
                if (!project(&m->cams_in[static_cast<size_t>(c) * kCamStride], X, px)) { positive = false; break; }
                const double du = px[0] - m->obs_u[k], dv = px[1] - m->obs_v[k];
                sq += sanitized_weight(m->obs_weight[k]) * (du * du + dv * dv);
                ++count;
            }
            const double rms = count > 0 ? std::sqrt(sq / (2.0 * count)) : kInf;
            if (count < 2 || !second || !positive) continue;
            if (op->max_initial_track_rms > 0.0 && rms > op->max_initial_track_rms) { ++gc->rejected; continue; }
            m->active_track[t] = 1;
            ++gc->active;
            gc->obs += count;
        }
    };
    {
        const int nthreads = host_threads(nt);
        std::vector<GateCounts> counts(nthreads);
        parallel_ranges(nt, nthreads, [&](int i, int t0, int t1) { gate(t0, t1, &counts[i]); });
        for (const GateCounts& gc : counts) {
            m->active_tracks += gc.active;
            m->obs_count += gc.obs;
            m->rejected += gc.rejected;
        }
    }
    for (int t = 0; t < nt; ++t)
        if (m->active_track[t])
            for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k)
                if (usable(k)) cam_has_residual[m->obs_cam[k]] = 1;
    m->ncb = 0;
    RigModel& rig = m->rig;
    if (op->refine_camera_pose && !rig.on) {
        for (int c = 0; c < nc; ++c)
            if (cam_has_residual[c] && !fixed_cam[c]) m->camera_block[c] = m->ncb++;
    } else if (op->refine_camera_pose) {
        // rig blocks (BundleAdjustPlaMatrixProblem.cpp:156-199): a capture with residuals gets a
        // block unless it is fixed, one of its cameras is fixed, or it holds the gauge scale
        // camera; a sensor with residuals gets one unless its extrinsic is fixed; sensor blocks
        // follow the capture blocks
        rig.capture_block.assign(rig.ncap, -1);
        rig.sensor_block.assign(rig.nsen, -1);
        std::vector<char> cap_res(rig.ncap, 0), cap_fixed(rig.ncap, 0), sen_res(rig.nsen, 0);
        for (int k = 0; k < rig.ncap; ++k) cap_fixed[k] = rig.cap_info[2 * k + 1] != 0;
        for (int c = 0; c < nc; ++c) {
            const int k = rig.cam_capture[c], s = rig.cam_sensor[c];
            cap_res[k] = cap_res[k] || cam_has_residual[c];
            cap_fixed[k] = cap_fixed[k] || fixed_cam[c] || c == m->gauge_scale;
            sen_res[s] = sen_res[s] || cam_has_residual[c];
        }
        rig.ncapb = rig.nsenb = 0;
        for (int k = 0; k < rig.ncap; ++k)
            if (cap_res[k] && !cap_fixed[k]) rig.capture_block[k] = rig.ncapb++;
        for (int s = 0; s < rig.nsen; ++s)
            if (sen_res[s] && !rig.sen_info[2 * s + 1]) rig.sensor_block[s] = rig.ncapb + rig.nsenb++;
        rig.nrb = rig.ncapb + rig.nsenb;
        // camera blocks of the kernels: every camera with residuals whose pose has a free part
        rig.cb_camera.clear();
        rig.cb_cap_block.clear();
        rig.cb_sen_block.clear();
        for (int c = 0; c < nc; ++c) {
            const int kb = rig.capture_block[rig.cam_capture[c]], sb = rig.sensor_block[rig.cam_sensor[c]];
            if (!cam_has_residual[c] || (kb < 0 && sb < 0)) continue;
            m->camera_block[c] = m->ncb++;
            rig.cb_camera.push_back(c);
            rig.cb_cap_block.push_back(kb);
            rig.cb_sen_block.push_back(sb);
        }
    }
    m->P = m->ncb;
    m->ng = 0;
    m->ni = 0;
    if (op->intrinsic_mask != 0) {
        std::vector<int> ids;
        for (int c = 0; c < nc; ++c) {
            const int id = m->group_ids.empty() ? 0 : m->group_ids[c];
            auto it = std::find(ids.begin(), ids.end(), id);
            int g;
            if (it == ids.end()) { g = static_cast<int>(ids.size()); ids.push_back(id); }
            else g = static_cast<int>(it - ids.begin());
            m->calib_group[c] = g;
        }
        m->ng = static_cast<int>(ids.size());
        for (int c = 0; c < nc; ++c) m->intrinsic_block[c] = m->P + m->calib_group[c];
        m->P += m->ng;
        // Refined columns: enabled and supported by this camera model (f, aspect, cx, cy, k1-k3, p1, p2).
        for (int p = 0; p < 9; ++p)
            if ((op->intrinsic_mask >> p) & 1u) m->int_cols[m->ni++] = p;
        if (m->ng > kMaxGroups) { *err = "more calibration groups than the dense intrinsic border holds (4)"; return PB_SOLVE_UNSUPPORTED; }
    }
    // the active, non-fixed tracks of scale bars become primary point blocks, numbered after the
    // intrinsic groups in track order; the others are eliminated
    std::vector<char> promote(nt, 0);
    for (size_t i = 0; i < m->bar_tracks.size(); ++i) {
        const int t = m->bar_tracks[i];
        if (m->active_track[t] && !fixed_trk[t]) promote[t] = 1;
    }
    m->ntb = 0;
    m->npr = 0;
    m->prom_track.clear();
    m->track_prom.assign(nt, -1);
    for (int t = 0; t < nt; ++t) {
        if (!m->active_track[t] || fixed_trk[t]) continue;
        if (promote[t]) {
            m->track_prom[t] = m->npr++;
            m->prom_track.push_back(t);
        } else {
            m->track_block[t] = m->ntb++;
        }
    }
    m->P += m->npr;
    if (rig.on) rig.P = rig.nrb + m->ng + m->npr;

    // --- intrinsic groups (initializeIntrinsicGroups, BundleAdjustPlaMatrixModel.cpp:84-231)
    m->groups.assign(m->ng, HostGroup{});
    if (m->ng > 0) {
        const double* cal = op->calibration;
        std::vector<std::vector<double>> init(m->ng * kP), ref(m->ng * kP);
        for (int c = 0; c < nc; ++c) {
            const int g = m->calib_group[c];
            double p[kP], rp[kP];
            const double* cam = &m->cams_in[static_cast<size_t>(c) * kCamStride];
            const double* rcam = &m->cams_ref[static_cast<size_t>(c) * kCamStride];
            camera_parameter_block(cam, p);
            camera_parameter_block(rcam, rp);
            init[g * kP + 0].push_back(p[0]);
            ref[g * kP + 0].push_back(rp[0]);
            init[g * kP + 1].push_back(std::exp(p[1]));
            ref[g * kP + 1].push_back(std::exp(rp[1]));
            init[g * kP + 2].push_back(cam[14] - rcam[14]);
            init[g * kP + 3].push_back(cam[15] - rcam[15]);
            ref[g * kP + 2].push_back(0.0);
            ref[g * kP + 3].push_back(0.0);
            for (int i = 4; i < kP; ++i) {
                init[g * kP + i].push_back(p[i]);
                ref[g * kP + i].push_back(rp[i]);
            }
        }
        const double low = std::max(1.0, cal[26]);
        for (int g = 0; g < m->ng; ++g) {
            HostGroup& G = m->groups[g];
            for (int p = 0; p < kP; ++p) {
                G.lower[p] = -kInf;
                G.upper[p] = kInf;
                G.enabled[p] = p < 9 && ((op->intrinsic_mask >> p) & 1u);
            }
            G.focalRef = finite_median(ref[g * kP + 0], 1.0);
            G.aspectRef = finite_median(ref[g * kP + 1], 1.0);
            G.params[0] = std::max(1e-12, finite_median(init[g * kP + 0], G.focalRef));
            G.params[1] = std::log(std::max(1e-12, finite_median(init[g * kP + 1], G.aspectRef)));
            G.prior[0] = G.focalRef;
            G.prior[1] = std::log(G.aspectRef);
            for (int p = 2; p < kP; ++p) {
                G.prior[p] = finite_median(ref[g * kP + p], 0.0);
                G.params[p] = finite_median(init[g * kP + p], G.prior[p]);
            }
            G.lower[0] = G.focalRef * cal[0];
            G.upper[0] = G.focalRef * cal[1];
            G.lower[1] = std::log(G.aspectRef * cal[2]);
            G.upper[1] = std::log(G.aspectRef * cal[3]);
            G.lower[2] = G.lower[3] = -G.focalRef * cal[4];
            G.upper[2] = G.upper[3] = G.focalRef * cal[4];
            const double lim[9] = {cal[8] * low, cal[9], cal[10], cal[11] * low, cal[12] * low, G.focalRef * cal[13],
                                   cal[14], cal[15], cal[16]};
            for (int i = 0; i < 9; ++i) { G.lower[4 + i] = -lim[i]; G.upper[4 + i] = lim[i]; }
            const double pps = std::max(1e-6, G.focalRef * cal[6]);
            const double sigma[kP] = {cal[5] * G.focalRef, cal[7], pps, pps, cal[17] * low, cal[18], cal[19],
                                      cal[20] * low, cal[21] * low, G.focalRef * cal[22], cal[23], cal[24], cal[25]};
            for (int p = 0; p < kP; ++p) {
                G.params[p] = std::min(std::max(G.params[p], G.lower[p]), G.upper[p]);
                G.invSigma[p] = G.enabled[p] ? 1.0 / std::max(1e-9, sigma[p]) : 0.0;
            }
        }
    }

    // --- reference topology: upper block pairs over all primary blocks, numbered row-major
    // (prepareOffDiagonalTopology, BundleAdjustPlaMatrixReferenceSchur.cpp:568-659)
    {
        const int P = m->P;
        // Upper pairs (lo, hi) as bits lo * P + hi of a P x P bitset.  Tracks are split over host
        // threads, each with its own bitset (a pair is recorded once however many tracks share
        // it); the bitsets are OR-ed and read out row-major, which is the sorted, deduplicated
        // pair list.
        const size_t words = (static_cast<size_t>(P) * P + 63) / 64;
        const int nthreads = host_threads(nt);
        std::vector<std::vector<unsigned long long>> bits(nthreads, std::vector<unsigned long long>(words, 0ull));
        parallel_ranges(nt, nthreads, [&](int i, int t0, int t1) {
            unsigned long long* mask = bits[i].data();
            auto connect = [&](int a, int b) {
                if (a < 0 || b < 0 || a == b) return;
                const size_t bit = static_cast<size_t>(std::min(a, b)) * P + std::max(a, b);
                mask[bit >> 6] |= 1ull << (bit & 63);
            };
            std::vector<int> tb;
            for (int t = t0; t < t1; ++t) {
                if (!m->active_track[t]) continue;
                tb.clear();
                for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k) {
                    if (!usable(k)) continue;
                    const int c = m->obs_cam[k];
                    connect(m->camera_block[c], m->intrinsic_block[c]);
                    if (m->track_block[t] >= 0) {
                        if (m->camera_block[c] >= 0) tb.push_back(m->camera_block[c]);
                        if (m->intrinsic_block[c] >= 0) tb.push_back(m->intrinsic_block[c]);
                    }
                }
                if (m->track_block[t] < 0) continue;
                std::sort(tb.begin(), tb.end());
                tb.erase(std::unique(tb.begin(), tb.end()), tb.end());
                for (size_t l = 0; l < tb.size(); ++l)
                    for (size_t r = l + 1; r < tb.size(); ++r) connect(tb[l], tb[r]);
            }
        });
        std::vector<unsigned long long>& all = bits[0];
        for (int i = 1; i < nthreads; ++i)
            for (size_t w = 0; w < words; ++w) all[w] |= bits[i][w];
        m->pairs.clear();
        for (int r = 0; r < P; ++r) {
            const size_t b0 = static_cast<size_t>(r) * P + r + 1, b1 = static_cast<size_t>(r + 1) * P;
            for (size_t b = b0; b < b1;) {
                const size_t w = b >> 6;
                unsigned long long v = all[w] >> (b & 63);
                if (!v) {
                    b = (w + 1) << 6;
                    continue;
                }
                const size_t hit = b + static_cast<size_t>(__builtin_ctzll(v));
                if (hit >= b1) break;
                m->pairs.emplace_back(r, static_cast<int>(hit - static_cast<size_t>(r) * P));
                b = hit + 1;
            }
        }
        // pose CSR (both triangles), diagonal always present
        const int nb = m->ncb;
        std::vector<std::vector<int>> rows(nb);
        for (int i = 0; i < nb; ++i) rows[i].push_back(i);
        for (const auto& pr2 : m->pairs)
            if (pr2.second < nb) {
                rows[pr2.first].push_back(pr2.second);
                rows[pr2.second].push_back(pr2.first);
            }
        m->row_ptr.assign(nb + 1, 0);
        m->col_idx.clear();
        m->diag_pos.assign(nb, -1);
        for (int i = 0; i < nb; ++i) {
            std::sort(rows[i].begin(), rows[i].end());
            for (int c : rows[i]) {
                if (c == i) m->diag_pos[i] = static_cast<int>(m->col_idx.size());
                m->col_idx.push_back(c);
            }
            m->row_ptr[i + 1] = static_cast<int>(m->col_idx.size());
        }
        // upper blocks (diagonal first in each row), with CSR positions of both orientations
        m->up_row.clear();
        m->up_col.clear();
        m->up_csr.clear();
        m->up_csr_t.clear();
        for (int i = 0; i < nb; ++i)
            for (int p = m->row_ptr[i]; p < m->row_ptr[i + 1]; ++p) {
                const int j = m->col_idx[p];
                if (j < i) continue;
                m->up_row.push_back(i);
                m->up_col.push_back(j);
                m->up_csr.push_back(p);
                int pt = -1;
                if (j != i) {
                    const int* b = &m->col_idx[m->row_ptr[j]];
                    const int* e = &m->col_idx[m->row_ptr[j + 1]];
                    pt = static_cast<int>(std::lower_bound(b, e, i) - &m->col_idx[0]);
                }
                m->up_csr_t.push_back(pt);
            }
        if (rig.on) build_rig_pattern(m, use);
    }

    // --- processing order: active tracks sorted by their smallest pose block so that a chunk of
    // consecutive tracks touches few cameras; observations of each track kept in input order.
    // The key is bounded (pose block, or nc + camera for cameras without one), so a stable
    // counting sort gives the order of sorting (key, track index).
    {
        const int nkeys = 2 * nc + 1;
        // keys and usable-observation counts per track (threads over tracks), then the counting
        // sort and the observation ranges in processing order, filled by threads over ranges
        std::vector<int> key(nt, -1), nuse(nt, 0), count(nkeys + 1, 0);
        const int nthreads = host_threads(m->no);
        parallel_ranges(nt, nthreads, [&](int, int t0, int t1) {
            for (int t = t0; t < t1; ++t) {
                if (!m->active_track[t]) continue;
                int mn = nkeys - 1, cnt = 0;
                for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k)
                    if (usable(k)) {
                        const int c = m->obs_cam[k];
                        mn = std::min(mn, m->camera_block[c] >= 0 ? m->camera_block[c] : nc + c);
                        ++cnt;
                    }
                key[t] = mn;
                nuse[t] = cnt;
            }
        });
        for (int t = 0; t < nt; ++t)
            if (key[t] >= 0) ++count[key[t] + 1];
        for (int i = 0; i < nkeys; ++i) count[i + 1] += count[i];
        m->trk_order.assign(static_cast<size_t>(count[nkeys]), 0);
        for (int t = 0; t < nt; ++t)
            if (key[t] >= 0) m->trk_order[count[key[t]]++] = t;
        const size_t ntp = m->trk_order.size();
        m->trk_obs_begin.assign(ntp + 1, 0);
        for (size_t i = 0; i < ntp; ++i) m->trk_obs_begin[i + 1] = m->trk_obs_begin[i] + nuse[m->trk_order[i]];
        m->p_obs_orig.assign(static_cast<size_t>(m->trk_obs_begin[ntp]), 0);
        parallel_ranges(static_cast<int>(ntp), nthreads, [&](int, int i0, int i1) {
            for (int i = i0; i < i1; ++i) {
                const int t = m->trk_order[i];
                int pos = m->trk_obs_begin[i];
                for (long long k = m->offs[t]; k < m->offs[t + 1]; ++k)
                    if (usable(k)) m->p_obs_orig[pos++] = static_cast<int>(k);
            }
        });
    }
    // control points of the processed tracks, in processing order
    {
        const size_t ntp = m->trk_order.size();
        std::vector<int> proc(nt, -1);
        for (size_t i = 0; i < ntp; ++i) proc[m->trk_order[i]] = static_cast<int>(i);
        std::vector<int> cnt(ntp + 1, 0);
        for (int t : m->cp_track)
            if (proc[t] >= 0) ++cnt[proc[t] + 1];
        for (size_t i = 0; i < ntp; ++i) cnt[i + 1] += cnt[i];
        m->trk_cp_begin = cnt;
        m->cp_proc.assign(static_cast<size_t>(cnt[ntp]) * 12, 0.0);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (size_t i = 0; i < m->cp_track.size(); ++i) {
            const int p = proc[m->cp_track[i]];
            if (p < 0) continue;
            std::copy(&m->cp_rec[i * 12], &m->cp_rec[i * 12] + 12, &m->cp_proc[static_cast<size_t>(fill[p]++) * 12]);
        }
    }
    // structure hash for pattern reuse
    {
        unsigned long long h = 1469598103934665603ull;
        auto mix = [&](long long v) { h = (h ^ static_cast<unsigned long long>(v)) * 1099511628211ull; };
        mix(nc); mix(nt); mix(m->no); mix(m->ncb); mix(m->ng); mix(m->ni);
        // the processing-order observations in 16 fixed segments hashed by host threads, the
        // segment hashes mixed in order (the value does not depend on the thread count)
        {
            constexpr int kHashSegments = 16;
            const int nobs = static_cast<int>(m->p_obs_orig.size());
            unsigned long long seg_h[kHashSegments];
            parallel_ranges(kHashSegments, std::min(kHashSegments, host_threads(nobs)), [&](int, int s0, int s1) {
                for (int sgm = s0; sgm < s1; ++sgm) {
                    unsigned long long g = 1469598103934665603ull;
                    const int i0 = static_cast<int>(static_cast<long long>(nobs) * sgm / kHashSegments);
                    const int i1 = static_cast<int>(static_cast<long long>(nobs) * (sgm + 1) / kHashSegments);
                    for (int i = i0; i < i1; ++i) {
                        g = (g ^ static_cast<unsigned long long>(m->p_obs_orig[i])) * 1099511628211ull;
                        g = (g ^ static_cast<unsigned long long>(m->obs_cam[m->p_obs_orig[i]])) * 1099511628211ull;
                    }
                    seg_h[sgm] = g;
                }
            });
            for (int sgm = 0; sgm < kHashSegments; ++sgm) mix(static_cast<long long>(seg_h[sgm]));
        }
        for (int t : m->trk_order) mix(t);
        if (m->rig.on) {
            const RigModel& R = m->rig;
            mix(R.nrb);
            for (int c = 0; c < nc; ++c) { mix(R.cam_capture[c]); mix(R.cam_sensor[c]); }
            for (int v : R.capture_block) mix(v);
            for (int v : R.sensor_block) mix(v);
        }
        m->structure_hash = static_cast<long long>(h);
    }
    m->chunks_ready[0] = m->chunks_ready[1] = false;
    return 0;
}

size_t chunk_smem_bytes(int precision, int max_obs, int max_tracks, int ni, int nb) {
    const size_t ts = precision == PB_PRECISION_FP64 ? 8 : 4;  // Jacobian storage
    const size_t vs = 8;                                        // double / float-float values
    const size_t nA = 6 + static_cast<size_t>(ni);
    const size_t mo = static_cast<size_t>(max_obs), mt = static_cast<size_t>(max_tracks);
    auto al = [](size_t v) { return (v + 15) & ~static_cast<size_t>(15); };
    size_t s = 0;
    auto st = [](size_t words) { return static_cast<size_t>(chunk_stride(static_cast<int>(words))); };
    s += al(mo * 9 * 8);            // point normal equations per observation, then the track factor (FP64)
    s += al(mo * st(2 * nA) * ts);  // A_o = [J_pose | J_intrinsic]
    s += al(mo * st(18) * vs);      // G_o = J_pose^T Y_o
    s += al(mo * st(6) * vs);       // Y_o
    s += al(mo * st(6) * vs);       // M_o, Y_o q, w
    s += al(mo * st(nA) * vs);      // gradient -J^T w r of the pose and intrinsic columns
    s += al(mo * 4) * 2;        // observation flags, track records
    s += al(mt * st(static_cast<size_t>(nb) * 3) * vs);  // per-track K
    s += al((mt + 1) * 4);      // track starts
    s += al(mt * 4);            // calibration groups present per track
    s += al(mt * 8);            // control-point cost per track
    s += al(40 * 8);            // warp partial costs and track counts, flags
    return s;
}

namespace {

struct ChunkLimits {
    int max_obs, max_cams, max_pairs, max_tracks, precision;
};

// Owner-gather schedule of one chunk (phase D of the assembly kernel).  The chunk's tasks are
// the rows of its pose pair blocks (6 per pair slot: task id 6 s + x) followed by its camera rows
// (2 + ng ni per chunk camera: rhs, direct rhs, border columns).  A task's cost is estimated from
// the terms its owner thread sums (compensated multiply-adds: 18 per own term and 20 per coupling
// of a pose row; per observation 20 / 8 for the two gradient rows, and for a border row 2, plus
// 12 for a direct term and 18 for a coupling through the track's intrinsic sums K).  The tasks are
// cut into rounds of 32 (one per warp lane) and the rounds are dealt to the kAssembleWarps warps
// by longest processing time: each round, costed by its longest task, goes to the warp with the
// least load so far.
//   - FP32 path: the rounds keep the natural task order.  Neighbouring lanes then own rows of the
//     same pair block or camera and read the same observation records (shared-memory broadcasts);
//     sorting by cost broke that and was measured slower (3.49 against 2.82 ms per 500-camera
//     launch).
//   - FP64 path: the FP64 pipe executes every lane slot of a warp instruction whether the lane is
//     active or not, so the rounds are built from whole pair blocks and cameras sorted by
//     decreasing cost (lanes of a round then run loops of similar length): 7.16 against 7.77 ms.
// The schedule only decides which thread owns a task: every output is still summed by one thread
// in the order of its item list, so results do not depend on it.
void schedule_owner_tasks(const HostModel* m, int chunk_obs_start, int obs_end, int p_first, int p_end,
                          const std::vector<unsigned char>& obs_lcam, ChunkSet& cs, int slot0, int nslots,
                          int lcam0, int ncl) {
    const int ng = m->ng, ni = m->ni;
    const int crow = 2 + ng * ni;
    const int nobs = obs_end - chunk_obs_start;
    // calibration group and eliminated flag of every chunk observation, groups present per track
    // (per-thread buffers: the planner calls this once per chunk)
    thread_local std::vector<int> grp, tmask;
    thread_local std::vector<char> elim;
    thread_local std::vector<std::pair<long long, int>> cost;
    grp.assign(nobs, -1);
    tmask.assign(nobs, 0);
    elim.assign(nobs, 0);
    for (int p = p_first; p < p_end; ++p) {
        const int o0 = m->trk_obs_begin[p], o1 = m->trk_obs_begin[p + 1];
        const bool el = m->track_block[m->trk_order[p]] >= 0;
        int mask = 0;
        for (int o = o0; o < o1; ++o) {
            const int g = ng > 0 ? m->calib_group[m->obs_cam[m->p_obs_orig[o]]] : -1;
            grp[o - chunk_obs_start] = g;
            if (g >= 0) mask |= 1 << g;
        }
        for (int o = o0; o < o1; ++o) {
            tmask[o - chunk_obs_start] = mask;
            elim[o - chunk_obs_start] = el ? 1 : 0;
        }
    }
    const int ntask = 6 * nslots + crow * ncl;
    cost.resize(ntask);
    for (int sl = 0; sl < nslots; ++sl) {
        long long c = 0;
        for (int it = cs.slot_item_begin[slot0 + sl]; it < cs.slot_item_begin[slot0 + sl + 1]; ++it) {
            const unsigned item = cs.slot_items[it];
            c += (item & 0xFF) == (item >> 8) ? 18 : 20;
        }
        for (int x = 0; x < 6; ++x) cost[6 * sl + x] = {c, 6 * sl + x};
    }
    for (int l = 0; l < ncl; ++l) {
        const int b0 = cs.lcam_obs_begin[lcam0 + l], b1 = cs.lcam_obs_begin[lcam0 + l + 1];
        for (int row = 0; row < crow; ++row) {
            long long c = 0;
            if (row < 2) {
                c = static_cast<long long>(b1 - b0) * (row == 0 ? 20 : 8);
            } else {
                const int g = (row - 2) / ni;
                for (int it = b0; it < b1; ++it) {
                    const int ob = cs.lcam_obs[it];
                    c += 2 + (grp[ob] == g ? 12 : 0) + (elim[ob] && ((tmask[ob] >> g) & 1) ? 18 : 0);
                }
            }
            const int id = 6 * nslots + l * crow + row;
            cost[id] = {c, id};
        }
    }
    {
        // The rows are grouped by the code path they take, so that a round's lanes run the same
        // branch (on the FP64 path the FP64 pipe spends a warp instruction's slots on idle lanes
        // too).  Pair rows: the rows of diagonal slots (own terms J^T M J) before those
        // of off-diagonal slots (couplings G G^T).  Camera rows: the gradient rows of every camera,
        // then the border rows of each camera's own calibration group (own term and intrinsic
        // coupling), then the border rows of the other groups (coupling only, often empty).  The
        // six rows of a slot, and a camera's rows of one class, stay on neighbouring lanes, which
        // read the same observation records.  Each row sums the same terms in the same order
        // whatever its lane, so the order changes no result.
        thread_local std::vector<std::pair<long long, int>> order;
        order.clear();
        order.reserve(cost.size());
        // pair slots of each class and the cameras by decreasing work (stable: ties keep their
        // order), so that the lanes of a round loop over similar numbers of terms
        thread_local std::vector<std::pair<long long, int>> diag, offdiag, cams;
        diag.clear();
        offdiag.clear();
        cams.clear();
        for (int sl = 0; sl < nslots; ++sl) {
            const int pk = cs.pairs[slot0 + sl];
            ((pk & 0xFFFF) == (pk >> 16) ? diag : offdiag).push_back({cost[6 * sl].first, sl});
        }
        auto by_work = [](const auto& a, const auto& b) { return a.first > b.first; };
        std::stable_sort(diag.begin(), diag.end(), by_work);
        std::stable_sort(offdiag.begin(), offdiag.end(), by_work);
        for (const auto* cls : {&diag, &offdiag})
            for (const auto& s : *cls)
                for (int x = 0; x < 6; ++x) order.push_back(cost[6 * s.second + x]);
        for (int l = 0; l < ncl; ++l)
            cams.push_back({cs.lcam_obs_begin[lcam0 + l + 1] - cs.lcam_obs_begin[lcam0 + l], l});
        std::stable_sort(cams.begin(), cams.end(), by_work);
        auto cam_group = [&](int l) {
            const int b0 = cs.lcam_obs_begin[lcam0 + l], b1 = cs.lcam_obs_begin[lcam0 + l + 1];
            return b1 > b0 ? grp[cs.lcam_obs[b0]] : -1;
        };
        for (const auto& c : cams)
            for (int row = 0; row < std::min(2, crow); ++row) order.push_back(cost[6 * nslots + c.second * crow + row]);
        for (int pass = 0; pass < 2; ++pass)
            for (const auto& c : cams) {
                const int l = c.second, g = cam_group(l);
                for (int row = 2; row < crow; ++row)
                    if (((row - 2) / ni == g) == (pass == 0)) order.push_back(cost[6 * nslots + l * crow + row]);
            }
        cost.swap(order);
    }
    const int nrounds = (ntask + 31) / 32;
    thread_local std::vector<int> owner;
    owner.assign(nrounds, 0);
    long long load[kAssembleWarps] = {};
    int nown[kAssembleWarps] = {};
    for (int r = 0; r < nrounds; ++r) {
        long long rc = 0;
        for (int k = 32 * r; k < std::min(ntask, 32 * r + 32); ++k) rc = std::max(rc, cost[k].first);
        const int w = static_cast<int>(std::min_element(load, load + kAssembleWarps) - load);
        load[w] += rc;
        owner[r] = w;
        ++nown[w];
    }
    // each warp's rounds in round order, the warps one after the other
    const size_t base = cs.task_list.size();
    cs.task_list.resize(base + 32 * static_cast<size_t>(nrounds));
    size_t at[kAssembleWarps];
    size_t pos = base;
    for (int w = 0; w < kAssembleWarps; ++w) {
        cs.warp_task_begin.push_back(static_cast<int>(pos));
        at[w] = pos;
        pos += 32 * static_cast<size_t>(nown[w]);
    }
    unsigned short* out = cs.task_list.data();
    for (int r = 0; r < nrounds; ++r) {
        unsigned short* dst = out + at[owner[r]];
        at[owner[r]] += 32;
        for (int lane = 0; lane < 32; ++lane) {
            const int k = 32 * r + lane;
            dst[lane] = k < ntask ? static_cast<unsigned short>(cost[k].second) : kNoTask;
        }
    }
}

// Greedy chunk plan of the processing-order tracks [p_begin, p_range_end) into `cs` (a partial plan:
// its begin arrays are local to it, obs_begin holds global observation indices).  obs_lcam is
// the plan-wide per-observation array; this range writes only its own observations.
int plan_range(const HostModel* m, const ChunkLimits& lim, int p_begin, int p_range_end, ChunkSet& cs,
               std::vector<unsigned char>& obs_lcam, std::string* err) {
    const int max_obs = lim.max_obs, max_cams = lim.max_cams, max_pairs = lim.max_pairs, max_tracks = lim.max_tracks;
    const int obs_range_end = m->trk_obs_begin[p_range_end];
    std::vector<int> stamp(m->nc, -1), local(m->nc, -1);
    std::vector<unsigned char> pair_seen;  // max_cams * max_cams
    std::vector<int> ccams;                // cameras (with pose blocks) of the open chunk
    std::vector<std::pair<int, int>> cpairs;
    int chunk = 0;
    int chunk_obs_start = m->trk_obs_begin[p_begin];
    int chunk_trk_start = p_begin;
    std::vector<int> slot_of;                        // local pair (a, b) -> chunk slot
    cs.obs_begin.push_back(chunk_obs_start);
    cs.slot_item_begin.push_back(0);
    cs.lcam_obs_begin.push_back(0);
    cs.cam_begin.push_back(0);
    cs.pair_begin.push_back(0);
    auto close_chunk = [&](int obs_end) {
        // order local cameras by pose block so that li < lj <=> block_i < block_j
        std::vector<int> order(ccams.size());
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int a, int b) {
            return m->camera_block[ccams[a]] < m->camera_block[ccams[b]];
        });
        std::vector<int> remap(ccams.size());
        for (size_t i = 0; i < order.size(); ++i) remap[order[i]] = static_cast<int>(i);
        for (size_t i = 0; i < order.size(); ++i) cs.cams.push_back(ccams[order[i]]);
        for (int o = chunk_obs_start; o < obs_end; ++o)
            if (obs_lcam[o] != 255) obs_lcam[o] = static_cast<unsigned char>(remap[obs_lcam[o]]);
        // the chunk's pairs in remapped local indices, numbered in (lower, upper) order: marked in
        // the slot matrix, then read out row by row
        const int ncl = static_cast<int>(ccams.size());
        slot_of.assign(static_cast<size_t>(ncl) * ncl, -1);
        for (auto& p : cpairs) {
            int a = remap[p.first], b = remap[p.second];
            if (a > b) std::swap(a, b);
            slot_of[static_cast<size_t>(a) * ncl + b] = 0;
        }
        int nslot = 0;
        for (int a = 0; a < ncl; ++a)
            for (int b = a; b < ncl; ++b) {
                int& sl = slot_of[static_cast<size_t>(a) * ncl + b];
                if (sl < 0) continue;
                sl = nslot++;
                cs.pairs.push_back(a | (b << 16));
                cs.pair_upper.push_back(-1);  // resolved once all chunks exist
            }
        // Items of every pair slot, in track order: the observation's own term (oa == ob) on the
        // diagonal slot, and for eliminated tracks the coupling -G_oa G_ob^T of two observations
        // with oa on the lower chunk camera (both orientations when they share a camera).
        // Two passes over the chunk's tracks: count the items of every slot, then place them.
        std::vector<int> cnt(static_cast<size_t>(nslot) + 1, 0);
        const int p_first = chunk_trk_start;
        int p_end = chunk_trk_start;
        while (p_end < p_range_end && m->trk_obs_begin[p_end] < obs_end) ++p_end;
        for (int pass = 0; pass < 2; ++pass) {
            auto emit = [&](int a, int b, unsigned short item) {
                const int sl = slot_of[static_cast<size_t>(a) * ncl + b];
                if (pass == 0) ++cnt[sl + 1];
                else cs.slot_items[cnt[sl]++] = item;
            };
            for (int p = chunk_trk_start; p < p_end; ++p) {
                const int o0 = m->trk_obs_begin[p], o1 = m->trk_obs_begin[p + 1];
                const bool el = m->track_block[m->trk_order[p]] >= 0;
                for (int i = o0; i < o1; ++i) {
                    const int li = obs_lcam[i];
                    if (li == 255) continue;
                    const int ii = i - chunk_obs_start;
                    emit(li, li, static_cast<unsigned short>(ii | (ii << 8)));
                    if (!el) continue;
                    for (int j = i + 1; j < o1; ++j) {
                        const int lj = obs_lcam[j];
                        if (lj == 255) continue;
                        const int jj = j - chunk_obs_start;
                        if (li < lj) {
                            emit(li, lj, static_cast<unsigned short>(ii | (jj << 8)));
                        } else if (li > lj) {
                            emit(lj, li, static_cast<unsigned short>(jj | (ii << 8)));
                        } else {
                            emit(li, li, static_cast<unsigned short>(ii | (jj << 8)));
                            emit(li, li, static_cast<unsigned short>(jj | (ii << 8)));
                        }
                    }
                }
            }
            if (pass == 0) {
                const int base = static_cast<int>(cs.slot_items.size());
                cnt[0] = base;
                for (int i = 0; i < nslot; ++i) cnt[i + 1] += cnt[i];
                cs.slot_items.resize(static_cast<size_t>(cnt[nslot]));
                // cnt[i] is now the begin of slot i: the fill position of the second pass
                for (int i = 0; i < nslot; ++i) cs.slot_item_begin.push_back(cnt[i + 1]);
            }
        }
        chunk_trk_start = p_end;
        // observations of every chunk camera, in observation order (counting sort)
        {
            std::vector<int> cc(static_cast<size_t>(ncl) + 1, 0);
            for (int o = chunk_obs_start; o < obs_end; ++o)
                if (obs_lcam[o] != 255) ++cc[obs_lcam[o] + 1];
            const int base = static_cast<int>(cs.lcam_obs.size());
            cc[0] = base;
            for (int l = 0; l < ncl; ++l) {
                cc[l + 1] += cc[l];
                cs.lcam_obs_begin.push_back(cc[l + 1]);
            }
            cs.lcam_obs.resize(static_cast<size_t>(cc[ncl]));
            for (int o = chunk_obs_start; o < obs_end; ++o)
                if (obs_lcam[o] != 255) cs.lcam_obs[cc[obs_lcam[o]]++] = static_cast<unsigned char>(o - chunk_obs_start);
        }
        schedule_owner_tasks(m, chunk_obs_start, obs_end, p_first, p_end, obs_lcam, cs, cs.pair_begin.back(),
                             nslot, cs.cam_begin.back(), ncl);
        cs.obs_begin.push_back(obs_end);
        cs.cam_begin.push_back(static_cast<int>(cs.cams.size()));
        cs.pair_begin.push_back(static_cast<int>(cs.pairs.size()));
        for (int c : ccams) stamp[c] = -1;
        ccams.clear();
        cpairs.clear();
        ++chunk;
        chunk_obs_start = obs_end;
    };
    pair_seen.assign(static_cast<size_t>(max_cams) * max_cams, 0);
    std::vector<int> tcams, ol;
    std::vector<std::pair<int, int>> tpairs;
    for (int p = p_begin; p < p_range_end; ++p) {
        const int t = m->trk_order[p];
        const int o0 = m->trk_obs_begin[p], o1 = m->trk_obs_begin[p + 1];
        const bool elim = m->track_block[t] >= 0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            // cameras and pairs this track would add to the open chunk
            tcams.clear();
            tpairs.clear();
            int new_cams = 0;
            auto lidx = [&](int c) -> int {
                if (stamp[c] == chunk) return local[c];
                for (size_t i = 0; i < tcams.size(); ++i)
                    if (tcams[i] == c) return static_cast<int>(ccams.size() + i);
                tcams.push_back(c);
                ++new_cams;
                return static_cast<int>(ccams.size() + tcams.size() - 1);
            };
            ol.clear();
            for (int o = o0; o < o1; ++o) {
                const int c = m->obs_cam[m->p_obs_orig[o]];
                ol.push_back(m->camera_block[c] >= 0 ? lidx(c) : -1);
            }
            const int ncams_after = static_cast<int>(ccams.size()) + new_cams;
            int new_pairs = 0;
            auto seen = [&](int a, int b) {
                if (a > b) std::swap(a, b);
                if (a < max_cams && b < max_cams && pair_seen[static_cast<size_t>(a) * max_cams + b]) return true;
                for (auto& q : tpairs)
                    if (q.first == a && q.second == b) return true;
                return false;
            };
            for (int i = 0; i < o1 - o0; ++i) {
                if (ol[i] < 0) continue;
                if (!seen(ol[i], ol[i])) { tpairs.emplace_back(ol[i], ol[i]); ++new_pairs; }
                if (!elim) continue;
                for (int j = i + 1; j < o1 - o0; ++j) {
                    if (ol[j] < 0) continue;
                    const int a = std::min(ol[i], ol[j]), b = std::max(ol[i], ol[j]);
                    if (!seen(a, b)) { tpairs.emplace_back(a, b); ++new_pairs; }
                }
            }
            const int obs_after = o1 - chunk_obs_start;
            const bool fits = obs_after <= max_obs && ncams_after <= max_cams &&
                              static_cast<int>(cpairs.size()) + new_pairs <= max_pairs &&
                              p - chunk_trk_start + 1 <= max_tracks;
            if (!fits) {
                if (attempt == 0 && o0 > chunk_obs_start) {
                    for (auto& q : cpairs) pair_seen[static_cast<size_t>(q.first) * max_cams + q.second] = 0;
                    close_chunk(o0);
                    continue;
                }
                *err = "a track has more observations than one assembly chunk holds";
                return PB_SOLVE_UNSUPPORTED;
            }
            for (size_t i = 0; i < tcams.size(); ++i) {
                stamp[tcams[i]] = chunk;
                local[tcams[i]] = static_cast<int>(ccams.size());
                ccams.push_back(tcams[i]);
            }
            for (auto& q : tpairs) {
                pair_seen[static_cast<size_t>(q.first) * max_cams + q.second] = 1;
                cpairs.push_back(q);
            }
            for (int i = 0; i < o1 - o0; ++i) obs_lcam[o0 + i] = ol[i] < 0 ? 255 : static_cast<unsigned char>(ol[i]);
            break;
        }
    }
    if (chunk_obs_start < obs_range_end || p_range_end == p_begin) {
        for (auto& q : cpairs) pair_seen[static_cast<size_t>(q.first) * max_cams + q.second] = 0;
        close_chunk(obs_range_end);
    }
    return 0;
}

}  // namespace

// Chunk plan of the whole problem: fixed segments of the processing order (16 for problems of
// 64k observations or more, else one) are planned concurrently and concatenated in order.  The
// segment count does not depend on the host's thread count, so the plan - and the summation
// order of the assembly - is the same on every machine.
int build_chunks(HostModel* m, int precision, size_t smem_budget, std::string* err) {
    ChunkSet& cs = m->chunks[precision];
    // A chunk is bounded by its observations (one thread each, shared-memory records); cameras
    // are chunk-local 8-bit indices (255 marks an observation without a pose block) and pairs
    // only size the partial buffers.
    // two CTAs per SM: at most half of the 228 KB of shared memory of an SM each, less the
    // 1 KB the runtime reserves per CTA
    const size_t per_cta = std::min(smem_budget, static_cast<size_t>(113 * 1024));
    const int nb = m->ng * m->ni;
    int max_obs = 256;
    const int max_cams = 254;
    // pair slots of a chunk: its owner-gather task ids (6 per slot plus the camera rows) are 16-bit
    const int max_pairs = 8192;
    // tracks of a chunk: per-track intrinsic sums in shared memory; a quarter of the observations
    // (tracks of four or more views fill a chunk, shorter ones close it early)
    auto tracks_for = [](int mo) { return std::max(8, mo / 4); };
    while (chunk_smem_bytes(precision, max_obs, tracks_for(max_obs), m->ni, nb) > per_cta && max_obs > 32) max_obs -= 32;
    const int max_tracks = tracks_for(max_obs);
    if (chunk_smem_bytes(precision, max_obs, max_tracks, m->ni, nb) > per_cta) {
        *err = "assembly chunk does not fit in shared memory";
        return PB_SOLVE_UNSUPPORTED;
    }
    cs = ChunkSet{};
    cs.max_obs = max_obs;
    cs.max_cams = max_cams;
    cs.max_pairs = max_pairs;
    cs.max_tracks = max_tracks;
    const ChunkLimits lim{max_obs, max_cams, max_pairs, max_tracks, precision};
    const int ntp = static_cast<int>(m->trk_order.size());
    const long long nop = static_cast<long long>(m->p_obs_orig.size());
    cs.obs_lcam.assign(static_cast<size_t>(nop), 255);
    constexpr int kPlanSegments = 16;
    const int nseg = nop >= 65536 && ntp >= kPlanSegments ? kPlanSegments : 1;
    std::vector<int> seg(nseg + 1, 0);
    seg[nseg] = ntp;
    for (int k = 1; k < nseg; ++k) {
        const long long target = nop * k / nseg;
        const int* b = m->trk_obs_begin.data();
        seg[k] = std::max(seg[k - 1], static_cast<int>(std::lower_bound(b, b + ntp, target) - b));
    }
    std::vector<ChunkSet> parts(nseg);
    std::vector<int> rcs(nseg, 0);
    std::vector<std::string> errs(nseg);
    parallel_ranges(nseg, std::min(nseg, host_threads(nop)), [&](int, int k0, int k1) {
        for (int k = k0; k < k1; ++k) rcs[k] = plan_range(m, lim, seg[k], seg[k + 1], parts[k], cs.obs_lcam, &errs[k]);
    });
    for (int k = 0; k < nseg; ++k)
        if (rcs[k]) {
            *err = errs[k];
            return rcs[k];
        }
    // concatenate the segment plans
    cs.obs_begin.push_back(0);
    cs.cam_begin.push_back(0);
    cs.pair_begin.push_back(0);
    cs.slot_item_begin.push_back(0);
    cs.lcam_obs_begin.push_back(0);
    for (const ChunkSet& q : parts) {
        const int cam0 = static_cast<int>(cs.cams.size()), pair0 = static_cast<int>(cs.pairs.size());
        const int item0 = static_cast<int>(cs.slot_items.size()), lobs0 = static_cast<int>(cs.lcam_obs.size());
        cs.obs_begin.insert(cs.obs_begin.end(), q.obs_begin.begin() + 1, q.obs_begin.end());
        for (size_t i = 1; i < q.cam_begin.size(); ++i) cs.cam_begin.push_back(cam0 + q.cam_begin[i]);
        for (size_t i = 1; i < q.pair_begin.size(); ++i) cs.pair_begin.push_back(pair0 + q.pair_begin[i]);
        for (size_t i = 1; i < q.slot_item_begin.size(); ++i) cs.slot_item_begin.push_back(item0 + q.slot_item_begin[i]);
        for (size_t i = 1; i < q.lcam_obs_begin.size(); ++i) cs.lcam_obs_begin.push_back(lobs0 + q.lcam_obs_begin[i]);
        cs.cams.insert(cs.cams.end(), q.cams.begin(), q.cams.end());
        cs.pairs.insert(cs.pairs.end(), q.pairs.begin(), q.pairs.end());
        cs.pair_upper.insert(cs.pair_upper.end(), q.pair_upper.begin(), q.pair_upper.end());
        cs.slot_items.insert(cs.slot_items.end(), q.slot_items.begin(), q.slot_items.end());
        cs.lcam_obs.insert(cs.lcam_obs.end(), q.lcam_obs.begin(), q.lcam_obs.end());
        const int task0 = static_cast<int>(cs.task_list.size());
        for (int v : q.warp_task_begin) cs.warp_task_begin.push_back(task0 + v);
        cs.task_list.insert(cs.task_list.end(), q.task_list.begin(), q.task_list.end());
    }
    cs.warp_task_begin.push_back(static_cast<int>(cs.task_list.size()));
    // map each chunk pair to its upper pose block and build the reduce lists
    const int nupper = static_cast<int>(m->up_row.size());
    // upper index lookup per row: sorted by col
    std::vector<int> up_begin(m->ncb + 1, 0);
    for (int u = 0; u < nupper; ++u) up_begin[m->up_row[u] + 1]++;
    for (int i = 0; i < m->ncb; ++i) up_begin[i + 1] += up_begin[i];
    std::vector<int> count_up(nupper + 1, 0), count_cam(m->ncb + 1, 0);
    // upper block of a camera-block pair: a dense table for up to 1024 camera blocks, else a
    // binary search in the row
    const bool dense = m->ncb <= 1024;
    std::vector<int> up_of;
    if (dense) {
        up_of.assign(static_cast<size_t>(m->ncb) * m->ncb, -1);
        for (int u = 0; u < nupper; ++u) up_of[static_cast<size_t>(m->up_row[u]) * m->ncb + m->up_col[u]] = u;
    }
    for (int c = 0; c < cs.n(); ++c) {
        for (int s = cs.pair_begin[c]; s < cs.pair_begin[c + 1]; ++s) {
            const int a = cs.pairs[s] & 0xFFFF, b = cs.pairs[s] >> 16;
            const int bi = m->camera_block[cs.cams[cs.cam_begin[c] + a]];
            const int bj = m->camera_block[cs.cams[cs.cam_begin[c] + b]];
            int u;
            if (dense) {
                u = up_of[static_cast<size_t>(bi) * m->ncb + bj];
            } else {
                const int* cb = &m->up_col[up_begin[bi]];
                const int* ce = &m->up_col[0] + up_begin[bi + 1];
                const int* f = std::lower_bound(cb, ce, bj);
                u = (f == ce || *f != bj) ? -1 : static_cast<int>(f - &m->up_col[0]);
            }
            if (u < 0) { *err = "internal: chunk pair outside the reduced pattern"; return PB_SOLVE_NUMERICAL_FAILURE; }
            cs.pair_upper[s] = u;
            count_up[u + 1]++;
        }
        for (int l = cs.cam_begin[c]; l < cs.cam_begin[c + 1]; ++l) count_cam[m->camera_block[cs.cams[l]] + 1]++;
    }
    for (int u = 0; u < nupper; ++u) count_up[u + 1] += count_up[u];
    for (int i = 0; i < m->ncb; ++i) count_cam[i + 1] += count_cam[i];
    cs.up_contrib_begin = count_up;
    cs.cam_contrib_begin = count_cam;
    cs.up_contrib.assign(count_up[nupper], 0);
    cs.cam_contrib.assign(count_cam[m->ncb], 0);
    std::vector<int> fill_up(count_up.begin(), count_up.end() - 1), fill_cam(count_cam.begin(), count_cam.end() - 1);
    for (int c = 0; c < cs.n(); ++c) {
        for (int s = cs.pair_begin[c]; s < cs.pair_begin[c + 1]; ++s) cs.up_contrib[fill_up[cs.pair_upper[s]]++] = s;
        for (int l = cs.cam_begin[c]; l < cs.cam_begin[c + 1]; ++l)
            cs.cam_contrib[fill_cam[m->camera_block[cs.cams[l]]]++] = l;
    }
    m->chunks_ready[precision] = true;
    return 0;
}

}  // namespace pb
