// pb_internal.h -- host/device shared declarations of the GB300 reduced-Schur BA backend.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pb_gpu.h"

namespace pb {

constexpr int kCamStride = PB_CAMERA_STRIDE;
constexpr int kP = PB_INTRINSIC_COUNT;  // intrinsic parameters per calibration group
constexpr int kMaxNI = 9;               // refinable intrinsic columns of this camera model
constexpr int kMaxGroups = 4;           // calibration groups held in the dense border
constexpr int kMaxNB = kMaxGroups * kMaxNI;
constexpr int kGroupRec = 6 * kP;       // params, prior, invSigma, lower, upper, enabled
constexpr int kTrackRec = 12;           // L (upper 3x3: 6), q (3), rhs (3)
constexpr int kAssembleWarps = 8;       // warps of an assembly CTA (256 threads)
constexpr unsigned short kNoTask = 0xFFFF;  // idle lane of an owner-gather round

// Device-side descriptors passed by value to kernels.
struct Shape {
    int nc;          // cameras
    int ntp;         // processed (active) tracks
    long long nop;   // processed observations
    int ncb;         // pose blocks
    int ng;          // calibration groups (0 when no intrinsic is refined)
    int ni;          // refined intrinsic columns per group
    int nb;          // ng * ni
    int n;           // reduced dimension 6 * ncb + nb
    int nchunks;
    int nupper;      // upper pose blocks incl. diagonal
    int nnzb;        // CSR pose blocks (both triangles)
    int loss;
    double loss_scale;
    int gauge_anchor, gauge_scale;
    double gauge_baseline;
    int int_cols[kMaxNI];
    int max_obs, max_cams, max_pairs, max_tracks;  // chunk limits of the active chunk set
    // 1: the reference point parameterisation of image-only problems (point steps X + s(X) dX,
    // Euler target rotation steps); 0: plain X + dX and world-frame rotation-vector steps
    // (useReferencePointParameterization, BundleAdjustPlaMatrixAssembly.cpp:24-30)
    int ref_param;
    int ncp;             // control-point constraints of processed tracks
    double cp_huber;     // Huber delta of the control-point residuals (m)
    int npr;             // tracks promoted to primary point blocks (scale bars)
    int nbar;            // scale bars
    double bar_huber;    // Huber delta of the scale-bar residuals (m)
    float loss_scale_hi, loss_scale_lo;  // loss_scale as float-float (mixed-path linearisation)
    int rig;             // 1: camera blocks are chained to rig blocks (no gauge tangent, damping after the map)
};

// float-float pair (hi, lo) of device state copies: CUDA's float2 in device code, a struct of the
// same layout for the host-only compilation of this header
#if defined(__CUDACC__)
using ff2 = float2;
#else
struct alignas(8) ff2 {
    float x, y;
};
#endif

struct DevPtrs {
    // cameras
    double* cams_state;   // nc * 32, pose state (intrinsics as input)
    double* cams_input;   // nc * 32
    double* cams_ref;     // nc * 32 intrinsic reference cameras
    double* cams_eff;     // nc * 32 effective cameras of the current state
    double* cams_trial;   // n_alpha * nc * 32 trial cameras
    int* cam_block;       // nc
    int* cam_group;       // nc (-1 without groups)
    double* groups;       // ng * kGroupRec
    double* groups_trial; // n_alpha * ng * kGroupRec
    double* gauge_basis;  // 6 (two world-frame tangent directions)
    // tracks (processing order)
    int* trk_obs_begin;   // ntp + 1
    int* trk_block;       // ntp
    int* trk_free;        // ntp: 1 when the point moves (eliminated or promoted), else 0
    int* trk_prom;        // ntp: promoted index (scale bars), or -1
    int* prom_proc;       // npr: processing index of each promoted track
    int* bar_pidx;        // 2 per scale bar: processing indices of its tracks, -1 when not processed
    double* bar_par;      // 2 per scale bar: measured distance, residual scale sqrt(weight) / sigma
    int* trk_orig;        // ntp
    double* points;       // ntp * 3
    double* points0;      // ntp * 3
    double* pscale;       // ntp: point step scale s(X) of the current points
    int* trk_cp_begin;    // ntp + 1: control points of each processed track
    double* cp_rec;       // 12 per control point: whitening sqrt(weight) W (row-major), target P
    // float-float copies read by the mixed-path weight and gradient, written with the FP64 state
    // (k_effective, k_accept) and the observations
    ff2* cams_ff;      // nc * kCamFF: effective cameras
    ff2* pscale_ff;    // ntp
    ff2* obs_w_ff;     // nop: observation weight (processing order)
    // observations (processing order)
    int* obs_cam;
    double* obs_u;
    double* obs_v;
    double* obs_w;        // sanitized weight / measurementScale^2
    int* obs_trk;
    unsigned char* obs_lcam;
    int* obs_orig;        // original observation index
    // chunks
    int* ch_obs_begin;
    int* ch_cam_begin;
    int* ch_cams;         // global camera indices
    int* ch_pair_begin;
    int* ch_pairs;        // li | lj << 16, li <= lj
    int* slot_item_begin; // pair slots + 1: items of each chunk pair slot
    unsigned short* slot_items;  // oa | ob << 8 (chunk-local observations); oa == ob: own term
    int* lcam_obs_begin;  // chunk cameras + 1: observations of each chunk camera
    unsigned char* lcam_obs;     // chunk-local observation indices
    // owner-gather schedule: per chunk and warp, the first entry of the warp's task rounds
    // (kAssembleWarps per chunk + 1); rounds of 32 task ids, kNoTask for an idle lane
    int* warp_task_begin;
    unsigned short* task_list;
    // reduce lists
    int* up_contrib_begin;  // nupper + 1
    int* up_contrib;        // partial pair slots
    int* up_csr;            // nupper: CSR position of the upper block
    int* up_csr_t;          // nupper: CSR position of the transposed block (-1 on the diagonal)
    int* cam_contrib_begin; // ncb + 1
    int* cam_contrib;       // partial cam slots
    // CSR pattern of pose blocks (both triangles)
    int* row_ptr;         // ncb + 1
    int* col_idx;         // nnzb
    int* diag_pos;        // ncb
    // raw observations (original order) for the strict RMS
    long long* raw_offsets;  // nt + 1
    int* raw_cam;
    double* raw_u;
    double* raw_v;
    double* raw_w;        // sanitized weight / scale^2 (0 for unusable)
    int* raw_bad;         // 1 when the observation makes the strict RMS infinite
};

// Host model built from the problem (gauge, active tracks, block numbering, groups, pattern).
struct HostGroup {
    double params[kP], prior[kP], invSigma[kP], lower[kP], upper[kP];
    bool enabled[kP];
    double focalRef, aspectRef;
};

struct ChunkSet {
    int max_obs = 0, max_cams = 0, max_pairs = 0, max_tracks = 0;
    std::vector<int> obs_begin, cam_begin, cams, pair_begin, pairs, pair_upper;
    std::vector<unsigned char> obs_lcam;
    std::vector<int> slot_item_begin, lcam_obs_begin;
    std::vector<unsigned short> slot_items;
    std::vector<unsigned char> lcam_obs;
    std::vector<int> up_contrib_begin, up_contrib, cam_contrib_begin, cam_contrib;
    // owner-gather schedule of phase D of the assembly (see schedule_owner_tasks in pb_host.cpp)
    std::vector<int> warp_task_begin;
    std::vector<unsigned short> task_list;
    size_t n_pair_partials() const { return pairs.size(); }
    size_t n_cam_partials() const { return cams.size(); }
    int n() const { return static_cast<int>(obs_begin.empty() ? 0 : obs_begin.size() - 1); }
};

// Rig topology of a problem and the map of the camera-block reduced system onto the rig's pose
// blocks.  Rig blocks: captures 0 .. ncapb - 1, then sensors ncapb .. nrb - 1.
struct RigModel {
    bool on = false;
    int ncap = 0, nsen = 0;
    std::vector<double> cap_in, sen_in;            // 12 per capture / sensor (input)
    std::vector<int> cap_info, sen_info;           // 2 per capture / sensor: rig id, fixed flag
    std::vector<int> cam_capture, cam_sensor;      // per camera
    std::vector<int> capture_block, sensor_block;  // per capture / sensor: rig block, or -1
    int ncapb = 0, nsenb = 0, nrb = 0;
    // per camera block (kernel numbering): its camera, rig blocks of its capture and sensor (-1)
    std::vector<int> cb_camera, cb_cap_block, cb_sen_block;
    // CSR of the rig pose blocks (both triangles, diagonal always present)
    std::vector<int> row_ptr, col_idx, diag_pos;
    // per upper rig block (row-major over the CSR, i <= j): its CSR position, the position of its
    // transpose (-1 on the diagonal), and its terms [term_begin[u], term_begin[u + 1]): camera
    // block CSR positions p of blocks (a, b) with the rig block's row in a's chain and its column
    // in b's, two ints each: p, then a << 2 | (row is a's sensor) << 1 | (column is b's sensor)
    std::vector<int> up_pos, up_tpos, term_begin, terms;
    // per rig block: the camera blocks chained to it, coded a << 1 | (the block is a's sensor)
    std::vector<int> blk_begin, blk_items;
    // the reference's numbering: primary blocks (rig blocks, groups, promoted points) and the
    // upper block pairs of prepareOffDiagonalTopology over them
    int P = 0;
    std::vector<std::pair<int, int>> pairs;
};

struct HostModel {
    int nc = 0, nt = 0;
    long long no = 0;
    std::vector<double> cams_in, cams_ref, points_in;
    std::vector<long long> offs;
    std::vector<int> obs_cam;
    std::vector<double> obs_u, obs_v, obs_weight, obs_scale;
    std::vector<int> fixed_cams, fixed_tracks, group_ids;
    // control points (valid constraints only): per original track, the whitened residual
    // sqrt(weight) W (X - P) as W (9, scaled) and P (3); ref_param == false when any exists
    // (the reference point parameterisation applies to image-only problems)
    std::vector<int> cp_track;
    std::vector<double> cp_rec;   // 12 per constraint
    std::vector<int> trk_cp_begin;  // processed tracks + 1
    std::vector<double> cp_proc;    // 12 per constraint of a processed track, processing order
    double cp_huber = 0.2;
    bool ref_param = true;
    // scale bars (Problem::scaleBarConstraints): two original track indices and (distance, sigma,
    // weight) per bar; the active, non-fixed tracks of the bars become primary point blocks,
    // promoted index k in track order (prepareActiveProblem, BundleAdjustPlaMatrixProblem.cpp:235-266)
    std::vector<int> bar_tracks;
    std::vector<double> bar_data;
    double bar_weight = 1.0, bar_huber = 0.2;
    std::vector<int> prom_track;  // promoted index -> original track
    std::vector<int> track_prom;  // original track -> promoted index, or -1
    int npr = 0;
    bool force_general = false;   // scale bars: the online path is not available
    // rig topology (Problem::rig).  The assembly runs on one 6-column pose block per camera with
    // a free capture or sensor (a "camera block" of the kernels, camera_block[c]); the reduced
    // system is then mapped to the pose blocks of the rig (captures, then sensors) by the
    // per-camera chain rule J_capture = J_camera Mc, J_sensor = J_camera Ms (pb_rig.cu).
    RigModel rig;
    int gauge_anchor = -1, gauge_scale = -1;
    double gauge_baseline = 0.0;
    int loss = 0;
    double loss_scale = 1.0;
    // active problem
    std::vector<signed char> active_track;
    std::vector<int> camera_block, intrinsic_block, calib_group, track_block;
    int P = 0, ncb = 0, ng = 0, ntb = 0, active_tracks = 0, obs_count = 0, rejected = 0;
    int ni = 0;
    int int_cols[kMaxNI] = {0};
    std::vector<HostGroup> groups;
    // reference topology (upper pairs over all primary blocks)
    std::vector<std::pair<int, int>> pairs;
    // processing order
    std::vector<int> trk_order;       // processing index -> original track
    std::vector<int> trk_obs_begin;   // processing obs ranges
    std::vector<int> p_obs_orig;      // processing obs -> original obs
    // pose CSR
    std::vector<int> row_ptr, col_idx, diag_pos, up_row, up_col, up_csr, up_csr_t;
    ChunkSet chunks[2];               // per precision
    bool chunks_ready[2] = {false, false};
    long long structure_hash = 0;
};

// Per-observation record stride of the assembly's shared-memory arrays: the field count rounded
// up to an odd number of words (bank-conflict-free strided access by the lanes of a warp).
#if defined(__CUDACC__)
#define PB_HOST_DEVICE __host__ __device__
#else
#define PB_HOST_DEVICE
#endif
inline PB_HOST_DEVICE int chunk_stride(int words) { return words | 1; }

// pb_host.cpp
int build_host_model(const pb_problem_desc* pr, const pb_solve_options* op, HostModel* m, std::string* err);
// validateControlPointConstraint + makeControlPointWhitening (control_point.cpp:91-220) of one
// 15-double control-point record; W receives the whitening matrix (row-major).
bool cp_valid(const double* data, double* W);
int build_chunks(HostModel* m, int precision, size_t smem_budget, std::string* err);
size_t chunk_smem_bytes(int precision, int max_obs, int max_tracks, int ni, int nb);
double finite_median(std::vector<double> v, double fallback);
// Largest number of threads the host planning of the calling thread may use (0: no cap).  The
// plan and every result are the same for any cap.
void set_host_thread_cap(int cap);
void camera_parameter_block(const double* cam, double* p);

}  // namespace pb
