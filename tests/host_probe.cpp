// host_probe.cpp -- test-only probe of the host-side planning code (pb_host.cpp) without a GPU.
//
// Builds the host model and the assembly chunks of a problem and checks every invariant the
// assembly kernel relies on, by re-deriving each list independently by brute force:
//   - chunks partition the processing-order observations into whole tracks, at most max_obs each;
//   - every observation's chunk camera maps back to its camera (or 255 without a pose block);
//   - every pair slot holds exactly the items of its camera pair: one own term (o, o) per
//     observation on the diagonal slot, one coupling per pair of observations of an eliminated
//     track (lower chunk camera first; both orientations when the two share a camera);
//   - every chunk camera lists exactly its observations, in order;
//   - every chunk pair is reduced into the upper pose block of its two cameras, exactly once;
//   - the owner-gather schedule holds every task of a chunk exactly once, in rounds of 32.
// Returns 0 when all hold, else a nonzero code with a message.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../plabundle_gb300/csrc/pb_internal.h"

namespace {
std::string g_msg;
int fail(const std::string& m) {
    g_msg = m;
    return 1;
}
}  // namespace

extern "C" const char* probe_message() { return g_msg.c_str(); }

// stats: [chunks, max_obs, slots, items, camera entries, processed obs, smem bytes]
extern "C" int probe_chunks(const pb_problem_desc* pr, const pb_solve_options* op, int precision, size_t smem_budget,
                            long long* stats) {
    using namespace pb;
    HostModel m;
    std::string err;
    int rc = build_host_model(pr, op, &m, &err);
    if (rc) return fail("build_host_model: " + err);
    rc = build_chunks(&m, precision, smem_budget, &err);
    if (rc) return fail("build_chunks: " + err);
    const ChunkSet& cs = m.chunks[precision];
    const int nch = cs.n();
    const int nobs = static_cast<int>(m.p_obs_orig.size());
    if (cs.obs_begin.front() != 0 || cs.obs_begin.back() != nobs) return fail("chunks do not cover the observations");
    if (static_cast<int>(cs.slot_item_begin.size()) != static_cast<int>(cs.pairs.size()) + 1)
        return fail("slot_item_begin size");
    if (static_cast<int>(cs.lcam_obs_begin.size()) != static_cast<int>(cs.cams.size()) + 1)
        return fail("lcam_obs_begin size");
    // track of every processing observation
    std::vector<int> trk_of(nobs, -1);
    for (size_t p = 0; p + 1 < m.trk_obs_begin.size(); ++p)
        for (int o = m.trk_obs_begin[p]; o < m.trk_obs_begin[p + 1]; ++o) trk_of[o] = static_cast<int>(p);
    long long items_total = 0;
    std::vector<int> slot_seen(cs.pairs.size(), 0);
    for (int c = 0; c < nch; ++c) {
        const int o0 = cs.obs_begin[c], o1 = cs.obs_begin[c + 1];
        if (o1 - o0 > cs.max_obs || o1 < o0) return fail("chunk larger than max_obs");
        {
            int tracks = 0;
            for (int o = o0; o < o1; ++o) tracks += m.trk_obs_begin[trk_of[o]] == o;
            if (tracks > cs.max_tracks || cs.max_tracks > 255) return fail("chunk holds more than max_tracks tracks");
        }
        if (o1 > o0 && (m.trk_obs_begin[trk_of[o0]] != o0 || (o1 < nobs && m.trk_obs_begin[trk_of[o1]] != o1)))
            return fail("chunk splits a track");
        const int c0 = cs.cam_begin[c], ncl = cs.cam_begin[c + 1] - c0;
        if (ncl > 254) return fail("too many chunk cameras");
        for (int l = 1; l < ncl; ++l)
            if (m.camera_block[cs.cams[c0 + l - 1]] >= m.camera_block[cs.cams[c0 + l]])
                return fail("chunk cameras not ordered by pose block");
        for (int o = o0; o < o1; ++o) {
            const int cam = m.obs_cam[m.p_obs_orig[o]];
            const int l = cs.obs_lcam[o];
            if (m.camera_block[cam] < 0) {
                if (l != 255) return fail("observation without pose block has a chunk camera");
            } else if (l >= ncl || cs.cams[c0 + l] != cam) {
                return fail("observation chunk camera mismatch");
            }
        }
        // expected items per (a, b) chunk-camera pair, by brute force
        std::vector<std::vector<unsigned short>> expect(static_cast<size_t>(ncl) * ncl);
        for (int o = o0; o < o1; ++o) {
            const int la = cs.obs_lcam[o];
            if (la == 255) continue;
            const int i = o - o0;
            expect[static_cast<size_t>(la) * ncl + la].push_back(static_cast<unsigned short>(i | (i << 8)));
            const int p = trk_of[o];
            if (m.track_block[m.trk_order[p]] < 0) continue;
            for (int o2 = m.trk_obs_begin[p]; o2 < m.trk_obs_begin[p + 1]; ++o2) {
                if (o2 == o) continue;
                const int lb = cs.obs_lcam[o2];
                if (lb == 255) continue;
                const int j = o2 - o0;
                // item (i, j) with i on the lower camera; same camera: both orientations
                if (la < lb || (la == lb))
                    expect[static_cast<size_t>(std::min(la, lb)) * ncl + std::max(la, lb)].push_back(
                        static_cast<unsigned short>(i | (j << 8)));
            }
        }
        std::vector<char> pair_used(static_cast<size_t>(ncl) * ncl, 0);
        for (int s = cs.pair_begin[c]; s < cs.pair_begin[c + 1]; ++s) {
            const int a = cs.pairs[s] & 0xFFFF, b = cs.pairs[s] >> 16;
            if (a > b || b >= ncl) return fail("pair slot out of order / range");
            if (pair_used[static_cast<size_t>(a) * ncl + b]) return fail("duplicate pair slot");
            pair_used[static_cast<size_t>(a) * ncl + b] = 1;
            std::vector<unsigned short> got(cs.slot_items.begin() + cs.slot_item_begin[s],
                                            cs.slot_items.begin() + cs.slot_item_begin[s + 1]);
            std::vector<unsigned short> want = expect[static_cast<size_t>(a) * ncl + b];
            for (unsigned short it : got)
                if ((it & 0xFF) >= o1 - o0 || (it >> 8) >= o1 - o0) return fail("item index outside the chunk");
            items_total += static_cast<long long>(got.size());
            std::sort(got.begin(), got.end());
            std::sort(want.begin(), want.end());
            if (got != want) {
                char buf[160];
                std::snprintf(buf, sizeof buf, "slot items differ: chunk %d slot %d (%d,%d): got %zu want %zu", c, s, a, b,
                              got.size(), want.size());
                return fail(buf);
            }
            // reduce mapping: this slot feeds the upper block of its two pose blocks, once
            const int u = cs.pair_upper[s];
            const int bi = m.camera_block[cs.cams[c0 + a]], bj = m.camera_block[cs.cams[c0 + b]];
            if (u < 0 || m.up_row[u] != bi || m.up_col[u] != bj) return fail("pair slot mapped to the wrong block");
            int hits = 0;
            for (int k = cs.up_contrib_begin[u]; k < cs.up_contrib_begin[u + 1]; ++k) hits += cs.up_contrib[k] == s;
            if (hits != 1) return fail("pair slot not reduced exactly once");
            slot_seen[s] = 1;
        }
        for (size_t q = 0; q < expect.size(); ++q)
            if (!expect[q].empty() && !pair_used[q]) return fail("a camera pair with items has no slot");
        for (int l = 0; l < ncl; ++l) {
            std::vector<int> want;
            for (int o = o0; o < o1; ++o)
                if (cs.obs_lcam[o] == l) want.push_back(o - o0);
            std::vector<int> got;
            for (int k = cs.lcam_obs_begin[c0 + l]; k < cs.lcam_obs_begin[c0 + l + 1]; ++k) got.push_back(cs.lcam_obs[k]);
            if (got != want) return fail("chunk camera observation list differs");
            int hits = 0;
            const int blk = m.camera_block[cs.cams[c0 + l]];
            for (int k = cs.cam_contrib_begin[blk]; k < cs.cam_contrib_begin[blk + 1]; ++k) hits += cs.cam_contrib[k] == c0 + l;
            if (hits != 1) return fail("chunk camera not reduced exactly once");
        }
        // owner-gather schedule: every task of the chunk exactly once, rounds of 32 per warp
        {
            const int ntask = 6 * (cs.pair_begin[c + 1] - cs.pair_begin[c]) + (2 + m.ng * m.ni) * ncl;
            std::vector<int> seen(static_cast<size_t>(ntask), 0);
            for (int w = 0; w < kAssembleWarps; ++w) {
                const int b = cs.warp_task_begin[c * kAssembleWarps + w], e = cs.warp_task_begin[c * kAssembleWarps + w + 1];
                if (e < b || (e - b) % 32 != 0) return fail("warp task range not made of rounds of 32");
                for (int k = b; k < e; ++k) {
                    const int id = cs.task_list[k];
                    if (id == kNoTask) continue;
                    if (id >= ntask) return fail("task id outside the chunk");
                    ++seen[id];
                }
            }
            for (int v : seen)
                if (v != 1) return fail("owner-gather task not scheduled exactly once");
        }
    }
    if (static_cast<int>(cs.warp_task_begin.size()) != nch * kAssembleWarps + 1 ||
        cs.warp_task_begin.back() != static_cast<int>(cs.task_list.size()))
        return fail("warp task table size");
    for (int v : slot_seen)
        if (!v) return fail("pair slot outside every chunk");
    if (stats) {
        stats[0] = nch;
        stats[1] = cs.max_obs;
        stats[2] = static_cast<long long>(cs.pairs.size());
        stats[3] = items_total;
        stats[4] = static_cast<long long>(cs.cams.size());
        stats[5] = nobs;
        stats[6] = static_cast<long long>(chunk_smem_bytes(precision, cs.max_obs, cs.max_tracks, m.ni, m.ng * m.ni));
    }
    return 0;
}

// Host model of a problem: status, message, and the gauge the host settled on.
// out_i (11 ints): [status, ref_param, n_fixed_cams, gauge_anchor, gauge_scale, n_control_points
//         kept, camera_blocks, active_tracks, observations, rejected tracks, track_blocks];
// fixed: the fixed cameras (n_cameras capacity); out_d: [gauge_baseline]
extern "C" int probe_model(const pb_problem_desc* pr, const pb_solve_options* op, int* out_i, int* fixed,
                           double* out_d) {
    using namespace pb;
    HostModel m;
    std::string err;
    const int rc = build_host_model(pr, op, &m, &err);
    g_msg = err;
    out_i[0] = rc;
    if (rc) return rc;
    out_i[1] = m.ref_param ? 1 : 0;
    out_i[2] = static_cast<int>(m.fixed_cams.size());
    out_i[3] = m.gauge_anchor;
    out_i[4] = m.gauge_scale;
    out_i[5] = static_cast<int>(m.cp_track.size());
    out_i[6] = m.ncb;
    out_i[7] = m.active_tracks;
    out_i[8] = m.obs_count;
    out_i[9] = m.rejected;
    out_i[10] = m.ntb;
    for (size_t i = 0; i < m.fixed_cams.size(); ++i) fixed[i] = m.fixed_cams[i];
    out_d[0] = m.gauge_baseline;
    return 0;
}

// The host's control-point validation and whitening of one record.
extern "C" int probe_cp_whitening(const double* rec, double* W) { return pb::cp_valid(rec, W) ? 1 : 0; }

// Rig model of a problem as the host built it (the reference's numbering).
// out_i (8 ints): [status, rig capture blocks, rig sensor blocks, primary blocks (rig numbering),
//                  rig pairs, camera blocks of the kernels, n fixed cameras, ref_param];
// capture_block (captures), sensor_block (sensors), pairs (2 per pair; capacity max_pairs),
// cameras (n_cameras * 32: the composed input cameras), fixed (n_cameras capacity),
// groups (n_cameras: calibration group of each camera, -1 without refined intrinsics).
extern "C" int probe_rig(const pb_problem_desc* pr, const pb_solve_options* op, int* out_i, int* capture_block,
                         int* sensor_block, int* pairs, int max_pairs, double* cameras, int* fixed, int* groups) {
    using namespace pb;
    HostModel m;
    std::string err;
    const int rc = build_host_model(pr, op, &m, &err);
    g_msg = err;
    out_i[0] = rc;
    if (rc) return rc;
    const RigModel& R = m.rig;
    out_i[1] = R.ncapb;
    out_i[2] = R.nsenb;
    out_i[3] = R.P;
    out_i[4] = static_cast<int>(R.pairs.size());
    out_i[5] = m.ncb;
    out_i[6] = static_cast<int>(m.fixed_cams.size());
    out_i[7] = m.ref_param ? 1 : 0;
    for (int k = 0; k < R.ncap; ++k) capture_block[k] = R.capture_block.empty() ? -1 : R.capture_block[k];
    for (int s = 0; s < R.nsen; ++s) sensor_block[s] = R.sensor_block.empty() ? -1 : R.sensor_block[s];
    for (int i = 0; i < static_cast<int>(R.pairs.size()) && i < max_pairs; ++i) {
        pairs[2 * i] = R.pairs[i].first;
        pairs[2 * i + 1] = R.pairs[i].second;
    }
    std::copy(m.cams_in.begin(), m.cams_in.end(), cameras);
    for (size_t i = 0; i < m.fixed_cams.size(); ++i) fixed[i] = m.fixed_cams[i];
    for (int c = 0; c < m.nc; ++c) groups[c] = m.ng > 0 ? m.calib_group[c] : -1;
    return 0;
}

// The rig term lists checked by brute force: every rig block pair (I, J) of the CSR gets exactly the
// camera-block CSR entries (a, b) with I chained to a and J chained to b, and every rig block the
// camera blocks chained to it.  Returns 0 when they agree, else the first failing rig block + 1.
extern "C" int probe_rig_terms(const pb_problem_desc* pr, const pb_solve_options* op) {
    using namespace pb;
    HostModel m;
    std::string err;
    if (build_host_model(pr, op, &m, &err)) {
        g_msg = err;
        return -1;
    }
    const RigModel& R = m.rig;
    const int nrb = R.nrb;
    std::vector<std::vector<std::pair<int, int>>> want(R.up_pos.size());
    auto up_index = [&](int I, int J) {
        for (size_t u = 0; u < R.up_pos.size(); ++u) {
            const int p = R.up_pos[u];
            int row = 0;
            while (R.row_ptr[row + 1] <= p) ++row;
            if (row == I && R.col_idx[p] == J) return static_cast<int>(u);
        }
        return -1;
    };
    for (int a = 0; a < m.ncb; ++a)
        for (int p = m.row_ptr[a]; p < m.row_ptr[a + 1]; ++p) {
            const int b = m.col_idx[p];
            const int ra[2] = {R.cb_cap_block[a], R.cb_sen_block[a]}, rb[2] = {R.cb_cap_block[b], R.cb_sen_block[b]};
            for (int x = 0; x < 2; ++x)
                for (int y = 0; y < 2; ++y) {
                    if (ra[x] < 0 || rb[y] < 0 || ra[x] > rb[y]) continue;
                    const int u = up_index(ra[x], rb[y]);
                    if (u < 0) return 1 + ra[x];
                    want[u].emplace_back(p, a << 2 | x << 1 | y);
                }
        }
    for (size_t u = 0; u < want.size(); ++u) {
        const int n = R.term_begin[u + 1] - R.term_begin[u];
        if (n != static_cast<int>(want[u].size())) return 1 + static_cast<int>(u);
        for (int t = 0; t < n; ++t) {
            const int q = R.term_begin[u] + t;
            if (R.terms[2 * q] != want[u][t].first || R.terms[2 * q + 1] != want[u][t].second)
                return 1 + static_cast<int>(u);
        }
    }
    for (int I = 0; I < nrb; ++I) {
        std::vector<int> items;
        for (int a = 0; a < m.ncb; ++a) {
            if (R.cb_cap_block[a] == I) items.push_back(a << 1);
            if (R.cb_sen_block[a] == I) items.push_back(a << 1 | 1);
        }
        const std::vector<int> got(R.blk_items.begin() + R.blk_begin[I], R.blk_items.begin() + R.blk_begin[I + 1]);
        if (got != items) return 1 + I;
    }
    return 0;
}
