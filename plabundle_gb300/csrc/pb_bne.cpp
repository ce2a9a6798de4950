// pb_bne.cpp -- host block normal equations of the general (non-online) path: the container that
// plabundle's general assembly fills and hands to the damped Schur solve.
//
// It restates plamatrix::internal::BlockNormalEquations<double>, which lives in the PlaMatrix
// library (absent from the reference tree), from its use sites:
//   construction (primaryBlocks, eliminatedBlocks, 13, 3) and clearValues
//     (src/internal/BundleAdjustPlaMatrixAssembly.cpp:852-863);
//   addResidualBlocks / addPrimaryResidualBlocks / addEliminatedResidualBlock /
//     addPrimaryResidualBlock (:356-438, AssemblySurvey.cpp:35-40, :80-84);
//   addPrimaryGradientBlock / addPrimaryHessianBlock / finalizePrimaryDiagonal
//     (BundleAdjustPlaMatrixReferenceSchur.cpp:911-930);
//   mergeFrom / mergeEliminatedShardFrom (BundleAdjustPlaMatrixAssembly.cpp:899-912).
// A residual block r (rows) with Jacobians J_b (rows x block size) and weight w adds
//   H_bc += w J_b^T J_c,   g_b += w J_b^T r
// for every pair of its blocks (primary-primary, primary-eliminated and eliminated-eliminated);
// g is the gradient of 1/2 sum w |r|^2 and the damped solve returns the step of (H + D) x = -g.
// Storage: dense primary diagonal blocks, a hash of the upper off-diagonal primary pairs, dense
// eliminated diagonal blocks and a hash of the primary-eliminated couplings.  A container is used
// by one thread at a time; per-thread shards are merged with pb_bne_merge_from /
// pb_bne_merge_eliminated_shard_from, as the reference's OpenMP assembly does.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "pb_internal.h"

struct pb_bne {
    int P = 0, E = 0, pb = 0, eb = 0;
    std::vector<double> diag;   // P * pb * pb
    std::vector<double> gp;     // P * pb
    std::vector<double> hee;    // E * eb * eb
    std::vector<double> ge;     // E * eb
    // upper primary pairs (row block < column block): key row * P + col
    std::unordered_map<long long, int> off_index;
    std::vector<int> off_row, off_col;
    std::vector<double> off;    // pb * pb per pair, row-major (rows of the row block)
    // couplings H_pe: key eliminated * P + primary
    std::unordered_map<long long, int> cpl_index;
    std::vector<int> cpl_elim, cpl_prim;
    std::vector<double> cpl;    // pb * eb per coupling, row-major (rows of the primary block)
};

namespace pb {

long long bne_structure_hash(const pb_bne* q) {
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](long long v) {
        h ^= static_cast<unsigned long long>(v);
        h *= 1099511628211ull;
    };
    mix(q->P);
    mix(q->E);
    mix(q->pb);
    mix(q->eb);
    // pair and coupling sets, independent of their insertion order
    std::vector<long long> keys;
    keys.reserve(q->off_row.size() + q->cpl_elim.size() + 1);
    for (size_t i = 0; i < q->off_row.size(); ++i) keys.push_back(static_cast<long long>(q->off_row[i]) * q->P + q->off_col[i]);
    keys.push_back(-1);
    for (size_t i = 0; i < q->cpl_elim.size(); ++i)
        keys.push_back((static_cast<long long>(q->cpl_elim[i]) * q->P + q->cpl_prim[i]) ^ (1ll << 62));
    std::sort(keys.begin(), keys.end());
    for (long long k : keys) mix(k);
    return static_cast<long long>(h);
}

// Read access for the device solve (pb_schur.cu).
const std::vector<double>& bne_diag(const pb_bne* q) { return q->diag; }
const std::vector<double>& bne_gp(const pb_bne* q) { return q->gp; }
const std::vector<double>& bne_hee(const pb_bne* q) { return q->hee; }
const std::vector<double>& bne_ge(const pb_bne* q) { return q->ge; }
void bne_dims(const pb_bne* q, int* P, int* E, int* pbs, int* ebs) {
    *P = q->P;
    *E = q->E;
    *pbs = q->pb;
    *ebs = q->eb;
}
void bne_pairs(const pb_bne* q, const std::vector<int>** row, const std::vector<int>** col, const std::vector<double>** vals) {
    *row = &q->off_row;
    *col = &q->off_col;
    *vals = &q->off;
}
void bne_couplings(const pb_bne* q, const std::vector<int>** elim, const std::vector<int>** prim,
                   const std::vector<double>** vals) {
    *elim = &q->cpl_elim;
    *prim = &q->cpl_prim;
    *vals = &q->cpl;
}

}  // namespace pb

namespace {

double* off_block(pb_bne* q, int r, int c) {
    const long long key = static_cast<long long>(r) * q->P + c;
    auto it = q->off_index.find(key);
    int idx;
    if (it == q->off_index.end()) {
        idx = static_cast<int>(q->off_row.size());
        q->off_index.emplace(key, idx);
        q->off_row.push_back(r);
        q->off_col.push_back(c);
        q->off.resize(q->off.size() + static_cast<size_t>(q->pb) * q->pb, 0.0);
    } else {
        idx = it->second;
    }
    return q->off.data() + static_cast<size_t>(idx) * q->pb * q->pb;
}

double* coupling(pb_bne* q, int e, int p) {
    const long long key = static_cast<long long>(e) * q->P + p;
    auto it = q->cpl_index.find(key);
    int idx;
    if (it == q->cpl_index.end()) {
        idx = static_cast<int>(q->cpl_elim.size());
        q->cpl_index.emplace(key, idx);
        q->cpl_elim.push_back(e);
        q->cpl_prim.push_back(p);
        q->cpl.resize(q->cpl.size() + static_cast<size_t>(q->pb) * q->eb, 0.0);
    } else {
        idx = it->second;
    }
    return q->cpl.data() + static_cast<size_t>(idx) * q->pb * q->eb;
}

// H_(a,b) += w J_a^T J_b for primary blocks a, b (any order; stored in the upper block).
void add_primary_pair(pb_bne* q, int a, const double* Ja, int b, const double* Jb, int rows, double w) {
    const int n = q->pb;
    if (a == b) {
        double* D = q->diag.data() + static_cast<size_t>(a) * n * n;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double s = 0.0;
                for (int r = 0; r < rows; ++r) s += Ja[r * n + i] * Jb[r * n + j];
                D[i * n + j] += w * s;
            }
        return;
    }
    const bool ordered = a < b;
    const int lo = ordered ? a : b, hi = ordered ? b : a;
    const double* Jl = ordered ? Ja : Jb;
    const double* Jh = ordered ? Jb : Ja;
    double* O = off_block(q, lo, hi);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int r = 0; r < rows; ++r) s += Jl[r * n + i] * Jh[r * n + j];
            O[i * n + j] += w * s;
        }
}

void add_primary_gradient(pb_bne* q, int a, const double* Ja, const double* r, int rows, double w) {
    const int n = q->pb;
    double* g = q->gp.data() + static_cast<size_t>(a) * n;
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < rows; ++k) s += Ja[k * n + i] * r[k];
        g[i] += w * s;
    }
}

void add_eliminated(pb_bne* q, int e, const double* Je, const double* r, int rows, double w) {
    const int m = q->eb;
    double* H = q->hee.data() + static_cast<size_t>(e) * m * m;
    double* g = q->ge.data() + static_cast<size_t>(e) * m;
    for (int i = 0; i < m; ++i) {
        double sg = 0.0;
        for (int k = 0; k < rows; ++k) sg += Je[k * m + i] * r[k];
        g[i] += w * sg;
        for (int j = 0; j < m; ++j) {
            double s = 0.0;
            for (int k = 0; k < rows; ++k) s += Je[k * m + i] * Je[k * m + j];
            H[i * m + j] += w * s;
        }
    }
}

void add_coupling(pb_bne* q, int a, const double* Ja, int e, const double* Je, int rows, double w) {
    const int n = q->pb, m = q->eb;
    double* W = coupling(q, e, a);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
            double s = 0.0;
            for (int k = 0; k < rows; ++k) s += Ja[k * n + i] * Je[k * m + j];
            W[i * m + j] += w * s;
        }
}

bool finite_weight(double w) { return std::isfinite(w); }

}  // namespace

extern "C" {

pb_status pb_bne_create(int32_t primary_blocks, int32_t eliminated_blocks, int32_t primary_block_size,
                        int32_t eliminated_block_size, pb_bne** out) {
    if (!out || primary_blocks < 0 || eliminated_blocks < 0 || primary_block_size < 1 ||
        primary_block_size > PB_BNE_MAX_PRIMARY_BLOCK_SIZE || eliminated_block_size != 3)
        return PB_ERR_INVALID_ARGUMENT;
    try {
        auto* q = new pb_bne;
        q->P = primary_blocks;
        q->E = eliminated_blocks;
        q->pb = primary_block_size;
        q->eb = eliminated_block_size;
        q->diag.assign(static_cast<size_t>(q->P) * q->pb * q->pb, 0.0);
        q->gp.assign(static_cast<size_t>(q->P) * q->pb, 0.0);
        q->hee.assign(static_cast<size_t>(q->E) * q->eb * q->eb, 0.0);
        q->ge.assign(static_cast<size_t>(q->E) * q->eb, 0.0);
        *out = q;
        return PB_OK;
    } catch (const std::bad_alloc&) {
        return PB_ERR_INVALID_ARGUMENT;
    }
}

pb_status pb_bne_destroy(pb_bne* eq) {
    delete eq;
    return PB_OK;
}

pb_status pb_bne_clear_values(pb_bne* eq) {
    if (!eq) return PB_ERR_INVALID_ARGUMENT;
    std::fill(eq->diag.begin(), eq->diag.end(), 0.0);
    std::fill(eq->gp.begin(), eq->gp.end(), 0.0);
    std::fill(eq->hee.begin(), eq->hee.end(), 0.0);
    std::fill(eq->ge.begin(), eq->ge.end(), 0.0);
    std::fill(eq->off.begin(), eq->off.end(), 0.0);
    std::fill(eq->cpl.begin(), eq->cpl.end(), 0.0);
    return PB_OK;
}

pb_status pb_bne_sizes(const pb_bne* eq, int32_t* sizes) {
    if (!eq || !sizes) return PB_ERR_INVALID_ARGUMENT;
    sizes[0] = eq->P;
    sizes[1] = eq->E;
    sizes[2] = eq->pb;
    sizes[3] = eq->eb;
    sizes[4] = static_cast<int32_t>(eq->off_row.size());
    sizes[5] = static_cast<int32_t>(eq->cpl_elim.size());
    return PB_OK;
}

pb_status pb_bne_add_residual_blocks(pb_bne* eq, const int32_t* primary, const double* const* primary_jacobians,
                                     int32_t n_primary, int32_t eliminated, const double* eliminated_jacobian,
                                     const double* residual, int32_t rows, double weight) {
    if (!eq || rows < 1 || n_primary < 0 || !residual || !finite_weight(weight)) return PB_ERR_INVALID_ARGUMENT;
    if (n_primary > 0 && (!primary || !primary_jacobians)) return PB_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < n_primary; ++k)
        if (primary[k] < 0 || primary[k] >= eq->P || !primary_jacobians[k]) return PB_ERR_BOUNDS;
    if (eliminated >= 0 && (eliminated >= eq->E || !eliminated_jacobian)) return PB_ERR_BOUNDS;
    for (int a = 0; a < n_primary; ++a) {
        add_primary_gradient(eq, primary[a], primary_jacobians[a], residual, rows, weight);
        for (int b = a; b < n_primary; ++b) {
            if (b == a) {
                add_primary_pair(eq, primary[a], primary_jacobians[a], primary[a], primary_jacobians[a], rows, weight);
            } else if (primary[a] == primary[b]) {
                // two terms on one block: both cross products land on its diagonal block
                add_primary_pair(eq, primary[a], primary_jacobians[a], primary[b], primary_jacobians[b], rows, weight);
                add_primary_pair(eq, primary[b], primary_jacobians[b], primary[a], primary_jacobians[a], rows, weight);
            } else {
                add_primary_pair(eq, primary[a], primary_jacobians[a], primary[b], primary_jacobians[b], rows, weight);
            }
        }
        if (eliminated >= 0) add_coupling(eq, primary[a], primary_jacobians[a], eliminated, eliminated_jacobian, rows, weight);
    }
    if (eliminated >= 0) add_eliminated(eq, eliminated, eliminated_jacobian, residual, rows, weight);
    return PB_OK;
}

pb_status pb_bne_add_primary_residual_blocks(pb_bne* eq, const int32_t* primary, const double* const* primary_jacobians,
                                             int32_t n_primary, const double* residual, int32_t rows, double weight) {
    return pb_bne_add_residual_blocks(eq, primary, primary_jacobians, n_primary, -1, nullptr, residual, rows, weight);
}

pb_status pb_bne_add_primary_residual_block(pb_bne* eq, int32_t block, const double* jacobian, const double* residual,
                                            int32_t rows, double weight) {
    const double* j[1] = {jacobian};
    return pb_bne_add_residual_blocks(eq, &block, j, 1, -1, nullptr, residual, rows, weight);
}

pb_status pb_bne_add_eliminated_residual_block(pb_bne* eq, int32_t block, const double* jacobian, const double* residual,
                                               int32_t rows, double weight) {
    if (block < 0) return PB_ERR_BOUNDS;
    return pb_bne_add_residual_blocks(eq, nullptr, nullptr, 0, block, jacobian, residual, rows, weight);
}

pb_status pb_bne_add_residual_block(pb_bne* eq, int32_t primary, const double* primary_jacobian, int32_t eliminated,
                                    const double* eliminated_jacobian, const double* residual, int32_t rows,
                                    double weight) {
    const double* j[1] = {primary_jacobian};
    return pb_bne_add_residual_blocks(eq, &primary, j, 1, eliminated, eliminated_jacobian, residual, rows, weight);
}

pb_status pb_bne_add_primary_gradient_block(pb_bne* eq, int32_t block, const double* gradient) {
    if (!eq || !gradient) return PB_ERR_INVALID_ARGUMENT;
    if (block < 0 || block >= eq->P) return PB_ERR_BOUNDS;
    double* g = eq->gp.data() + static_cast<size_t>(block) * eq->pb;
    for (int i = 0; i < eq->pb; ++i) g[i] += gradient[i];
    return PB_OK;
}

pb_status pb_bne_add_primary_hessian_block(pb_bne* eq, int32_t row_block, int32_t col_block, const double* block) {
    if (!eq || !block) return PB_ERR_INVALID_ARGUMENT;
    if (row_block < 0 || row_block >= eq->P || col_block < 0 || col_block >= eq->P) return PB_ERR_BOUNDS;
    const int n = eq->pb;
    if (row_block == col_block) {
        double* D = eq->diag.data() + static_cast<size_t>(row_block) * n * n;
        for (int i = 0; i < n * n; ++i) D[i] += block[i];
    } else if (row_block < col_block) {
        double* O = off_block(eq, row_block, col_block);
        for (int i = 0; i < n * n; ++i) O[i] += block[i];
    } else {
        // the lower block (row > col) is the transpose of the stored upper one
        double* O = off_block(eq, col_block, row_block);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) O[j * n + i] += block[i * n + j];
    }
    return PB_OK;
}

pb_status pb_bne_finalize_primary_diagonal(pb_bne* eq, double scale, double add) {
    if (!eq || !std::isfinite(scale) || !std::isfinite(add)) return PB_ERR_INVALID_ARGUMENT;
    const int n = eq->pb;
    for (int b = 0; b < eq->P; ++b)
        for (int i = 0; i < n; ++i) {
            double& d = eq->diag[static_cast<size_t>(b) * n * n + i * n + i];
            d = d != 0.0 ? d * scale : add;
        }
    return PB_OK;
}

pb_status pb_bne_merge_eliminated_shard_from(pb_bne* eq, const pb_bne* shard, int32_t eliminated_offset) {
    if (!eq || !shard || eq->P != shard->P || eq->pb != shard->pb || eq->eb != shard->eb) return PB_ERR_INVALID_ARGUMENT;
    if (eliminated_offset < 0 || eliminated_offset + shard->E > eq->E) return PB_ERR_BOUNDS;
    for (size_t i = 0; i < eq->diag.size(); ++i) eq->diag[i] += shard->diag[i];
    for (size_t i = 0; i < eq->gp.size(); ++i) eq->gp[i] += shard->gp[i];
    const int m = eq->eb;
    for (size_t i = 0; i < shard->hee.size(); ++i) eq->hee[static_cast<size_t>(eliminated_offset) * m * m + i] += shard->hee[i];
    for (size_t i = 0; i < shard->ge.size(); ++i) eq->ge[static_cast<size_t>(eliminated_offset) * m + i] += shard->ge[i];
    const int n = eq->pb;
    for (size_t k = 0; k < shard->off_row.size(); ++k) {
        double* O = off_block(eq, shard->off_row[k], shard->off_col[k]);
        const double* S = shard->off.data() + k * n * n;
        for (int i = 0; i < n * n; ++i) O[i] += S[i];
    }
    for (size_t k = 0; k < shard->cpl_elim.size(); ++k) {
        double* W = coupling(eq, eliminated_offset + shard->cpl_elim[k], shard->cpl_prim[k]);
        const double* S = shard->cpl.data() + k * n * m;
        for (int i = 0; i < n * m; ++i) W[i] += S[i];
    }
    return PB_OK;
}

pb_status pb_bne_merge_from(pb_bne* eq, const pb_bne* other) {
    if (!eq || !other || eq->E != other->E) return PB_ERR_INVALID_ARGUMENT;
    return pb_bne_merge_eliminated_shard_from(eq, other, 0);
}

pb_status pb_bne_export(const pb_bne* eq, double* primary_matrix, double* primary_gradient, double* eliminated_blocks,
                        double* eliminated_gradient, int32_t* coupling_index, double* couplings) {
    if (!eq) return PB_ERR_INVALID_ARGUMENT;
    const int n = eq->pb, m = eq->eb;
    const size_t N = static_cast<size_t>(eq->P) * n;
    if (primary_matrix) {
        std::fill(primary_matrix, primary_matrix + N * N, 0.0);
        for (int b = 0; b < eq->P; ++b)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    primary_matrix[(static_cast<size_t>(b) * n + i) * N + static_cast<size_t>(b) * n + j] =
                        eq->diag[static_cast<size_t>(b) * n * n + i * n + j];
        for (size_t k = 0; k < eq->off_row.size(); ++k) {
            const size_t r0 = static_cast<size_t>(eq->off_row[k]) * n, c0 = static_cast<size_t>(eq->off_col[k]) * n;
            const double* O = eq->off.data() + k * n * n;
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    primary_matrix[(r0 + i) * N + c0 + j] = O[i * n + j];
                    primary_matrix[(c0 + j) * N + r0 + i] = O[i * n + j];
                }
        }
    }
    if (primary_gradient) std::copy(eq->gp.begin(), eq->gp.end(), primary_gradient);
    if (eliminated_blocks) std::copy(eq->hee.begin(), eq->hee.end(), eliminated_blocks);
    if (eliminated_gradient) std::copy(eq->ge.begin(), eq->ge.end(), eliminated_gradient);
    for (size_t k = 0; k < eq->cpl_elim.size(); ++k) {
        if (coupling_index) {
            coupling_index[2 * k] = eq->cpl_elim[k];
            coupling_index[2 * k + 1] = eq->cpl_prim[k];
        }
        if (couplings) std::copy(eq->cpl.begin() + k * n * m, eq->cpl.begin() + (k + 1) * n * m, couplings + k * n * m);
    }
    return PB_OK;
}

}  // extern "C"
